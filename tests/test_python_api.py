"""pp.neighbors plumbing against a fake core, as the reference tests its
Python layer (tests/test_python_api.py:38-119, :438-473): the uns entry, k
forwarding, use_rep="X", the missing representation, and the CSR layout."""

from __future__ import annotations

import numpy as np
import pytest
import scipy.sparse as sp

from mrustsc_gb300 import pp
from mrustsc_gb300.anndata_lite import AnnData

N_OBS, N_VARS = 7, 5


class FakeCore:
    def __init__(self):
        self.calls = []

    def args_of(self, name):
        return next(args for n, args, _ in self.calls if n == name)

    def knn(self, embedding, k, device, **kw):
        self.calls.append(("knn", (embedding, k, device), kw))
        n = embedding.shape[0]
        idx = np.array([[(i + j + 1) % n for j in range(k)] for i in range(n)], np.uint32)
        return idx, np.ones((n, k), np.float32)

    def connectivities(self, indices, distances):
        self.calls.append(("connectivities", (indices, distances), {}))
        n = indices.shape[0]
        return np.arange(n + 1, dtype=np.uint32), (np.arange(n, dtype=np.uint32) + 1) % n, \
            np.ones(n, np.float32), n


@pytest.fixture
def core(monkeypatch):
    fake = FakeCore()
    import mrustsc_gb300._shared as shared
    monkeypatch.setattr(shared, "_extension", lambda: fake)
    monkeypatch.setattr(pp, "_extension", lambda: fake)
    return fake


def _adata():
    rng = np.random.default_rng(0)
    return AnnData(rng.normal(size=(N_OBS, N_VARS)).astype(np.float32),
                   obsm={"X_pca": rng.normal(size=(N_OBS, 3)).astype(np.float32)})


def test_neighbors_writes_both_graphs_and_the_uns_entry(core):
    adata = _adata()
    assert pp.neighbors(adata) is None
    for key in ("distances", "connectivities"):
        assert sp.issparse(adata.obsp[key]) and adata.obsp[key].shape == (N_OBS, N_OBS)
    assert adata.uns["neighbors"]["params"] == {"n_neighbors": 15, "method": "umap", "use_rep": "X_pca"}
    assert adata.uns["neighbors"]["distances_key"] == "distances"
    assert adata.uns["neighbors"]["connectivities_key"] == "connectivities"


def test_k_forwarding_and_distances_layout(core):
    adata = _adata()
    pp.neighbors(adata, n_neighbors=4, device="cpu")
    embedding, k, device = core.args_of("knn")
    assert embedding.shape == (N_OBS, 3) and embedding.dtype == np.float32
    assert (k, device) == (3, "cpu")
    assert core.args_of("connectivities")[0].shape == (N_OBS, 3)
    d = adata.obsp["distances"]
    assert d.indptr.tolist() == list(range(0, N_OBS * 3 + 1, 3))
    # nearest-first order kept, stored zeros kept
    idx, _ = core.knn(adata.obsm["X_pca"], 3, "cpu")
    np.testing.assert_array_equal(d.indices.reshape(N_OBS, 3), idx)


def test_use_rep_x(core):
    pp.neighbors(_adata(), use_rep="X", n_neighbors=3)
    assert core.args_of("knn")[0].shape == (N_OBS, N_VARS)


def test_missing_representation_raises(core):
    adata = AnnData(np.zeros((N_OBS, 2), np.float32))
    with pytest.raises(KeyError, match="X_pca"):
        pp.neighbors(adata)


def test_n_neighbors_below_two_raises(core):
    with pytest.raises(ValueError):
        pp.neighbors(_adata(), n_neighbors=1)


def test_metric_is_forwarded_and_recorded(core):
    adata = _adata()
    pp.neighbors(adata, n_neighbors=3, metric="cosine")
    assert core.calls[0][2]["metric"] == "cosine"
    assert adata.uns["neighbors"]["params"]["metric"] == "cosine"
    with pytest.raises(ValueError):
        pp.neighbors(adata, metric="manhattan")


class RecordingBackend(FakeCore):
    """Stands in for this backend in the routing tests (no GPU needed)."""

    def gpu_available(self):
        return True


@pytest.mark.parametrize("device", ["auto", "gpu", "cuda", "metal"])
def test_core_routes_non_cpu_knn_to_this_backend(device):
    from mrustsc_gb300.core import Core

    real, ours = FakeCore(), RecordingBackend()
    core = Core(real, device_setting=lambda: "auto", backend=ours)
    x = np.zeros((6, 3), np.float32)
    core.knn(x, 2, device)
    core.connectivities(np.zeros((6, 2), np.uint32), np.ones((6, 2), np.float32))
    assert [c[0] for c in ours.calls] == ["knn", "connectivities"] and real.calls == []
    assert ours.args_of("knn")[2] == device


def test_core_routes_cpu_to_the_reference_module():
    from mrustsc_gb300.core import Core

    real, ours = FakeCore(), RecordingBackend()
    core = Core(real, device_setting=lambda: "cpu", backend=ours)
    x = np.zeros((6, 3), np.float32)
    core.knn(x, 2, "cpu")
    core.connectivities(np.zeros((6, 2), np.uint32), np.ones((6, 2), np.float32))
    assert [c[0] for c in real.calls] == ["knn", "connectivities"] and ours.calls == []
    # every other attribute is the reference module's
    real.pca = lambda *a: "pca"
    assert core.pca() == "pca"


def test_unmodified_neighbors_surface_through_the_core_on_cpu(monkeypatch):
    """pp.neighbors(device="cpu") through the swapped module reaches the
    reference's own core (a FakeCore here), arguments unchanged."""
    from mrustsc_gb300 import core as core_mod

    real, ours = FakeCore(), RecordingBackend()
    swapped = core_mod.Core(real, device_setting=lambda: "cpu", backend=ours)
    monkeypatch.setattr(pp, "_extension", lambda: swapped)
    adata = _adata()
    pp.neighbors(adata, n_neighbors=4, device="cpu")
    assert real.args_of("knn")[1:] == (3, "cpu") and ours.calls == []
    assert adata.obsp["distances"].shape == (N_OBS, N_OBS)
