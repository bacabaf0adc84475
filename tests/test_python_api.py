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
    real.morans_i = lambda *a: "morans_i"
    assert core.morans_i() == "morans_i"


class Tagged:
    """Answers every call with (its own tag, the call's name, the args)."""

    def __init__(self, tag):
        self.tag = tag

    def __getattr__(self, name):
        return lambda *args: (self.tag, name, args)


@pytest.mark.parametrize("name,args", [
    ("umap", ("ip", "ix", "vl", 5, 2, 10, 0.5, 1.0, 1.0, 5, 0)),
    ("pca", ("ip", "ix", "vl", 5, 2, True, 0)),
    ("leiden", ("ip", "ix", "vl", 5, 1.0, 2, 0)),
    ("louvain", ("ip", "ix", "vl", 5, 1.0, 0)),
])
def test_core_routes_the_other_stages_by_their_device(name, args):
    from mrustsc_gb300.core import Core

    core = Core(Tagged("reference"), device_setting=lambda: "auto", backend=Tagged("gb300"))
    assert getattr(core, name)(*args, "cpu") == ("reference", name, args + ("cpu",))
    for device in ("auto", "gpu", "cuda:0"):
        assert getattr(core, name)(*args, device) == ("gb300", name, args + (device,))


def test_core_routes_modularity_by_the_settings_device():
    from mrustsc_gb300.core import Core

    args = ("ip", "ix", "vl", 5, "labels", 1.0)
    assert Core(Tagged("reference"), lambda: "cpu", Tagged("gb300")).modularity(*args)[0] == "reference"
    assert Core(Tagged("reference"), lambda: "auto", Tagged("gb300")).modularity(*args)[0] == "gb300"


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


class ClusterCore(FakeCore):
    def leiden(self, indptr, indices, values, n_cols, resolution, n_iterations, seed, device):
        self.calls.append(("leiden", (n_cols, resolution, n_iterations, seed, device), {}))
        return np.array([1, 0, 0, 1, 2, 0, 1], np.uint32), 0.25, 3

    def louvain(self, indptr, indices, values, n_cols, resolution, seed, device):
        self.calls.append(("louvain", (n_cols, resolution, seed, device), {}))
        return np.array([0, 0, 1, 1, 0, 1, 0], np.uint32), 0.5, 2


@pytest.fixture
def cluster_core(monkeypatch):
    fake = ClusterCore()
    import mrustsc_gb300.tl as tl
    monkeypatch.setattr(tl, "_extension", lambda: fake)
    return fake


def _graph_adata():
    adata = _adata()
    adata.obsp["connectivities"] = sp.csr_matrix(np.ones((N_OBS, N_OBS), np.float32) - np.eye(N_OBS, dtype=np.float32))
    return adata


def _labels_of(column):
    return [str(x) for x in np.asarray(column)]


def test_leiden_writes_obs_and_uns_as_scanpy(cluster_core):
    """python/scrust/tl/_cluster.py:51-79: obs[key] labels as strings,
    uns[key] = {params, modularity}; the arguments reach the core unchanged."""
    from mrustsc_gb300 import tl

    adata = _graph_adata()
    assert tl.leiden(adata, 0.7, n_iterations=3, random_state=4) is None
    assert cluster_core.args_of("leiden") == (N_OBS, 0.7, 3, 4, "auto")
    assert _labels_of(adata.obs["leiden"]) == ["1", "0", "0", "1", "2", "0", "1"]
    assert adata.uns["leiden"] == {"params": {"resolution": 0.7, "random_state": 4, "n_iterations": 3},
                                   "modularity": 0.25}


def test_louvain_writes_under_its_key(cluster_core):
    from mrustsc_gb300 import tl

    adata = _graph_adata()
    tl.louvain(adata, key_added="groups", random_state=2, device="cuda")
    assert cluster_core.args_of("louvain") == (N_OBS, 1.0, 2, "cuda")
    assert _labels_of(adata.obs["groups"]) == ["0", "0", "1", "1", "0", "1", "0"]
    assert adata.uns["groups"] == {"params": {"resolution": 1.0, "random_state": 2}, "modularity": 0.5}


def test_clustering_reads_the_graph_neighbors_key_names(cluster_core):
    """uns[neighbors_key]["connectivities_key"] picks the obsp entry
    (python/scrust/tl/_cluster.py:18-28); no graph at all raises KeyError."""
    from mrustsc_gb300 import tl

    adata = _adata()
    adata.obsp["alt"] = sp.csr_matrix(np.ones((N_OBS, N_OBS), np.float32))
    adata.uns["nbrs"] = {"connectivities_key": "alt"}
    tl.leiden(adata, neighbors_key="nbrs")
    assert "leiden" in adata.obs
    with pytest.raises(KeyError):
        tl.leiden(_adata())
