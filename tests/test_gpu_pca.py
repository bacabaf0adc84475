"""PCA on the GPU (scrust_cuda_pca) against the reference's own PCA tests
(crates/scrust-core/src/pca.rs tests module: scanpy's golden PCA of the
300 x 200 fixture, the planted spectrum, reconstruction error, seeds,
uncentred statistics, argument errors) and against the exact FP64 PCA.

Parity is on the subspace, as the reference's own tests hold it: the GPU's
Gaussian sketch is its own counter-based one, not the reference's StdRng
stream.  Separated components correlate >= 0.999 with the exact PCA and their
explained variance is within 1e-3 relative; repeat runs are bit-identical.
"""

from __future__ import annotations

import json
import pathlib

import numpy as np
import pytest
import scipy.sparse as sp

import refdata
from oracle import pca_oracle

pytestmark = pytest.mark.gpu

GOLDEN = pathlib.Path(__file__).resolve().parent / "golden" / "pca_scanpy_300x200.json"


@pytest.fixture(scope="module")
def scrust(built_library):
    from mrustsc_gb300 import _scrust

    assert _scrust.gpu_available(), "these tests need an sm_103a GPU"
    return _scrust


def run(scrust, dense, k, zero_center=True, seed=0):
    m = sp.csr_matrix(dense)
    return scrust.pca(m.indptr.astype(np.uint32), m.indices.astype(np.uint32), m.data.astype(np.float32),
                      m.shape[1], k, zero_center, seed, "auto")


def test_matches_scanpy_on_the_reference_fixture(scrust):
    g = json.loads(GOLDEN.read_text())
    res = run(scrust, refdata.pca_scanpy_fixture(), g["bars"]["n_comps"])
    assert res["embedding"].shape == (300, 10) and res["components"].shape == (10, 200)
    tol = g["bars"]["variance_relative_tolerance"]
    for c in range(3):
        assert abs(pca_oracle.correlation(res["embedding"][:, c], g["scanpy_embedding"][c])) >= 0.99
        assert abs(res["explained_variance_ratio"][c] - g["scanpy_variance_ratio"][c]) <= tol * g["scanpy_variance_ratio"][c]
        assert abs(res["explained_variance"][c] - g["scanpy_variance"][c]) <= tol * g["scanpy_variance"][c]


def test_recovers_the_planted_spectrum_and_matches_the_exact_pca(scrust):
    x = refdata.pca_planted()
    res = run(scrust, x, 6)
    var = res["explained_variance"]
    assert abs(var[0] / var[1] - 720.0 / 320.0) < 0.1 and abs(var[1] / var[2] - 320.0 / 80.0) < 0.2
    assert np.all(np.diff(var) <= 0)
    assert res["explained_variance_ratio"][:3].sum() > 0.9 and res["explained_variance_ratio"][3] < 0.01
    emb, comps, evar, eratio = pca_oracle.exact_pca(x, 6)
    for c in range(3):
        assert pca_oracle.correlation(res["embedding"][:, c], emb[:, c]) >= 0.999
        assert pca_oracle.correlation(res["components"][c], comps[c]) >= 0.999
        assert abs(var[c] - evar[c]) <= 1e-3 * evar[c]


def test_reconstruction_error_falls_with_more_components(scrust):
    x = refdata.pca_planted().astype(np.float64)
    xc = x - x.mean(0)
    errs = []
    for k in (2, 3, 8):
        res = run(scrust, x, k)
        approx = res["embedding"].astype(np.float64) @ res["components"].astype(np.float64)
        errs.append(np.sqrt(((xc - approx) ** 2).sum() / (xc ** 2).sum()))
    assert errs[0] > errs[1] > errs[2] and errs[2] < 0.3


def test_seeds(scrust):
    x = refdata.pca_scanpy_fixture()
    a, b = run(scrust, x, 5, seed=3), run(scrust, x, 5, seed=3)
    for key in a:
        np.testing.assert_array_equal(a[key], b[key])
    c = run(scrust, x, 5, seed=999)
    d = run(scrust, x, 5, seed=0)
    for i in range(3):
        assert abs(pca_oracle.correlation(c["embedding"][:, i], d["embedding"][:, i])) >= 0.99


def test_uncentred_pca_reports_truncated_svd_statistics(scrust):
    x = refdata.pca_scanpy_fixture()
    res = run(scrust, x, 4, zero_center=False)
    var = res["explained_variance"]
    assert np.all(var > 0) and var[0] < var[1]
    for i in range(4):
        s = res["embedding"][:, i].astype(np.float64)
        assert abs(var[i] - s.var()) <= 1e-4 * s.var()
    _, _, evar, eratio = pca_oracle.exact_pca(x, 4, zero_center=False)
    np.testing.assert_allclose(res["explained_variance_ratio"][1:3], eratio[1:3], rtol=1e-3)


def test_pp_pca_feeds_pp_neighbors(built_library):
    from mrustsc_gb300 import pp
    from mrustsc_gb300.anndata_lite import AnnData

    adata = AnnData(sp.csr_matrix(refdata.pca_scanpy_fixture()))
    pp.pca(adata, n_comps=20)
    assert adata.obsm["X_pca"].shape == (300, 20) and adata.varm["PCs"].shape == (200, 20)
    assert adata.uns["pca"]["params"] == {"zero_center": True, "n_comps": 20, "random_state": 0}
    pp.neighbors(adata, n_neighbors=15)
    assert adata.obsp["connectivities"].shape == (300, 300)


def test_rejects_invalid_component_counts(scrust):
    x = np.array([[1.0, 2.0], [3.0, 4.0], [5.0, 6.0]], np.float32)
    with pytest.raises(ValueError):
        run(scrust, x, 0)
    with pytest.raises(ValueError):
        run(scrust, x, 3)
    res = run(scrust, x, 2)
    assert res["embedding"].shape == (3, 2)
