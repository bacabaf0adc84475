"""kNN through the C ABI on the GPU, checked against the oracle.

Exact mode: neighbour lists equal the FP64 exact kNN (lowest-index
tie-break) bit for bit; distances within 1e-6 relative of FP64 (exact zeros
stay zero).  Reference-snap mode: equal, bit for bit, to the CPU twin of the
reference's Metal kernel.  Cases follow crates/scrust-gpu/src/kernels/knn.rs:339-415,
crates/scrust-core/src/neighbors.rs:408-446 and tests/test_neighbors_audit.py.
"""

from __future__ import annotations

import numpy as np
import pytest

import refdata
from mrustsc_gb300 import synthetic

pytestmark = pytest.mark.gpu

DIST_RTOL = 1e-6
FORMS = ["plain", "tensor", "tensor-ordered"]


def kw(form):
    """Keyword arguments of a form id: the ordered tensor form forces the row
    ordering on, so small inputs exercise the permuted operands and rerank."""
    if form == "tensor-ordered":
        return {"form": "tensor", "ordering": "on"}
    return {"form": form}


@pytest.fixture(scope="module")
def scrust(built_library):
    from mrustsc_gb300 import _scrust

    assert _scrust.gpu_available(), "these tests need an sm_103a GPU"
    return _scrust


def assert_exact(oracle, x, k, idx, dist, rows=None, metric="euclidean"):
    oi, od64, od = oracle.knn_fp64(x, k, rows, metric=metric)
    gi = idx if rows is None else idx[rows]
    gd = dist if rows is None else dist[rows]
    bad = np.nonzero((gi != oi).any(axis=1))[0]
    assert len(bad) == 0, f"{len(bad)} rows differ from FP64, first {bad[:5]}: {gi[bad[0]]} vs {oi[bad[0]]}"
    if metric == "cosine":
        np.testing.assert_array_equal(gd, od)
        return
    zero = od64 == 0
    assert np.all(gd[zero] == 0)
    rel = np.abs(gd[~zero].astype(np.float64) - od64[~zero]) / od64[~zero]
    assert rel.max(initial=0) <= DIST_RTOL, rel.max()


@pytest.mark.parametrize("form", FORMS)
def test_line_and_grid_known_answers(scrust, form):
    idx, dist = scrust.knn(refdata.line(6), 2, "auto", **kw(form))
    assert idx[0].tolist() == [1, 2] and dist[0].tolist() == [1.0, 2.0]
    assert idx[2].tolist() == [1, 3] and idx[5].tolist() == [4, 3]
    idx, dist = scrust.knn(refdata.grid(3), 4, "auto", **kw(form))
    assert idx[4].tolist() == [1, 3, 5, 7]
    assert idx[0].tolist() == [1, 3, 4, 2]
    assert abs(dist[0, 2] - np.sqrt(2.0)) < 1e-6 and abs(dist[0, 3] - 2.0) < 1e-6


@pytest.mark.parametrize("form", FORMS)
@pytest.mark.parametrize(("n", "d", "k"), [(64, 8, 1), (100, 5, 7), (257, 3, 15), (300, 32, 16)])
def test_random_embeddings_match_fp64(scrust, oracle, n, d, k, form):
    x = refdata.random_embedding(n, d, n)
    idx, dist = scrust.knn(x, k, "auto", **kw(form))
    assert_exact(oracle, x, k, idx, dist)


@pytest.mark.parametrize("k", [1, 2, 16, 17, 31, 32])
def test_ordered_solves_every_top_k_width(scrust, oracle, k):
    """Ordered tensor solves (3000 clustered cells) at the k that select each
    threshold-pass kind: k = 1 (one value a lane), 2..16 (a register top-16
    whose two column parts' lists are merged into each row's threshold) and
    17..32 (top-32)."""
    x = synthetic.mixture(3000, 20, clusters=6, dup_frac=0.01, seed=k)
    idx, dist = scrust.knn(x, k, "auto", form="tensor", ordering="on")
    assert_exact(oracle, x, k, idx, dist)


@pytest.mark.parametrize(("n", "d", "k"), [(64, 8, 1), (100, 5, 7), (257, 3, 15), (300, 32, 16)])
def test_reference_snap_equals_the_metal_twin(scrust, oracle, n, d, k):
    x = refdata.random_embedding(n, d, n)
    idx, dist = scrust.knn(x, k, "auto", mode="reference_snap")
    oi, od = oracle.knn_metal_twin(x, k)
    np.testing.assert_array_equal(idx, oi)
    np.testing.assert_array_equal(dist, od)


@pytest.mark.parametrize("form", FORMS)
def test_largest_supported_k(scrust, oracle, form):
    x = refdata.random_embedding(128 + 71, 4, 7)
    idx, dist = scrust.knn(x, 128, "auto", **kw(form))
    assert_exact(oracle, x, 128, idx, dist)


@pytest.mark.parametrize("form", FORMS)
def test_line_ties_and_forty_duplicates(scrust, form):
    idx, dist = scrust.knn(refdata.line(50), 2, "auto", **kw(form))
    assert idx[10].tolist() == [9, 11] and dist[10].tolist() == [1.0, 1.0]
    x = np.zeros((41, 2), np.float32)
    x[40, 0] = 100.0
    idx, _ = scrust.knn(x, 3, "auto", **kw(form))
    assert idx[5].tolist() == [0, 1, 2] and idx[0].tolist() == [1, 2, 3]


@pytest.mark.parametrize("form", FORMS)
def test_two_runs_are_identical(scrust, form):
    x = refdata.random_embedding(500, 6, 11)
    a = scrust.knn(x, 9, "auto", **kw(form))
    b = scrust.knn(x, 9, "auto", **kw(form))
    np.testing.assert_array_equal(a[0], b[0])
    np.testing.assert_array_equal(a[1], b[1])


@pytest.mark.parametrize("form", FORMS)
def test_plain_small_workload_matches_fp64(scrust, oracle, form):
    x = synthetic.plain_small(seed=0)
    for k in (15, 14):
        idx, dist = scrust.knn(x, k, "auto", **kw(form))
        assert_exact(oracle, x, k, idx, dist)


@pytest.mark.parametrize("precision", ["fp16", "bf16"])
def test_tensor_precisions_match_fp64(scrust, oracle, precision):
    x = synthetic.mixture(6000, 50, clusters=20, dup_frac=0.01, near_dup_frac=0.01, seed=12)
    idx, dist = scrust.knn(x, 15, "auto", form="tensor", precision=precision)
    assert_exact(oracle, x, 15, idx, dist)
    idx, dist = scrust.knn(x, 15, "auto", form="tensor", precision=precision, ordering="on")
    assert_exact(oracle, x, 15, idx, dist)


@pytest.mark.parametrize("form", FORMS)
@pytest.mark.parametrize("k,cap", [(15, 47), (24, 60), (40, 90)])
def test_small_list_capacity_forces_prunes(scrust, oracle, form, k, cap):
    """Short lists prune after nearly every tile: both prune paths (one list
    per lane for k <= 32, one list per warp above) and the overflow path."""
    x = synthetic.mixture(5000, 30, clusters=10, dup_frac=0.01, seed=21)
    idx, dist = scrust.knn(x, k, "auto", list_capacity=cap, **kw(form))
    assert_exact(oracle, x, k, idx, dist)


@pytest.mark.parametrize("form", FORMS)
def test_explicit_segments(scrust, oracle, form):
    x = synthetic.mixture(3000, 20, clusters=6, dup_frac=0.01, seed=22)
    for segments in (1, 2, 3):
        idx, dist = scrust.knn(x, 12, "auto", segments=segments, **kw(form))
        assert_exact(oracle, x, 12, idx, dist)


def test_plain_small_reference_snap_matches_twin_and_cpu_path(scrust, oracle):
    x = synthetic.plain_small(seed=1)
    idx, dist = scrust.knn(x, 15, "auto", mode="reference_snap")
    ti, td = oracle.knn_metal_twin(x, 15)
    np.testing.assert_array_equal(idx, ti)
    np.testing.assert_array_equal(dist, td)
    # Identical to the reference CPU path wherever its f32 distances are not
    # tied within its own expansion resolution.
    ci, cd = oracle.knn_reference_cpu(x, 15)
    c = oracle.centred(x)
    n2 = (c.astype(np.float64) ** 2).sum(1)
    res = 52 * np.finfo(np.float32).eps * 2 * n2.max()
    sq = cd.astype(np.float64) ** 2
    gaps = np.diff(sq, axis=1)
    untied = (gaps > res).all(axis=1) & (sq[:, 0] > res)
    assert untied.sum() > 0.5 * len(x)
    np.testing.assert_array_equal(idx[untied], ci[untied])


@pytest.mark.parametrize("form", FORMS)
@pytest.mark.parametrize("offset", [0.0, 1e2, 1e4, 1e5])
def test_far_from_the_origin(scrust, oracle, offset, form):
    x = (np.random.default_rng(2).normal(size=(300, 12)) + offset).astype(np.float32)
    idx, dist = scrust.knn(x, 14, "auto", **kw(form))
    assert_exact(oracle, x, 14, idx, dist)


@pytest.mark.parametrize("form", FORMS)
def test_lattice_ties_break_towards_the_smaller_index(scrust, oracle, form):
    side = 8
    lattice = np.array([[i, j] for i in range(side) for j in range(side)], dtype=np.float32)
    idx, dist = scrust.knn(lattice, 14, "auto", **kw(form))
    assert_exact(oracle, lattice, 14, idx, dist)


@pytest.mark.parametrize("form", FORMS)
def test_duplicates_sit_at_distance_zero(scrust, oracle, form):
    x = refdata.audit_embedding(180, 6, 5)
    x[20:30] = x[20]
    idx, dist = scrust.knn(x, 14, "auto", **kw(form))
    assert np.count_nonzero(dist == 0.0) == 10 * 9
    assert_exact(oracle, x, 14, idx, dist)
    x = refdata.audit_embedding(200, 6, 9)
    x[:20] = x[0]
    idx, dist = scrust.knn(x, 14, "auto", **kw(form))
    assert np.count_nonzero(dist[:20]) == 0
    assert_exact(oracle, x, 14, idx, dist)


@pytest.mark.parametrize("form", FORMS)
def test_many_duplicates_take_the_fallback(scrust, oracle, form):
    x = synthetic.mixture(1500, 20, clusters=5, dup_frac=0.0, seed=4)
    x[100:500] = x[100]  # 400 identical cells: far more than any candidate list holds
    idx, dist = scrust.knn(x, 15, "auto", **kw(form))
    assert_exact(oracle, x, 15, idx, dist)
    assert idx[100].tolist() == list(range(101, 116))


@pytest.mark.parametrize("k", [5, 15])
def test_tie_groups_of_copies_and_mirror_pairs(scrust, oracle, k):
    """Tie groups of both kinds, on a 1/16 lattice where every difference is
    exact: mirror pairs r + e, r - e (equal distances from r, different rows:
    ordered by FP64 then id) and triple copies (same rows: the sort's id order
    and the FP32 value stand).  Every form gives the FP64 ids and the same
    distance bits."""
    g = np.random.default_rng(31)
    x = (g.integers(-64, 64, size=(1200, 8)) / 16.0).astype(np.float32)
    for r in range(40):
        e = (g.integers(1, 4, size=8) / 64.0).astype(np.float32)
        x[200 + 2 * r] = x[r] + e
        x[201 + 2 * r] = x[r] - e
    for r in range(40, 80):
        x[400 + 3 * (r - 40):403 + 3 * (r - 40)] = x[r] + np.float32(1.0 / 32.0)
    outs = {}
    for form in FORMS:
        idx, dist = scrust.knn(x, k, "auto", **kw(form))
        assert_exact(oracle, x, k, idx, dist)
        outs[form] = (idx, dist)
    for form in FORMS[1:]:
        np.testing.assert_array_equal(outs[form][0], outs["plain"][0])
        np.testing.assert_array_equal(outs[form][1], outs["plain"][1])


def test_knot_below_resolution_collapses_like_the_reference(scrust, oracle):
    x = refdata.audit_embedding(150, 8, 21)
    x[:10] = x[0] + np.float32(1e-7) * np.arange(10, dtype=np.float32)[:, None]
    idx, dist = scrust.knn(x, 5, "auto", mode="reference_snap")
    ti, td = oracle.knn_metal_twin(x, 5)
    np.testing.assert_array_equal(idx, ti)
    np.testing.assert_array_equal(dist == 0.0, td == 0.0)
    # exact mode resolves the knot instead
    idx, dist = scrust.knn(x, 5, "auto")
    assert_exact(oracle, x, 5, idx, dist)


@pytest.mark.parametrize("form", FORMS)
def test_near_duplicates_and_high_dimension(scrust, oracle, form):
    x = synthetic.mixture(3000, 50, clusters=12, dup_frac=0.02, near_dup_frac=0.02, seed=8)
    idx, dist = scrust.knn(x, 30, "auto", **kw(form))
    assert_exact(oracle, x, 30, idx, dist)
    x = synthetic.mixture(700, 130, clusters=6, dup_frac=0.01, seed=9)
    idx, dist = scrust.knn(x, 10, "auto", **kw(form))
    assert_exact(oracle, x, 10, idx, dist)


@pytest.mark.parametrize("form", FORMS)
def test_cosine_matches_fp64_cosine(scrust, oracle, form):
    x = synthetic.mixture(2000, 50, clusters=10, dup_frac=0.01, near_dup_frac=0.01, seed=3)
    idx, dist = scrust.knn(x, 15, "auto", metric="cosine", **kw(form))
    assert_exact(oracle, x, 15, idx, dist, metric="cosine")


def test_cosine_rejects_zero_rows(scrust):
    x = refdata.random_embedding(50, 4, 1)
    x[3] = 0
    with pytest.raises(ValueError, match="non-zero norm"):
        scrust.knn(x, 3, "auto", metric="cosine")


@pytest.mark.slow
@pytest.mark.parametrize("form", FORMS)
def test_scale_workload_sampled_rows_match_fp64(scrust, oracle, form):
    x = synthetic.plain_scale(seed=0)
    idx, dist = scrust.knn(x, 30, "auto", **kw(form))
    n = len(x)
    assert np.all(np.diff(dist, axis=1) >= 0)
    assert not np.any(idx == np.arange(n, dtype=np.uint32)[:, None])
    rng = np.random.default_rng(0)
    dups = np.nonzero((dist[:, :1] < 1e-2).ravel())[0]
    rows = np.unique(np.concatenate([rng.choice(n, 300, replace=False), dups[:100]]))
    assert_exact(oracle, x, 30, idx, dist, rows=rows)
    ci, cd = scrust.knn(x, 30, "auto", metric="cosine", **kw(form))
    assert_exact(oracle, x, 30, ci, cd, rows=rows[:150], metric="cosine")


def test_default_form_runs_the_tensor_sweep_and_notes_fallbacks(scrust, oracle):
    """The default options pick the tensor form where it applies (exact mode,
    d <= 61: the sweep's own tile counter moves); an explicit tensor request
    it cannot serve runs the plain form, returns OK and says so."""
    import ctypes

    from mrustsc_gb300 import _lib

    L = _lib.lib()
    ctx = _lib.context(0)
    st = _lib.Status()
    opts = _lib.KnnOptions()
    L.scrust_knn_options_default(ctypes.byref(opts))
    assert opts.form == _lib.FORM_AUTO
    x = synthetic.mixture(3000, 50, clusters=6, dup_frac=0.01, seed=41)
    idx = np.empty((3000, 15), np.uint32)
    dist = np.empty((3000, 15), np.float32)
    cnt = (ctypes.c_uint64 * 16)()
    L.scrust_cuda_kernel_stats(ctx, 1, cnt, 16)
    _lib.check(L.scrust_cuda_knn(ctx, _lib.ptr(x), 3000, 50, 15, ctypes.byref(opts), _lib.ptr(idx), _lib.ptr(dist),
                                 ctypes.byref(st)), st)
    L.scrust_cuda_kernel_stats(ctx, 0, cnt, 16)
    assert cnt[8] > 0  # (row block, column tile) pairs of the tensor sweep
    assert st.message.decode() == ""
    assert_exact(oracle, x, 15, idx, dist)
    x100 = synthetic.mixture(800, 100, clusters=4, dup_frac=0.01, seed=42)
    tensor = _lib.options(form="tensor")
    idx = np.empty((800, 15), np.uint32)
    dist = np.empty((800, 15), np.float32)
    rc = L.scrust_cuda_knn(ctx, _lib.ptr(x100), 800, 100, 15, ctypes.byref(tensor), _lib.ptr(idx), _lib.ptr(dist),
                           ctypes.byref(st))
    assert rc == _lib.OK and "ran the plain form" in st.message.decode()
    assert_exact(oracle, x100, 15, idx, dist)
