"""The seeded workload generator: shapes, determinism, duplicate fractions."""

import numpy as np

from mrustsc_gb300 import synthetic


def test_plain_small_shape_and_duplicates():
    x = synthetic.plain_small(seed=3)
    assert x.shape == (2638, 50) and x.dtype == np.float32
    uniq = np.unique(x, axis=0)
    assert len(x) - len(uniq) == round(0.01 * 2638)
    np.testing.assert_array_equal(x, synthetic.plain_small(seed=3))


def test_near_duplicates_are_close_but_distinct():
    x = synthetic.mixture(4000, 50, clusters=40, dup_frac=0.005, near_dup_frac=0.005, seed=1)
    assert len(np.unique(x, axis=0)) == 4000 - 20
    near = np.sort(np.linalg.norm(x[:, None, :] - x[None, :50, :], axis=-1), axis=1)[:50]
    assert near.shape == (50, 50)


def test_spectrum_decays():
    x = synthetic.mixture(20000, 50, clusters=1, dup_frac=0.0, seed=2)
    sd = x.std(axis=0)
    np.testing.assert_allclose(sd, 2 / np.sqrt(np.arange(1, 51)), rtol=0.05)


def test_batch_and_serving_generators():
    samples = synthetic.batch_samples(seed=0, n_samples=6, lo=500, hi=2000)
    assert len(samples) == 6 and all(500 <= len(s) <= 2000 for s in samples)
    atlas, centres = synthetic.serving_atlas(seed=0, m=5000)
    q = synthetic.serving_queries(centres, 17, seed=5)
    assert atlas.shape == (5000, 50) and q.shape == (17, 50)
    t, c = synthetic.poisson_arrivals(200.0, 2.0, seed=1)
    assert 300 < len(t) < 500 and c.min() >= 1 and c.max() <= 20000
