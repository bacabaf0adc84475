"""The exact-PCA checker against scanpy's golden PCA of the reference's
300 x 200 fixture (crates/scrust-core/src/pca.rs tests), and the planted
spectrum the reference's tests recover.  CPU only."""

from __future__ import annotations

import json
import pathlib

import numpy as np

import refdata
from oracle import pca_oracle

GOLDEN = pathlib.Path(__file__).resolve().parent / "golden" / "pca_scanpy_300x200.json"


def test_exact_pca_matches_scanpy_golden():
    g = json.loads(GOLDEN.read_text())
    x = refdata.pca_scanpy_fixture()
    emb, comps, var, ratio = pca_oracle.exact_pca(x, g["bars"]["n_comps"])
    for c in range(3):
        assert abs(pca_oracle.correlation(emb[:, c], g["scanpy_embedding"][c])) >= g["bars"]["correlation_min"]
        tol = g["bars"]["variance_relative_tolerance"]
        assert abs(var[c] - g["scanpy_variance"][c]) <= tol * g["scanpy_variance"][c]
        assert abs(ratio[c] - g["scanpy_variance_ratio"][c]) <= tol * g["scanpy_variance_ratio"][c]


def test_exact_pca_recovers_the_planted_spectrum():
    x = refdata.pca_planted()
    _, _, var, ratio = pca_oracle.exact_pca(x, 6)
    assert abs(var[0] / var[1] - 720.0 / 320.0) < 0.1
    assert abs(var[1] / var[2] - 320.0 / 80.0) < 0.2
    assert ratio[:3].sum() > 0.9 and ratio[3] < 0.01
