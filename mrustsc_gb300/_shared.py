"""AnnData plumbing for the neighbours path, as python/scrust/_shared.py:22-102
defines it: the CSR dtypes, the lazy extension import, CSR assembly and the
``use_rep`` resolution."""

from __future__ import annotations

from typing import Any

import numpy as np
import scipy.sparse as sp

_INDEX_DTYPE = np.uint32
_VALUE_DTYPE = np.float32


def _extension():
    """The compiled core, imported on use so tests can replace it."""
    from . import _scrust

    return _scrust


def _csr_from_parts(parts, shape: tuple[int, int]) -> sp.csr_matrix:
    """CSR from (indptr, indices, values[, n_cols]); only the first three are read."""
    indptr, indices, values = parts[0], parts[1], parts[2]
    return sp.csr_matrix((values, indices, indptr), shape=shape)


def _dense(matrix: Any) -> np.ndarray:
    array = matrix.toarray() if sp.issparse(matrix) else np.asarray(matrix)
    return np.ascontiguousarray(array, dtype=_VALUE_DTYPE)


def _representation(adata, use_rep: str) -> np.ndarray:
    if use_rep == "X":
        return _dense(adata.X)
    if use_rep not in adata.obsm:
        raise KeyError(f"adata.obsm has no {use_rep!r}; run scrust.pp.pca first or pass use_rep")
    return _dense(adata.obsm[use_rep])
