"""``tl.umap`` with the reference's surface (python/scrust/tl/_embedding.py:45-68):
lays out ``obsp["connectivities"]`` and writes ``obsm["X_umap"]``."""

from __future__ import annotations

import numpy as np
import scipy.sparse as sp

from ._shared import _INDEX_DTYPE, _VALUE_DTYPE, _extension

_DEFAULT_EPOCHS = 200
_UMAP_LEARNING_RATE = 1.0
_UMAP_NEGATIVE_SAMPLE_RATE = 5


def _csr_args(matrix):
    csr = matrix if isinstance(matrix, sp.csr_matrix) else sp.csr_matrix(matrix)
    return (csr.indptr.astype(_INDEX_DTYPE, copy=False), csr.indices.astype(_INDEX_DTYPE, copy=False),
            csr.data.astype(_VALUE_DTYPE, copy=False), csr.shape[1])


def umap(adata, *, n_components: int = 2, min_dist: float = 0.5, spread: float = 1.0, n_epochs: int | None = None,
         random_state: int = 0, device: str = "auto") -> None:
    """Lay the neighbour graph out with UMAP, writing `obsm["X_umap"]`."""
    if "connectivities" not in adata.obsp:
        raise KeyError("adata.obsp has no 'connectivities'; run scrust.pp.neighbors first")
    embedding = _extension().umap(*_csr_args(adata.obsp["connectivities"]), n_components,
                                  _DEFAULT_EPOCHS if n_epochs is None else n_epochs, min_dist, spread,
                                  _UMAP_LEARNING_RATE, _UMAP_NEGATIVE_SAMPLE_RATE, random_state, device)
    adata.obsm["X_umap"] = np.asarray(embedding, dtype=_VALUE_DTYPE)
