"""``tl.umap``, ``tl.leiden`` and ``tl.louvain`` with the reference's surface
(python/scrust/tl/_embedding.py:45-68, python/scrust/tl/_cluster.py:18-104):
UMAP lays out ``obsp["connectivities"]`` into ``obsm["X_umap"]``; the
clusterings write ``obs[key_added]`` and ``uns[key_added]``."""

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


def _connectivities(adata, neighbors_key: str):
    """The graph to cluster: the ``obsp`` key ``uns[neighbors_key]`` names,
    else ``obsp["connectivities"]`` (python/scrust/tl/_cluster.py:18-28)."""
    settings = adata.uns.get(neighbors_key)
    if isinstance(settings, dict):
        key = settings.get("connectivities_key", "connectivities")
        if key in adata.obsp:
            return adata.obsp[key]
    if "connectivities" not in adata.obsp:
        raise KeyError("adata.obsp has no 'connectivities'; run scrust.pp.neighbors first")
    return adata.obsp["connectivities"]


def _write_clusters(adata, key_added: str, partition, params: dict) -> None:
    """``obs[key_added]``: the labels as strings, categories "0".."n-1" (a
    pandas Categorical when pandas is importable, else a str array);
    ``uns[key_added]``: the parameters and the modularity
    (python/scrust/tl/_cluster.py:31-48)."""
    labels, modularity, n_communities = partition
    text = np.asarray(labels).astype("U")
    try:
        import pandas as pd
    except ImportError:
        adata.obs[key_added] = text
    else:
        adata.obs[key_added] = pd.Categorical(values=text,
                                              categories=[str(c) for c in range(n_communities)])
    adata.uns[key_added] = {"params": params, "modularity": modularity}


def leiden(adata, resolution: float = 1.0, *, key_added: str = "leiden", neighbors_key: str = "neighbors",
           n_iterations: int = 2, random_state: int = 0, device: str = "auto") -> None:
    """Leiden clustering, writing ``obs[key_added]`` as ``scanpy.tl.leiden`` does."""
    graph = _connectivities(adata, neighbors_key)
    partition = _extension().leiden(*_csr_args(graph), resolution, n_iterations, random_state, device)
    _write_clusters(adata, key_added, partition,
                    {"resolution": resolution, "random_state": random_state, "n_iterations": n_iterations})


def louvain(adata, resolution: float = 1.0, *, key_added: str = "louvain", neighbors_key: str = "neighbors",
            random_state: int = 0, device: str = "auto") -> None:
    """Louvain clustering, writing ``obs[key_added]`` as ``scanpy.tl.louvain`` does."""
    graph = _connectivities(adata, neighbors_key)
    partition = _extension().louvain(*_csr_args(graph), resolution, random_state, device)
    _write_clusters(adata, key_added, partition, {"resolution": resolution, "random_state": random_state})
