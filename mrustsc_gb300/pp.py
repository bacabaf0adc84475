"""``pp.neighbors`` with the reference's surface (python/scrust/pp/_basics.py:186-215),
plus the ``metric`` keyword the scanpy API has ("euclidean" or "cosine").

Stores ``obsp["distances"]`` (one fixed-width row per cell, nearest first,
stored zeros kept), ``obsp["connectivities"]`` (UMAP fuzzy union) and
``uns["neighbors"]`` exactly as the reference does.
"""

from __future__ import annotations

import numpy as np

from ._shared import _INDEX_DTYPE, _VALUE_DTYPE, _csr_from_parts, _extension, _representation

METRICS = ("euclidean", "cosine")


def neighbors(adata, *, n_neighbors: int = 15, use_rep: str = "X_pca", device: str = "auto",
              metric: str = "euclidean", form: str = "auto") -> None:
    """Build the k-nearest-neighbour graph and its UMAP connectivities."""
    if n_neighbors < 2:
        raise ValueError(f"n_neighbors must be at least 2, got {n_neighbors}")
    if metric not in METRICS:
        raise ValueError(f"metric must be one of {list(METRICS)}, got {metric!r}")
    extension = _extension()
    # scanpy counts the cell itself among its n_neighbors; the core does not.
    kwargs = {} if metric == "euclidean" and form == "auto" else {"metric": metric, "form": form}
    indices, distances = extension.knn(_representation(adata, use_rep), n_neighbors - 1, device, **kwargs)
    indices = np.asarray(indices)
    distances = np.asarray(distances, dtype=_VALUE_DTYPE)

    n_obs, k = indices.shape
    indptr = np.arange(0, n_obs * k + 1, k, dtype=_INDEX_DTYPE)
    adata.obsp["distances"] = _csr_from_parts((indptr, indices.ravel(), distances.ravel()), (n_obs, n_obs))
    adata.obsp["connectivities"] = _csr_from_parts(extension.connectivities(indices, distances), (n_obs, n_obs))
    params = {"n_neighbors": n_neighbors, "method": "umap", "use_rep": use_rep}
    if metric != "euclidean":
        params["metric"] = metric
    adata.uns["neighbors"] = {
        "connectivities_key": "connectivities",
        "distances_key": "distances",
        "params": params,
    }


def pca(adata, *, n_comps: int = 50, zero_center: bool = True, random_state: int = 0, device: str = "auto") -> None:
    """Principal component analysis by randomised SVD (python/scrust/pp/_basics.py:166-183)."""
    import scipy.sparse as sp

    from ._shared import _INDEX_DTYPE

    x = adata.X if isinstance(adata.X, sp.csr_matrix) else sp.csr_matrix(adata.X)
    result = _extension().pca(x.indptr.astype(_INDEX_DTYPE, copy=False), x.indices.astype(_INDEX_DTYPE, copy=False),
                              x.data.astype(_VALUE_DTYPE, copy=False), x.shape[1], n_comps, zero_center, random_state,
                              device)
    adata.obsm["X_pca"] = np.asarray(result["embedding"], dtype=_VALUE_DTYPE)
    adata.varm["PCs"] = np.asarray(result["components"], dtype=_VALUE_DTYPE).T.copy()
    adata.uns["pca"] = {
        "variance_ratio": np.asarray(result["explained_variance_ratio"], dtype=_VALUE_DTYPE),
        "variance": np.asarray(result["explained_variance"], dtype=_VALUE_DTYPE),
        "params": {"zero_center": zero_center, "n_comps": n_comps, "random_state": random_state},
    }
