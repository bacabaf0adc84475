"""A minimal AnnData stand-in with the slots ``pp.pca``, ``pp.neighbors``,
``tl.umap``, ``tl.leiden`` and ``tl.louvain`` read and write (``X``, ``obs``,
``obsm``, ``obsp``, ``varm``, ``uns``, ``n_obs``), for environments without
the ``anndata`` package.  Any object
with those attributes works."""

from __future__ import annotations

import numpy as np


class AnnData:
    def __init__(self, X=None, *, obsm: dict | None = None, n_obs: int | None = None):
        self.X = X
        self.obs: dict = {}
        self.obsm = dict(obsm or {})
        self.obsp: dict = {}
        self.varm: dict = {}
        self.uns: dict = {}
        if n_obs is None:
            n_obs = X.shape[0] if X is not None else next(iter(self.obsm.values())).shape[0]
        self.n_obs = int(n_obs)

    @property
    def shape(self):
        return (self.n_obs, 0 if self.X is None else np.shape(self.X)[1])
