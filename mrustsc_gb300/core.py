"""The reference's extension module with its neighbours functions served by
this backend: the module swap a scrust installation makes to run its
unmodified ``pp.neighbors`` (python/scrust/pp/_basics.py:186-215) on a GB300.

Routing follows the reference's own device semantics
(crates/scrust-core/src/device.rs:20-35, crates/scrust-py/src/embedding.rs:42-58):

* ``knn(embedding, k, device)``: ``"cpu"`` goes to the reference's own
  module (its CPU path serves it); every other device name goes to this
  backend, which raises as the reference does for names it does not know and
  when no sm_103a GPU is present.
* ``connectivities(indices, distances)`` takes no device in the reference;
  it goes to the reference's module when the process-wide
  ``scrust.settings.device`` is ``"cpu"`` and to this backend otherwise.
* ``umap``, ``pca``, ``leiden`` and ``louvain`` take a device as their last
  argument and route as ``knn`` does; ``modularity`` takes none and routes
  as ``connectivities`` does.
* Every other attribute is the reference module's.

This is routing between the reference's implementation and this one, chosen
by the caller's device; this backend itself never falls back to a CPU path.
"""

from __future__ import annotations

import sys
from typing import Any, Callable

from . import _scrust


def settings_device() -> str:
    """The reference's process-wide default device, or "auto" when the
    reference's settings module is not importable."""
    try:
        from scrust.settings import settings
    except Exception:
        return "auto"
    return str(getattr(settings, "device", "auto"))


class Core:
    """Stands in for ``scrust._scrust`` with knn / connectivities routed."""

    def __init__(self, real: Any, device_setting: Callable[[], str] = settings_device, backend: Any = _scrust):
        self._real = real
        self._device_setting = device_setting
        self._backend = backend

    def __getattr__(self, name: str) -> Any:
        return getattr(self._real, name)

    def knn(self, embedding, k, device):
        if device == "cpu":
            return self._real.knn(embedding, k, device)
        return self._backend.knn(embedding, k, device)

    def connectivities(self, indices, distances):
        if self._device_setting() == "cpu":
            return self._real.connectivities(indices, distances)
        return self._backend.connectivities(indices, distances)

    def _by_device(self, name: str, args: tuple) -> Any:
        target = self._real if args[-1] == "cpu" else self._backend
        return getattr(target, name)(*args)

    def umap(self, *args):
        return self._by_device("umap", args)

    def pca(self, *args):
        return self._by_device("pca", args)

    def leiden(self, *args):
        return self._by_device("leiden", args)

    def louvain(self, *args):
        return self._by_device("louvain", args)

    def modularity(self, *args):
        target = self._real if self._device_setting() == "cpu" else self._backend
        return target.modularity(*args)

    def gpu_available(self) -> bool:
        return bool(self._backend.gpu_available())


def install() -> Core:
    """Replaces ``scrust._scrust`` (module and package attribute) with a Core
    over the installed reference extension; returns it."""
    import scrust
    import scrust._scrust as real

    core = Core(real)
    sys.modules["scrust._scrust"] = core
    scrust._scrust = core
    return core
