"""GB300-native (sm_103a) backend for scrust's ``pp.neighbors`` path.

``mrustsc_gb300.pp.neighbors`` mirrors ``scrust.pp.neighbors`` and
``mrustsc_gb300._scrust`` mirrors the neighbours half of the reference's
extension module; both run the CUDA library ``libscrust_cuda.so`` built from
``csrc/`` (C ABI in include/scrust_cuda.h).
"""

from . import pp  # noqa: F401

__all__ = ["pp"]
__version__ = "0.1.0"
