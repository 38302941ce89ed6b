"""novaphy_gb300: NovaPhy's Position Based Fluids step on the GB300.

The C ABI (include/novaphy_pbf.h, libnovaphy_pbf.so) holds the sm_103a
kernels; ``novaphy_gb300._core`` mirrors NovaPhy's pybind11 fluid bindings
(python/bindings/bind_fluid.cpp) on top of it.  There is no CPU fallback:
importing the native parts fails loudly when they have not been built.
"""
from . import capi  # noqa: F401

try:
    from ._core import *  # noqa: F401,F403
    from ._core import __all__ as _core_all  # noqa: F401
except ImportError as _e:  # pragma: no cover - only before build()
    _core_import_error = _e
