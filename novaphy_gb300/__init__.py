"""novaphy_gb300: NovaPhy's Position Based Fluids step on the GB300.

The C ABI (include/novaphy_pbf.h, libnovaphy_pbf.so) holds the sm_103a
kernels; ``novaphy_gb300._core`` mirrors NovaPhy's pybind11 fluid bindings
(python/bindings/bind_fluid.cpp) on top of it, so ``import novaphy_gb300 as
novaphy`` gives the reference's PBFSettings, PBFSolver, ParticleState,
FluidWorld, ... names.  There is no CPU fallback: the native parts must be
built (``__graft_entry__.build()``) and stepping needs a CUDA device.
"""
from . import capi  # noqa: F401

try:
    from ._core import *  # noqa: F401,F403
except ImportError as _e:  # only before build()
    _core_import_error = _e
