"""novaphy_gb300: NovaPhy's Position Based Fluids step on the GB300.

The C ABI (include/novaphy_pbf.h, libnovaphy_pbf.so) holds the sm_103a
kernels; ``novaphy_gb300._core`` mirrors NovaPhy's pybind11 fluid bindings
(python/bindings/bind_fluid.cpp) on top of it, so ``import novaphy_gb300 as
novaphy`` gives the reference's PBFSettings, PBFSolver, ParticleState,
FluidWorld, ... names.  There is no CPU fallback: the native parts must be
built (``__graft_entry__.build()``) and stepping needs a CUDA device.

The native module is loaded on first use of one of its names, so importing
the pure-Python parts (``workloads``, ``shard``) loads no native code.
"""
import importlib

from . import capi  # noqa: F401


def _native():
    return importlib.import_module("._core", __name__)


def __getattr__(name):
    if name.startswith("__"):
        raise AttributeError(name)
    try:
        core = _native()
    except ImportError as e:
        raise AttributeError(
            f"novaphy_gb300.{name}: the native module _core is not built or does not load "
            f"({e}); run __graft_entry__.build()") from e
    if name in globals():  # a submodule that the import just bound
        return globals()[name]
    try:
        value = getattr(core, name)
    except AttributeError:
        raise AttributeError(f"module 'novaphy_gb300' has no attribute {name!r}") from None
    globals()[name] = value
    return value


def __dir__():
    names = set(globals())
    try:
        names.update(n for n in dir(_native()) if not n.startswith("_"))
    except ImportError:
        pass
    return sorted(names)
