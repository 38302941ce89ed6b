"""Build recipe for the parity oracle (test infrastructure only).

* ``build_port()`` compiles the C restatement ``oracle/pbf_oracle.c`` into
  ``oracle/_build/liboracle_pbf.so`` with ``-O2 -ffp-contract=off`` (no fused
  multiply-add, so the operation order is the reference's on x86 and Arm).
* ``build_ref()`` compiles the reference's own, unmodified fluid sources from
  the NovaPhy tree named by ``$NOVAPHY_REFERENCE_ROOT`` (the fluid sources, src/sim/performance_monitor.cpp and
  the rigid World that FluidWorld inherits; see REF_SOURCES) with the C-ABI
  harness ``oracle/ref_harness.cpp`` against the Eigen-API subset in
  ``oracle/eigen_shim`` into ``oracle/_ref/libref_pbf.so``.  The reference's
  own CMake build needs Eigen3 and tinyxml2, which are not installed; it is
  never run.  When the reference tree is absent (the GPU host), this step is
  skipped.
"""
from __future__ import annotations

import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
# The NovaPhy source tree; $NOVAPHY_REFERENCE_ROOT overrides where it is read.
REFERENCE_ROOT = os.environ.get("NOVAPHY_REFERENCE_ROOT", "/root/reference")
REF_SOURCES = [
    "src/fluid/pbf_solver.cpp",
    "src/fluid/neighbor_search.cpp",
    "src/fluid/particle_state.cpp",
    "src/fluid/boundary.cpp",
    "src/fluid/fluid_world.cpp",
    "src/sim/performance_monitor.cpp",
    # the rigid World that FluidWorld inherits (free bodies, contacts)
    "src/sim/world.cpp",
    "src/sim/state.cpp",
    "src/core/body.cpp",
    "src/core/shape.cpp",
    "src/core/model_builder.cpp",
    "src/core/joint.cpp",
    "src/collision/broadphase.cpp",
    "src/collision/narrowphase.cpp",
    "src/dynamics/free_body_solver.cpp",
    "src/dynamics/integrator.cpp",
    "src/math/math_utils.cpp",
    "src/math/spatial.cpp",
]
PORT_LIB = os.path.join(HERE, "_build", "liboracle_pbf.so")
REF_LIB = os.path.join(HERE, "_ref", "libref_pbf.so")

FP_FLAGS = ["-O2", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-shared"]


def _newer(target: str, sources: list[str]) -> bool:
    if not os.path.exists(target):
        return False
    t = os.path.getmtime(target)
    return all(os.path.getmtime(s) <= t for s in sources)


def build_port(verbose: bool = False) -> str:
    src = os.path.join(HERE, "pbf_oracle.c")
    hdr = os.path.join(HERE, "pbf_oracle.h")
    if _newer(PORT_LIB, [src, hdr]):
        return PORT_LIB
    os.makedirs(os.path.dirname(PORT_LIB), exist_ok=True)
    cmd = ["gcc", "-std=c11", *FP_FLAGS, "-fopenmp", src, "-lm", "-o", PORT_LIB]
    if verbose:
        print(" ".join(cmd))
    if subprocess.call(cmd) != 0:
        # A host without OpenMP gets the single-threaded build.
        cmd.remove("-fopenmp")
        subprocess.check_call(cmd)
    return PORT_LIB


def reference_available() -> bool:
    return all(os.path.exists(os.path.join(REFERENCE_ROOT, s)) for s in REF_SOURCES)


def build_ref(verbose: bool = False) -> str | None:
    if not reference_available():
        return REF_LIB if os.path.exists(REF_LIB) else None
    srcs = [os.path.join(REFERENCE_ROOT, s) for s in REF_SOURCES]
    harness = os.path.join(HERE, "ref_harness.cpp")
    shim = [os.path.join(HERE, "eigen_shim", "Eigen", f) for f in ("Core", "Geometry", "Dense")]
    if _newer(REF_LIB, srcs + [harness] + shim):
        return REF_LIB
    os.makedirs(os.path.dirname(REF_LIB), exist_ok=True)
    cmd = [
        "g++", "-std=c++20", *FP_FLAGS,
        "-I", os.path.join(HERE, "eigen_shim"),
        "-I", os.path.join(REFERENCE_ROOT, "include"),
        "-DEIGEN_DEFAULT_DENSE_INDEX_TYPE=int",
        harness, *srcs, "-o", REF_LIB,
    ]
    if verbose:
        print(" ".join(cmd))
    subprocess.check_call(cmd)
    return REF_LIB


if __name__ == "__main__":
    print(build_port(verbose=True))
    print(build_ref(verbose=True))
    sys.exit(0)
