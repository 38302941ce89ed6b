"""In-tree build of the native parts of novaphy_gb300.

Produces, next to this file:
  libnovaphy_pbf.so  - the CUDA kernels and the C ABI (include/novaphy_pbf.h),
                       sm_103a only.
  _core*.so          - the pybind11 module mirroring NovaPhy's fluid bindings
                       (python/bindings/bind_fluid.cpp), a C++20 host layer
                       over the C ABI.

Translation units are compiled in parallel with nvcc / g++ directly (no
cmake).  Host code is compiled with -ffp-contract=off so that host-side
float constants round like the reference's on x86 and on Arm.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
import sysconfig

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
HOST = os.path.join(CSRC, "host")
INCLUDE = os.path.join(ROOT, "include")
BUILD = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "libnovaphy_pbf.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_COMMON = [
    *ARCH, "-O3", "-std=c++17", "-lineinfo", "--expt-relaxed-constexpr",
    "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off", "-I", INCLUDE, "-I", CSRC,
]
# Per-file arithmetic flags: the exact build must not contract a*b+c.
CU_FLAGS = {
    "pbf_exact.cu": ["-fmad=false", "-prec-div=true", "-prec-sqrt=true", "-ftz=false"],
    "pbf_fast.cu": ["-fmad=true", "-prec-div=false", "-prec-sqrt=false", "-ftz=false"],
    "pbf_boundary.cu": ["-fmad=false", "-prec-div=true", "-prec-sqrt=true", "-ftz=false"],
}
CU_SOURCES = ["radix_sort.cu", "pbf_exact.cu", "pbf_fast.cu", "pbf_boundary.cu", "pbf_capi.cu",
              "pbf_batch.cu", "pbf_serve.cu", "pbf_noalloc.cu"]


def nvcc() -> str:
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(cand):
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build novaphy_gb300")
    return cand


def _deps(src: str) -> list[str]:
    # This file holds the compiler flags: editing it rebuilds everything.
    out = [src, os.path.abspath(__file__)]
    for d in (CSRC, INCLUDE, HOST):
        if os.path.isdir(d):
            out += [os.path.join(d, f) for f in os.listdir(d) if f.endswith((".cuh", ".h", ".hpp"))]
    return out


def _stale(target: str, deps: list[str]) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def _run(cmd: list[str], verbose: bool) -> None:
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"command failed ({r.returncode}): {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    if verbose and (r.stdout.strip() or r.stderr.strip()):
        print(r.stdout + r.stderr, flush=True)


def _compile_cu(src: str, verbose: bool, extra: list[str]) -> str:
    obj = os.path.join(BUILD, os.path.basename(src) + ".o")
    if _stale(obj, _deps(os.path.join(CSRC, src))):
        _run([nvcc(), *NVCC_COMMON, *CU_FLAGS.get(src, []), *extra, "-c",
              os.path.join(CSRC, src), "-o", obj], verbose)
    return obj


def build_lib(verbose: bool = False, ptxas_verbose: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    extra = ["-Xptxas", "-v"] if ptxas_verbose else []
    with cf.ThreadPoolExecutor(max_workers=len(CU_SOURCES)) as ex:
        objs = list(ex.map(lambda s: _compile_cu(s, verbose, extra), CU_SOURCES))
    if _stale(LIB, objs):
        _run([nvcc(), *ARCH, "-shared", "-o", LIB + ".tmp", *objs, "-lcudart"], verbose)
        os.replace(LIB + ".tmp", LIB)
    return LIB


def _pybind_includes() -> list[str]:
    """pybind11 headers: the standalone package if present, else the copy torch ships."""
    incs = []
    try:
        import pybind11  # type: ignore

        incs.append(pybind11.get_include())
    except Exception:
        import torch  # noqa: F401  (only its header directory is used)

        incs.append(os.path.join(os.path.dirname(torch.__file__), "include"))
    incs.append(sysconfig.get_paths()["include"])
    return incs


def core_path() -> str:
    suffix = sysconfig.get_config_var("EXT_SUFFIX") or ".so"
    return os.path.join(PKG, "_core" + suffix)


def build_core(verbose: bool = False) -> str | None:
    """Builds the pybind11 host module when its sources are present."""
    if not os.path.isdir(HOST):
        return None
    srcs = sorted(os.path.join(HOST, f) for f in os.listdir(HOST) if f.endswith(".cpp"))
    if not srcs:
        return None
    os.makedirs(BUILD, exist_ok=True)
    out = core_path()
    incs = [f"-I{p}" for p in _pybind_includes()] + [f"-I{INCLUDE}", f"-I{HOST}", f"-I{CSRC}"]
    flags = ["-std=c++20", "-O2", "-fPIC", "-ffp-contract=off", "-fvisibility=hidden"]

    def comp(src: str) -> str:
        obj = os.path.join(BUILD, "host_" + os.path.basename(src) + ".o")
        if _stale(obj, [src] + _deps(src)):
            _run(["g++", *flags, *incs, "-c", src, "-o", obj], verbose)
        return obj

    with cf.ThreadPoolExecutor(max_workers=max(1, len(srcs))) as ex:
        objs = list(ex.map(comp, srcs))
    if _stale(out, objs + [LIB]):
        _run(["g++", "-shared", "-o", out + ".tmp", *objs, f"-L{PKG}", "-lnovaphy_pbf",
              "-Wl,-rpath,$ORIGIN"], verbose)
        os.replace(out + ".tmp", out)
    return out


def build(verbose: bool = False) -> None:
    build_lib(verbose)
    build_core(verbose)


if __name__ == "__main__":
    build(verbose="-v" in sys.argv)
