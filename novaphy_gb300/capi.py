"""ctypes binding of the C ABI in include/novaphy_pbf.h.

This is the thin Python view of ``libnovaphy_pbf.so`` used by tests and
bench.py; the user-facing NovaPhy API lives in ``novaphy_gb300._core``.
Loading fails loudly when the library has not been built: there is no CPU
fallback.
"""
from __future__ import annotations

import ctypes as C
import os
import re

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libnovaphy_pbf.so")
HEADER_PATH = os.path.join(os.path.dirname(_HERE), "include", "novaphy_pbf.h")

PBF_OK = 0
PBF_ERR_INVALID_ARG = 1
PBF_ERR_CUDA = 2
PBF_ERR_OOM = 3
PBF_ERR_TIMEOUT = 4
PBF_ERR_NO_DEVICE = 5
PBF_ERR_NONFINITE = 6
PBF_ERR_CAPACITY = 7

FIELD_POSITIONS = 0
FIELD_VELOCITIES = 1
FIELD_DENSITIES = 2
FIELD_LAMBDAS = 3


class PbfError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"pbf error {code}: {msg}")
        self.code = code


class Settings(C.Structure):
    """pbf_settings: PBFSettings field order plus the library's extensions."""

    _fields_ = [
        ("rest_density", C.c_float),
        ("kernel_radius", C.c_float),
        ("particle_radius", C.c_float),
        ("solver_iterations", C.c_int),
        ("epsilon", C.c_float),
        ("xsph_viscosity", C.c_float),
        ("vorticity_epsilon", C.c_float),
        ("corr_delta_q", C.c_float),
        ("corr_k", C.c_float),
        ("corr_n", C.c_int),
        ("use_domain_bounds", C.c_int),
        ("domain_lower", C.c_float * 3),
        ("domain_upper", C.c_float * 3),
        ("exact_arithmetic", C.c_int),
        ("hash_compat", C.c_int),
        ("boundary_two_way", C.c_int),
        ("boundary_friction", C.c_float),
    ]


_lib = None


def library_path() -> str:
    return LIB_PATH


def load() -> C.CDLL:
    """Loads libnovaphy_pbf.so (raises if it is missing: build it first)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise ImportError(
            f"{LIB_PATH} not found: build the CUDA extension with "
            "`python -c 'import __graft_entry__ as g; g.build()'`")
    L = C.CDLL(LIB_PATH)
    f32p = C.POINTER(C.c_float)
    vp = C.c_void_p
    sig = {
        "pbf_version": ([], C.c_char_p),
        "pbf_last_error": ([], C.c_char_p),
        "pbf_default_settings": ([C.POINTER(Settings)], C.c_int),
        "pbf_device_count": ([C.POINTER(C.c_int)], C.c_int),
        "pbf_scene_create": ([C.c_int, C.POINTER(Settings), C.c_int, vp, vp, C.c_float,
                              C.POINTER(vp)], C.c_int),
        "pbf_scene_destroy": ([vp], C.c_int),
        "pbf_scene_set_settings": ([vp, C.POINTER(Settings)], C.c_int),
        "pbf_scene_get_settings": ([vp, C.POINTER(Settings)], C.c_int),
        "pbf_scene_set_gravity": ([vp, f32p], C.c_int),
        "pbf_scene_set_mass": ([vp, C.c_float], C.c_int),
        "pbf_scene_num_particles": ([vp, C.POINTER(C.c_int)], C.c_int),
        "pbf_scene_reset": ([vp, C.c_int, vp, vp], C.c_int),
        "pbf_scene_step": ([vp, C.c_float, C.c_int], C.c_int),
        "pbf_scene_sync": ([vp], C.c_int),
        "pbf_scene_read": ([vp, C.c_int, vp], C.c_int),
        "pbf_scene_write": ([vp, C.c_int, vp], C.c_int),
        "pbf_scene_device_field": ([vp, C.c_int, C.POINTER(vp)], C.c_int),
        "pbf_scene_stream": ([vp, C.POINTER(vp)], C.c_int),
        "pbf_solver_step_host": ([vp, C.c_int, vp, vp, vp, vp, C.c_float, f32p, C.c_float],
                                 C.c_int),
        "pbf_scene_check_finite": ([vp], C.c_int),
        "pbf_scene_debug_cells": ([vp, C.c_float, vp], C.c_int),
        "pbf_scene_debug_neighbors": ([vp, C.c_float, vp, vp, C.c_longlong,
                                       C.POINTER(C.c_longlong)], C.c_int),
        "pbf_sort_pairs_host": ([C.c_int, C.c_int, vp, C.c_int, vp, vp], C.c_int),
        "pbf_phase_name": ([C.c_int], C.c_char_p),
        "pbf_scene_step_timed": ([vp, C.c_float, C.c_int, f32p], C.c_int),
        "pbf_snapshot_create": ([vp, C.POINTER(vp)], C.c_int),
        "pbf_snapshot_restore": ([vp, vp], C.c_int),
        "pbf_snapshot_destroy": ([vp], C.c_int),
        "pbf_snapshot_num_particles": ([vp, C.POINTER(C.c_int)], C.c_int),
        "pbf_scene_replay_timed": ([vp, vp, C.c_float, C.c_int, f32p], C.c_int),
        "pbf_scene_set_boundary": ([vp, C.c_int, vp, vp, vp], C.c_int),
        "pbf_scene_set_bodies": ([vp, C.c_int, vp, vp, vp], C.c_int),
        "pbf_scene_set_body_velocities": ([vp, C.c_int, vp, vp], C.c_int),
        "pbf_scene_step_coupled": ([vp, C.c_float, vp, vp], C.c_int),
        "pbf_scene_couple": ([vp, C.c_float, vp, vp], C.c_int),
        "pbf_scene_read_boundary": ([vp, vp], C.c_int),
        "pbf_boundary_volumes": ([C.c_int, C.c_int, vp, C.c_float, vp], C.c_int),
        "pbf_scene_step_profiled": ([vp, C.c_float, vp, vp], C.c_int),
        "pbf_batch_create": ([C.c_int, vp], C.c_int),
        "pbf_batch_destroy": ([vp], C.c_int),
        "pbf_batch_step": ([vp, C.c_int, vp, vp, vp], C.c_int),
        "pbf_batch_step_timed": ([vp, C.c_int, vp, vp, vp, f32p], C.c_int),
        "pbf_batch_replay_timed": ([vp, C.c_int, vp, vp, vp, C.c_int, f32p], C.c_int),
        "pbf_batch_sync": ([vp], C.c_int),
        "pbf_batch_device_bytes": ([vp, C.POINTER(C.c_size_t)], C.c_int),
        "pbf_scene_device_bytes": ([vp, C.POINTER(C.c_size_t)], C.c_int),
        "pbf_state_bytes_per_particle": ([], C.c_size_t),
        "pbf_batch_nonfinite": ([vp, C.c_int, vp], C.c_int),
        "pbf_batch_set_persistent": ([vp, C.c_int], C.c_int),
        "pbf_batch_set_autotune": ([vp, C.c_int], C.c_int),
        "pbf_batch_tuning": ([vp, vp, vp], C.c_int),
        "pbf_server_default_config": ([vp], C.c_int),
        "pbf_server_create": ([C.c_int, vp, vp], C.c_int),
        "pbf_server_destroy": ([vp], C.c_int),
        "pbf_server_open_scene": ([vp, vp, C.c_int, vp, vp, C.c_float, vp, vp, vp], C.c_int),
        "pbf_server_close_scene": ([vp, C.c_longlong], C.c_int),
        "pbf_server_submit": ([vp, C.c_longlong, C.c_float, C.c_int, vp], C.c_int),
        "pbf_server_wait": ([vp, C.c_longlong, C.c_double, vp], C.c_int),
        "pbf_server_read": ([vp, C.c_longlong, C.c_int, vp], C.c_int),
        "pbf_server_scene_state": ([vp, C.c_longlong, vp], C.c_int),
        "pbf_server_get_stats": ([vp, vp], C.c_int),
        "pbf_server_reset_stats": ([vp], C.c_int),
        "pbf_server_open_coupled_scene": ([vp, vp, C.c_int, vp, vp, C.c_float, vp, C.c_int, vp, vp,
                                           vp, C.c_int, vp, vp, vp], C.c_int),
        "pbf_server_read_bodies": ([vp, C.c_longlong, vp], C.c_int),
        "pbf_server_open_coupled_scene_contacts": (
            [vp, vp, C.c_int, vp, vp, C.c_float, vp, C.c_int, vp, vp, vp, C.c_int, vp, C.c_int, vp,
             vp, vp, vp], C.c_int),
        "pbf_host_alloc": ([C.c_size_t, C.POINTER(vp)], C.c_int),
        "pbf_host_free": ([vp], C.c_int),
    }
    for name, (args, res) in sig.items():
        fn = getattr(L, name)
        fn.argtypes = args
        fn.restype = res
    _lib = L
    return L


def declared_symbols() -> list[str]:
    """Function names declared in include/novaphy_pbf.h."""
    txt = open(HEADER_PATH).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(pbf_[a-z0-9_]+)\s*\(", txt)))


def check(rc: int) -> None:
    if rc != PBF_OK:
        msg = load().pbf_last_error()
        raise PbfError(rc, msg.decode() if msg else "")


def default_settings(**kw) -> Settings:
    s = Settings()
    check(load().pbf_default_settings(C.byref(s)))
    for k, v in kw.items():
        if k in ("domain_lower", "domain_upper"):
            getattr(s, k)[:] = [float(t) for t in v]
        elif k in ("use_domain_bounds", "exact_arithmetic", "hash_compat", "boundary_two_way"):
            setattr(s, k, int(bool(v)))
        else:
            setattr(s, k, v)
    return s


def device_count() -> int:
    n = C.c_int(0)
    load().pbf_device_count(C.byref(n))
    return n.value


def _f32(a, shape=None):
    a = np.ascontiguousarray(np.asarray(a, dtype=np.float32))
    return a.reshape(shape) if shape is not None else a


def _ptr(a):
    return a.ctypes.data_as(C.c_void_p)


class Scene:
    """Device-resident PBF scene (pbf_scene*)."""

    def __init__(self, settings: Settings, x, v=None, mass: float = 0.0, device: int = 0):
        L = load()
        x = _f32(x, (-1, 3))
        v = None if v is None else _f32(v, (-1, 3))
        h = C.c_void_p()
        check(L.pbf_scene_create(device, C.byref(settings), len(x), _ptr(x),
                                 None if v is None else _ptr(v), mass, C.byref(h)))
        self._h = h
        self._L = L

    @property
    def handle(self):
        return self._h

    def close(self):
        if self._h:
            self._L.pbf_scene_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def n(self) -> int:
        c = C.c_int()
        check(self._L.pbf_scene_num_particles(self._h, C.byref(c)))
        return c.value

    def set_settings(self, s: Settings):
        check(self._L.pbf_scene_set_settings(self._h, C.byref(s)))

    def get_settings(self) -> Settings:
        s = Settings()
        check(self._L.pbf_scene_get_settings(self._h, C.byref(s)))
        return s

    def set_gravity(self, g):
        g = _f32(g, (3,))
        check(self._L.pbf_scene_set_gravity(self._h, g.ctypes.data_as(C.POINTER(C.c_float))))

    def set_mass(self, m: float):
        check(self._L.pbf_scene_set_mass(self._h, m))

    def reset(self, x, v=None):
        x = _f32(x, (-1, 3))
        v = None if v is None else _f32(v, (-1, 3))
        check(self._L.pbf_scene_reset(self._h, len(x), _ptr(x), None if v is None else _ptr(v)))

    def step(self, dt: float, nsteps: int = 1, sync: bool = True):
        check(self._L.pbf_scene_step(self._h, dt, nsteps))
        if sync:
            self.sync()

    def step_timed(self, dt: float, nsteps: int) -> float:
        """Device milliseconds of `nsteps` steps (CUDA events on the scene stream)."""
        ms = C.c_float(0.0)
        check(self._L.pbf_scene_step_timed(self._h, dt, nsteps, C.byref(ms)))
        return ms.value

    # -- Akinci coupling --
    def set_boundary(self, local, body, psi):
        local = _f32(local, (-1, 3))
        body = np.ascontiguousarray(body, np.int32)
        psi = _f32(psi)
        check(self._L.pbf_scene_set_boundary(self._h, len(local), _ptr(local), _ptr(body),
                                             _ptr(psi)))
        self._nb = len(local)

    def set_bodies(self, pos, quat, dynamic):
        pos = _f32(pos, (-1, 3))
        quat = _f32(quat, (-1, 4))
        dyn = np.ascontiguousarray(dynamic, np.int32)
        check(self._L.pbf_scene_set_bodies(self._h, len(pos), _ptr(pos), _ptr(quat), _ptr(dyn)))

    def set_body_velocities(self, lin, ang):
        """World-frame linear and angular body velocities for the boundary
        friction of two-way steps (Settings.boundary_friction)."""
        lin = _f32(lin, (-1, 3))
        ang = _f32(ang, (-1, 3))
        if len(ang) != len(lin):
            raise ValueError("lin and ang must have one row per body")
        check(self._L.pbf_scene_set_body_velocities(self._h, len(lin), _ptr(lin), _ptr(ang)))

    def step_coupled(self, dt, force, torque):
        """One coupled fluid step; returns (force, torque) accumulated onto the inputs."""
        f = _f32(force, (-1, 3)).copy()
        t = _f32(torque, (-1, 3)).copy()
        check(self._L.pbf_scene_step_coupled(self._h, dt, _ptr(f), _ptr(t)))
        return f, t

    def couple(self, dt, force, torque):
        """The coupling half of step_coupled, after a step that ran elsewhere
        (e.g. in a batch); returns (force, torque) accumulated onto the inputs."""
        f = _f32(force, (-1, 3)).copy()
        t = _f32(torque, (-1, 3)).copy()
        check(self._L.pbf_scene_couple(self._h, dt, _ptr(f), _ptr(t)))
        return f, t

    def read_boundary(self):
        out = np.zeros((getattr(self, "_nb", 0), 3), np.float32)
        check(self._L.pbf_scene_read_boundary(self._h, _ptr(out)))
        return out

    def snapshot(self) -> "Snapshot":
        return Snapshot(self)

    def restore(self, snap: "Snapshot"):
        check(self._L.pbf_snapshot_restore(self._h, snap.handle))

    def replay_timed(self, seed: "Snapshot", dt: float, nsteps: int) -> float:
        """Device ms of nsteps x {restore seed; step}."""
        ms = C.c_float(0.0)
        check(self._L.pbf_scene_replay_timed(self._h, seed.handle, dt, nsteps, C.byref(ms)))
        return ms.value

    def sync(self):
        check(self._L.pbf_scene_sync(self._h))

    def read(self, field: int) -> np.ndarray:
        n = self.n
        shape = (n, 3) if field in (FIELD_POSITIONS, FIELD_VELOCITIES) else (n,)
        out = np.zeros(shape, np.float32)
        check(self._L.pbf_scene_read(self._h, field, _ptr(out)))
        return out

    def write(self, field: int, a):
        n = self.n
        a = _f32(a, (n, 3) if field in (FIELD_POSITIONS, FIELD_VELOCITIES) else (n,))
        check(self._L.pbf_scene_write(self._h, field, _ptr(a)))

    def state(self):
        return (self.read(FIELD_POSITIONS), self.read(FIELD_VELOCITIES),
                self.read(FIELD_DENSITIES), self.read(FIELD_LAMBDAS))

    def device_field(self, field: int) -> int:
        p = C.c_void_p()
        check(self._L.pbf_scene_device_field(self._h, field, C.byref(p)))
        return p.value or 0

    def stream(self) -> int:
        p = C.c_void_p()
        check(self._L.pbf_scene_stream(self._h, C.byref(p)))
        return p.value or 0

    def device_array(self, field: int) -> "DeviceArray":
        """Zero-copy view of a field in device memory: positions and
        velocities as (n, 3) float32 with row stride 16 bytes (float4 storage),
        densities and lambdas as (n,).  Waits for the scene's stream first, so
        the view holds the state after every step issued so far; it stays live
        (later steps show through once synchronised) until the scene is reset
        to more particles than it holds, restored from a larger snapshot, or
        closed.  Any consumer of __cuda_array_interface__ takes it, e.g.
        torch.as_tensor(view, device="cuda")."""
        ptr = self.device_field(field)
        self.sync()
        return DeviceArray(self, field, ptr, self.n)

    def check_finite(self) -> int:
        return self._L.pbf_scene_check_finite(self._h)

    def debug_cells(self, dt: float) -> np.ndarray:
        out = np.zeros((self.n, 3), np.int32)
        check(self._L.pbf_scene_debug_cells(self._h, dt, _ptr(out)))
        return out

    def debug_neighbors(self, dt: float):
        n = self.n
        offs = np.zeros(n + 1, np.int64)
        tot = C.c_longlong(0)
        check(self._L.pbf_scene_debug_neighbors(self._h, dt, _ptr(offs), None, 0, C.byref(tot)))
        out = np.zeros(max(tot.value, 1), np.int32)
        check(self._L.pbf_scene_debug_neighbors(self._h, dt, _ptr(offs), _ptr(out), tot.value,
                                                C.byref(tot)))
        return offs, out[:tot.value]

    def step_profiled(self, dt: float) -> dict:
        """One step with per-phase device times: {phase name: (ms, launches)}."""
        ms = np.zeros(NUM_PHASES, np.float32)
        nl = np.zeros(NUM_PHASES, np.int32)
        check(self._L.pbf_scene_step_profiled(self._h, dt, _ptr(ms), _ptr(nl)))
        return {phase_name(k): (float(ms[k]), int(nl[k])) for k in range(NUM_PHASES)}

    def solver_step_host(self, x, v, rho, lam, dt, g, mass):
        """pbf_solver_step_host on copies; returns the updated arrays."""
        x = _f32(x, (-1, 3)).copy()
        v = _f32(v, (-1, 3)).copy()
        rho = _f32(rho).copy()
        lam = _f32(lam).copy()
        g = _f32(g, (3,))
        check(self._L.pbf_solver_step_host(self._h, len(x), _ptr(x), _ptr(v), _ptr(rho),
                                           _ptr(lam), dt,
                                           g.ctypes.data_as(C.POINTER(C.c_float)), mass))
        return x, v, rho, lam


class _HostBlock:
    """Page-locked host memory from pbf_host_alloc, freed with its last view."""

    def __init__(self, nbytes: int):
        self.ptr = C.c_void_p()
        check(load().pbf_host_alloc(nbytes, C.byref(self.ptr)))

    def __del__(self):
        if self.ptr and self.ptr.value:
            load().pbf_host_free(self.ptr)
            self.ptr = None


def pinned_empty(shape, dtype=np.float32) -> np.ndarray:
    """An uninitialised numpy array in page-locked host memory (pbf_host_alloc),
    which the copies of pbf_solver_step_host and pbf_scene_read/write move by
    DMA without an intermediate pageable bounce."""
    dt = np.dtype(dtype)
    count = int(np.prod(shape))
    blk = _HostBlock(max(count * dt.itemsize, 1))
    buf = (C.c_byte * max(count * dt.itemsize, 1)).from_address(blk.ptr.value)
    buf._owner = blk  # the numpy array keeps buf, and buf the block, alive
    return np.frombuffer(buf, dtype=dt, count=count).reshape(shape)


def solver_step_host_inplace(scene: "Scene", x, v, rho, lam, dt, g, mass) -> None:
    """pbf_solver_step_host on the caller's arrays, updated in place (float32,
    C-contiguous; x and v n x 3)."""
    for a in (x, v, rho, lam):
        if a.dtype != np.float32 or not a.flags.c_contiguous:
            raise ValueError("arrays must be C-contiguous float32")
    g = _f32(g, (3,))
    check(scene._L.pbf_solver_step_host(scene.handle, len(x), _ptr(x), _ptr(v), _ptr(rho),
                                        _ptr(lam), dt, g.ctypes.data_as(C.POINTER(C.c_float)),
                                        mass))


def _handles(objs):
    arr = (C.c_void_p * max(len(objs), 1))()
    for k, o in enumerate(objs):
        arr[k] = o.handle
    return arr


def state_bytes_per_particle() -> int:
    return int(load().pbf_state_bytes_per_particle())


def scene_device_bytes(scene: "Scene") -> int:
    out = C.c_size_t(0)
    check(load().pbf_scene_device_bytes(scene.handle, C.byref(out)))
    return int(out.value)


class DeviceArray:
    """A scene field in device memory, exported through
    __cuda_array_interface__ (version 3).  Holds a reference to its scene."""

    def __init__(self, scene: "Scene", field: int, ptr: int, n: int):
        if field not in (FIELD_POSITIONS, FIELD_VELOCITIES, FIELD_DENSITIES, FIELD_LAMBDAS):
            raise ValueError("unknown field")
        self.scene = scene
        vec = field in (FIELD_POSITIONS, FIELD_VELOCITIES)
        self.shape = (n, 3) if vec else (n,)
        self.strides = (16, 4) if vec else (4,)
        self.ptr = ptr if n > 0 else 0

    @property
    def __cuda_array_interface__(self):
        return {"shape": self.shape, "typestr": "<f4", "data": (self.ptr, False),
                "strides": self.strides, "version": 3}


class Batch:
    """A batch context (pbf_batch*): steps many scenes with one launch per phase."""

    def __init__(self, device: int = 0):
        self._L = load()
        h = C.c_void_p()
        check(self._L.pbf_batch_create(device, C.byref(h)))
        self._h = h

    @property
    def handle(self):
        return self._h

    def close(self):
        if self._h:
            self._L.pbf_batch_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @staticmethod
    def _args(scenes, dt, nsteps):
        ns = len(scenes)
        dts = np.ascontiguousarray(np.broadcast_to(np.float32(dt) if np.isscalar(dt) else
                                                   np.asarray(dt, np.float32), (ns,)), np.float32)
        steps = None
        if nsteps is not None:
            steps = np.ascontiguousarray(np.broadcast_to(np.asarray(nsteps, np.int32), (ns,)),
                                         np.int32)
        return ns, _handles(scenes), dts, steps

    def step(self, scenes, dt, nsteps=None, sync: bool = True):
        ns, hs, dts, steps = self._args(scenes, dt, nsteps)
        check(self._L.pbf_batch_step(self._h, ns, hs, _ptr(dts),
                                     _ptr(steps) if steps is not None else None))
        if sync:
            self.sync()

    def step_timed(self, scenes, dt, nsteps=None) -> float:
        ns, hs, dts, steps = self._args(scenes, dt, nsteps)
        ms = C.c_float(0.0)
        check(self._L.pbf_batch_step_timed(self._h, ns, hs, _ptr(dts),
                                           _ptr(steps) if steps is not None else None,
                                           C.byref(ms)))
        return ms.value

    def replay_timed(self, scenes, seeds, dt, nsteps: int) -> float:
        ns, hs, dts, _ = self._args(scenes, dt, None)
        ms = C.c_float(0.0)
        check(self._L.pbf_batch_replay_timed(self._h, ns, hs, _handles(seeds), _ptr(dts),
                                             nsteps, C.byref(ms)))
        return ms.value

    def sync(self):
        check(self._L.pbf_batch_sync(self._h))

    def set_persistent(self, on: bool = True):
        check(self._L.pbf_batch_set_persistent(self._h, 1 if on else 0))

    def set_autotune(self, on: bool = True):
        check(self._L.pbf_batch_set_autotune(self._h, 1 if on else 0))

    def tuning(self) -> tuple[int, int]:
        blk, per = C.c_int(0), C.c_int(0)
        check(self._L.pbf_batch_tuning(self._h, C.byref(blk), C.byref(per)))
        return blk.value, per.value

    def device_bytes(self) -> int:
        out = C.c_size_t(0)
        check(self._L.pbf_batch_device_bytes(self._h, C.byref(out)))
        return int(out.value)

    def nonfinite(self, nscenes: int) -> np.ndarray:
        out = np.zeros(max(nscenes, 1), np.int32)
        check(self._L.pbf_batch_nonfinite(self._h, nscenes, _ptr(out)))
        return out[:nscenes]


SCENE_WAITING, SCENE_RESIDENT, SCENE_FAILED = 0, 1, 2
REQ_PENDING, REQ_DONE, REQ_FAILED = 0, 1, 2


class RigidBody(C.Structure):
    """pbf_rigid_body: pose (quaternion w, x, y, z), velocities, inverse mass and inertia."""

    _fields_ = [
        ("pos", C.c_float * 3),
        ("quat", C.c_float * 4),
        ("lin_vel", C.c_float * 3),
        ("ang_vel", C.c_float * 3),
        ("inv_mass", C.c_float),
        ("inv_inertia", C.c_float * 9),
    ]


SHAPE_SPHERE = 0
SHAPE_PLANE = 1


class RigidShape(C.Structure):
    """pbf_rigid_shape: a sphere on a body or a world plane of a served scene's contacts."""

    _fields_ = [
        ("type", C.c_int),
        ("body", C.c_int),
        ("radius", C.c_float),
        ("local_pos", C.c_float * 3),
        ("normal", C.c_float * 3),
        ("offset", C.c_float),
        ("friction", C.c_float),
        ("restitution", C.c_float),
    ]


class ContactSettings(C.Structure):
    """pbf_contact_settings: the contact solve's SolverSettings."""

    _fields_ = [
        ("velocity_iterations", C.c_int),
        ("baumgarte", C.c_float),
        ("slop", C.c_float),
        ("warm_starting", C.c_int),
    ]

    @classmethod
    def make(cls, velocity_iterations=30, baumgarte=0.3, slop=0.005, warm_starting=True):
        return cls(velocity_iterations, baumgarte, slop, 1 if warm_starting else 0)


class ServerConfig(C.Structure):
    """pbf_server_config."""

    _fields_ = [
        ("hbm_budget_bytes", C.c_size_t),
        ("max_batch_particles", C.c_int),
        ("max_batch_scenes", C.c_int),
        ("max_inflight", C.c_int),
        ("min_step_particles", C.c_int),
    ]


class ServerStats(C.Structure):
    """pbf_server_stats."""

    _fields_ = [
        ("scenes_resident", C.c_longlong), ("scenes_waiting", C.c_longlong),
        ("scenes_rejected", C.c_longlong), ("scenes_failed", C.c_longlong),
        ("requests_submitted", C.c_longlong), ("requests_done", C.c_longlong),
        ("requests_failed", C.c_longlong), ("steps_done", C.c_longlong),
        ("particle_steps", C.c_longlong), ("launches", C.c_longlong),
        ("queue_depth", C.c_longlong),
        ("step_ms_p50", C.c_double), ("step_ms_p99", C.c_double),
        ("request_ms_p50", C.c_double), ("request_ms_p99", C.c_double),
        ("particle_steps_per_s", C.c_double),
        ("mean_launch_scenes", C.c_double), ("mean_launch_particles", C.c_double),
        ("hbm_bytes_charged", C.c_size_t), ("hbm_bytes_scratch", C.c_size_t),
        ("state_bytes_per_particle", C.c_size_t), ("grid_bytes_per_slot", C.c_size_t),
        ("issue_ms_mean", C.c_double), ("graph_captures", C.c_longlong),
        ("graph_updates", C.c_longlong), ("graph_instantiations", C.c_longlong),
        ("launches_direct", C.c_longlong), ("post_ms_mean", C.c_double),
    ]

    def as_dict(self) -> dict:
        return {k: getattr(self, k) for k, _ in self._fields_}


def server_config(**kw) -> ServerConfig:
    c = ServerConfig()
    check(load().pbf_server_default_config(C.byref(c)))
    for k, v in kw.items():
        setattr(c, k, v)
    return c


class Server:
    """The serving loop (pbf_server*): device-resident scenes, continuous batching."""

    def __init__(self, config: ServerConfig | None = None, device: int = 0):
        self._L = load()
        cfg = config if config is not None else server_config()
        h = C.c_void_p()
        check(self._L.pbf_server_create(device, C.byref(cfg), C.byref(h)))
        self._h = h

    def close(self):
        if self._h:
            self._L.pbf_server_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def open_scene(self, settings: Settings, x, v=None, mass: float = 0.0, gravity=None):
        x = _f32(x, (-1, 3))
        vv = _f32(v, x.shape) if v is not None else None
        g = _f32(gravity, (3,)) if gravity is not None else None
        sid, st = C.c_longlong(0), C.c_int(0)
        check(self._L.pbf_server_open_scene(self._h, C.byref(settings), len(x), _ptr(x),
                                            _ptr(vv) if vv is not None else None, mass,
                                            _ptr(g) if g is not None else None, C.byref(sid),
                                            C.byref(st)))
        return sid.value, st.value

    def open_coupled_scene(self, settings: Settings, x, v, mass, gravity, local, body, psi,
                           bodies, shapes=None, contact_settings=None):
        """A FluidWorld-like scene: boundary particles (local, body, psi) owned by
        `bodies` (a sequence of RigidBody) that the server advances after each step:
        as free bodies, or, with `shapes` (a sequence of RigidShape, spheres and
        planes), through World's contact pipeline with `contact_settings`
        (ContactSettings, default SolverSettings())."""
        x = _f32(x, (-1, 3))
        vv = _f32(v, x.shape) if v is not None else None
        g = _f32(gravity, (3,))
        local = _f32(local, (-1, 3))
        body = np.ascontiguousarray(body, np.int32)
        psi = _f32(psi)
        arr = (RigidBody * max(len(bodies), 1))(*bodies)
        sid, st = C.c_longlong(0), C.c_int(0)
        if shapes:
            sarr = (RigidShape * len(shapes))(*shapes)
            cs = contact_settings if contact_settings is not None else ContactSettings.make()
            check(self._L.pbf_server_open_coupled_scene_contacts(
                self._h, C.byref(settings), len(x), _ptr(x),
                _ptr(vv) if vv is not None else None, mass, _ptr(g), len(local), _ptr(local),
                _ptr(body), _ptr(psi), len(bodies), arr, len(shapes), sarr, C.byref(cs),
                C.byref(sid), C.byref(st)))
            return sid.value, st.value
        check(self._L.pbf_server_open_coupled_scene(
            self._h, C.byref(settings), len(x), _ptr(x), _ptr(vv) if vv is not None else None,
            mass, _ptr(g), len(local), _ptr(local), _ptr(body), _ptr(psi), len(bodies), arr,
            C.byref(sid), C.byref(st)))
        return sid.value, st.value

    def read_bodies(self, sid: int, nbodies: int):
        arr = (RigidBody * max(nbodies, 1))()
        check(self._L.pbf_server_read_bodies(self._h, sid, arr))
        return list(arr)[:nbodies]

    def close_scene(self, sid: int):
        check(self._L.pbf_server_close_scene(self._h, sid))

    def submit(self, sid: int, dt: float, nsteps: int) -> int:
        rid = C.c_longlong(0)
        check(self._L.pbf_server_submit(self._h, sid, dt, nsteps, C.byref(rid)))
        return rid.value

    def wait(self, rid: int, timeout: float = -1.0) -> int:
        st = C.c_int(0)
        check(self._L.pbf_server_wait(self._h, rid, timeout, C.byref(st)))
        return st.value

    def read(self, sid: int, field: int, n: int) -> np.ndarray:
        shape = (n, 3) if field in (FIELD_POSITIONS, FIELD_VELOCITIES) else (n,)
        out = np.zeros(shape, np.float32)
        check(self._L.pbf_server_read(self._h, sid, field, _ptr(out)))
        return out

    def scene_state(self, sid: int) -> int:
        st = C.c_int(0)
        check(self._L.pbf_server_scene_state(self._h, sid, C.byref(st)))
        return st.value

    def stats(self) -> dict:
        s = ServerStats()
        check(self._L.pbf_server_get_stats(self._h, C.byref(s)))
        return s.as_dict()

    def reset_stats(self):
        check(self._L.pbf_server_reset_stats(self._h))


class Snapshot:
    """Device-resident copy of a scene's particle state (pbf_snapshot*)."""

    def __init__(self, scene: Scene):
        h = C.c_void_p()
        check(load().pbf_snapshot_create(scene.handle, C.byref(h)))
        self._h = h

    @property
    def handle(self):
        return self._h

    def close(self):
        if self._h:
            load().pbf_snapshot_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def boundary_volumes(world, kernel_radius: float, device: int = 0):
    world = _f32(world, (-1, 3))
    psi = np.zeros(len(world), np.float32)
    check(load().pbf_boundary_volumes(device, len(world), _ptr(world), kernel_radius, _ptr(psi)))
    return psi


NUM_PHASES = 7


def phase_name(k: int) -> str:
    return load().pbf_phase_name(k).decode()


def sort_pairs(keys, key_bits: int, device: int = 0):
    keys = np.ascontiguousarray(keys, dtype=np.uint32)
    ko = np.zeros_like(keys)
    vo = np.zeros_like(keys)
    check(load().pbf_sort_pairs_host(device, len(keys), _ptr(keys), key_bits, _ptr(ko), _ptr(vo)))
    return ko, vo
