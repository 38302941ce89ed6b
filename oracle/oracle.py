"""ctypes front end of the parity oracle (test infrastructure only).

Only tests/, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline leg use
this module, and only as the checker.  Two back ends share one interface:

* ``Port``: the C restatement (oracle/pbf_oracle.c), built on any host.
* ``Ref``: the reference's own PBF sources compiled by oracle/build_oracle.py
  (only where the reference tree is present).

Arrays are float32, positions/velocities shaped (n, 3).
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import build_oracle

_f32p = np.ctypeslib.ndpointer(np.float32, flags="C_CONTIGUOUS")
_i32p = np.ctypeslib.ndpointer(np.int32, flags="C_CONTIGUOUS")
_i64p = np.ctypeslib.ndpointer(np.int64, flags="C_CONTIGUOUS")


class Settings(C.Structure):
    """Field order of PBFSettings (include/novaphy/fluid/pbf_solver.h:13-38)."""

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
    ]

    @classmethod
    def make(cls, **kw) -> "Settings":
        s = cls()
        defaults = dict(
            rest_density=1000.0, kernel_radius=0.1, particle_radius=0.025, solver_iterations=4,
            epsilon=100.0, xsph_viscosity=0.01, vorticity_epsilon=0.0, corr_delta_q=0.3,
            corr_k=0.001, corr_n=4, use_domain_bounds=0,
            domain_lower=(-10.0, 0.0, -10.0), domain_upper=(10.0, 10.0, 10.0),
        )
        defaults.update(kw)
        for k, v in defaults.items():
            if k in ("domain_lower", "domain_upper"):
                getattr(s, k)[:] = [float(t) for t in v]
            elif k in ("use_domain_bounds",):
                setattr(s, k, int(bool(v)))
            else:
                setattr(s, k, v)
        return s

    def as_dict(self) -> dict:
        d = {f: getattr(self, f) for f, _ in self._fields_}
        d["domain_lower"] = tuple(self.domain_lower)
        d["domain_upper"] = tuple(self.domain_upper)
        return d


def _f32(a, shape=None):
    a = np.ascontiguousarray(np.asarray(a, dtype=np.float32))
    if shape is not None:
        a = a.reshape(shape)
    return a


class Port:
    """The C restatement."""

    def __init__(self, path: str | None = None):
        path = path or build_oracle.build_port()
        L = self.lib = C.CDLL(path)
        L.orc_pbf_step.argtypes = [C.POINTER(Settings), C.c_int, _f32p, _f32p, _f32p, _f32p,
                                   C.c_float, _f32p, C.c_float]
        L.orc_pbf_step.restype = C.c_int
        L.orc_set_threads.argtypes = [C.c_int]
        L.orc_max_threads.restype = C.c_int
        L.orc_poly6.argtypes = [C.c_float, C.c_float]
        L.orc_poly6.restype = C.c_float
        L.orc_spiky.argtypes = [C.c_float, C.c_float]
        L.orc_spiky.restype = C.c_float
        L.orc_cubic_spline.argtypes = [C.c_float, C.c_float]
        L.orc_cubic_spline.restype = C.c_float
        L.orc_spiky_grad.argtypes = [_f32p, C.c_float, _f32p]
        L.orc_cell_coords.argtypes = [_f32p, C.c_int, C.c_float, _i32p]
        L.orc_grid_query.argtypes = [_f32p, C.c_int, C.c_float, _f32p, _i32p, C.c_int]
        L.orc_grid_query.restype = C.c_int
        L.orc_hash_collisions.argtypes = [_f32p, C.c_int, C.c_float]
        L.orc_hash_collisions.restype = C.c_int
        L.orc_neighbor_sets.argtypes = [_f32p, C.c_int, C.c_float, C.c_void_p, C.c_void_p,
                                        C.c_longlong]
        L.orc_neighbor_sets.restype = C.c_longlong
        L.orc_predict.argtypes = [C.c_int, _f32p, _f32p, C.c_float, _f32p, _f32p, _f32p]
        L.orc_boundary_world_positions.argtypes = [C.c_int, _f32p, _i32p, C.c_int, _f32p, _f32p,
                                                   _f32p]
        L.orc_boundary_volumes.argtypes = [C.c_int, _f32p, C.c_float, _f32p]
        L.orc_boundary_volumes.restype = C.c_int
        L.orc_boundary_density.argtypes = [C.c_int, _f32p, _f32p, C.c_int, _f32p, _f32p,
                                           C.c_float, C.c_float]
        L.orc_boundary_density.restype = C.c_int
        L.orc_coupling_forces.argtypes = [C.c_int, _f32p, _f32p, C.c_float, C.c_int, _f32p, _i32p,
                                          _f32p, C.c_int, _i32p, _f32p, C.c_float, C.c_float,
                                          _f32p, _f32p]
        L.orc_coupling_forces.restype = C.c_int
        for fn in ("orc_sample_box",):
            getattr(L, fn).argtypes = [_f32p, _f32p, _f32p, C.c_float, C.c_void_p, C.c_int]
            getattr(L, fn).restype = C.c_int
        L.orc_sample_sphere.argtypes = [C.c_float, _f32p, _f32p, C.c_float, C.c_void_p, C.c_int]
        L.orc_sample_sphere.restype = C.c_int
        L.orc_sample_plane.argtypes = [_f32p, C.c_float, C.c_float, C.c_float, C.c_void_p,
                                       C.c_int]
        L.orc_sample_plane.restype = C.c_int
        L.orc_generate_block.argtypes = [_f32p, _f32p, C.c_float, C.c_void_p, C.c_int]
        L.orc_generate_block.restype = C.c_int

    # -- kernels --
    def poly6(self, r_sq, h):
        return self.lib.orc_poly6(r_sq, h)

    def spiky(self, r, h):
        return self.lib.orc_spiky(r, h)

    def cubic_spline(self, r, h):
        return self.lib.orc_cubic_spline(r, h)

    def spiky_grad(self, r, h):
        out = np.zeros(3, np.float32)
        self.lib.orc_spiky_grad(_f32(r, (3,)), h, out)
        return out

    # -- grid --
    def cell_coords(self, pts, cell):
        pts = _f32(pts, (-1, 3))
        out = np.zeros((len(pts), 3), np.int32)
        self.lib.orc_cell_coords(pts, len(pts), cell, out)
        return out

    def grid_query(self, pts, cell, q):
        pts = _f32(pts, (-1, 3))
        probe = np.zeros(1, np.int32)
        m = self.lib.orc_grid_query(pts, len(pts), cell, _f32(q, (3,)), probe, 0)
        out = np.zeros(max(m, 1), np.int32)
        self.lib.orc_grid_query(pts, len(pts), cell, _f32(q, (3,)), out, m)
        return out[:m].copy()

    def hash_collisions(self, pts, cell):
        pts = _f32(pts, (-1, 3))
        return self.lib.orc_hash_collisions(pts, len(pts), cell)

    def neighbor_sets(self, xs, h):
        xs = _f32(xs, (-1, 3))
        n = len(xs)
        off = np.zeros(n + 1, np.int64)
        tot = self.lib.orc_neighbor_sets(xs, n, h, off.ctypes.data, None, 0)
        idx = np.zeros(max(tot, 1), np.int32)
        tot = self.lib.orc_neighbor_sets(xs, n, h, off.ctypes.data, idx.ctypes.data, tot)
        return off, idx[:tot]

    def predict(self, x, v, dt, g):
        x = _f32(x, (-1, 3))
        v = _f32(v, (-1, 3))
        xs = np.zeros_like(x)
        vo = np.zeros_like(v)
        self.lib.orc_predict(len(x), x, v, dt, _f32(g, (3,)), xs, vo)
        return xs, vo

    # -- PBF step --
    def set_threads(self, t: int) -> int:
        """Host threads of the step's per-particle loops (results do not
        depend on it); returns the count used."""
        t = max(1, min(int(t), self.lib.orc_max_threads()))
        self.lib.orc_set_threads(t)
        return t

    def steps(self, settings: Settings, x, v, rho, lam, dt, g, mass, nsteps=1):
        x = _f32(x, (-1, 3)).copy()
        v = _f32(v, (-1, 3)).copy()
        rho = _f32(rho).copy()
        lam = _f32(lam).copy()
        g = _f32(g, (3,))
        for _ in range(nsteps):
            rc = self.lib.orc_pbf_step(C.byref(settings), len(x), x, v, rho, lam, dt, g, mass)
            if rc != 0:
                raise MemoryError("oracle step failed")
        return x, v, rho, lam

    # -- boundary --
    def boundary_world_positions(self, local, body, body_pos, body_quat):
        local = _f32(local, (-1, 3))
        body = np.ascontiguousarray(body, dtype=np.int32)
        bp = _f32(body_pos, (-1, 3))
        bq = _f32(body_quat, (-1, 4))
        out = np.zeros_like(local)
        self.lib.orc_boundary_world_positions(len(local), local, body, len(bp), bp, bq, out)
        return out

    def boundary_volumes(self, world, h):
        world = _f32(world, (-1, 3))
        psi = np.zeros(len(world), np.float32)
        if self.lib.orc_boundary_volumes(len(world), world, h, psi) != 0:
            raise MemoryError
        return psi

    def boundary_density(self, x, rho, bpos, psi, h, rho0):
        x = _f32(x, (-1, 3))
        rho = _f32(rho).copy()
        bpos = _f32(bpos, (-1, 3))
        if self.lib.orc_boundary_density(len(x), x, rho, len(bpos), bpos, _f32(psi), h, rho0):
            raise MemoryError
        return rho

    def coupling_forces(self, x, rho, mass, bpos, body, psi, body_dynamic, body_pos, h, rho0):
        x = _f32(x, (-1, 3))
        bpos = _f32(bpos, (-1, 3))
        body_pos = _f32(body_pos, (-1, 3))
        nbodies = len(body_pos)
        f = np.zeros((nbodies, 3), np.float32)
        t = np.zeros((nbodies, 3), np.float32)
        rc = self.lib.orc_coupling_forces(
            len(x), x, _f32(rho), mass, len(bpos), bpos, np.ascontiguousarray(body, np.int32),
            _f32(psi), nbodies, np.ascontiguousarray(body_dynamic, np.int32), body_pos, h, rho0,
            f, t)
        if rc:
            raise MemoryError
        return f, t

    def _sampled(self, fn, *args):
        m = fn(*args, None, 0)
        out = np.zeros((max(m, 1), 3), np.float32)
        fn(*args, out.ctypes.data, m)
        return out[:m]

    def sample_box(self, half, lt_pos=(0, 0, 0), lt_quat=(1, 0, 0, 0), spacing=0.1):
        return self._sampled(self.lib.orc_sample_box, _f32(half, (3,)), _f32(lt_pos, (3,)),
                             _f32(lt_quat, (4,)), spacing)

    def sample_sphere(self, radius, lt_pos=(0, 0, 0), lt_quat=(1, 0, 0, 0), spacing=0.1):
        return self._sampled(self.lib.orc_sample_sphere, radius, _f32(lt_pos, (3,)),
                             _f32(lt_quat, (4,)), spacing)

    def sample_plane(self, normal, offset, spacing, extent):
        return self._sampled(self.lib.orc_sample_plane, _f32(normal, (3,)), offset, spacing,
                             extent)

    def generate_block(self, lower, upper, spacing):
        return self._sampled(self.lib.orc_generate_block, _f32(lower, (3,)), _f32(upper, (3,)),
                             spacing)


class Ref:
    """The reference's own PBF sources (oracle/_ref), where they could be built."""

    def __init__(self, path: str | None = None):
        path = path or build_oracle.build_ref()
        if path is None or not os.path.exists(path):
            raise FileNotFoundError("reference build unavailable (reference tree absent)")
        L = self.lib = C.CDLL(path)
        L.ref_pbf_steps.argtypes = [C.POINTER(Settings), C.c_int, _f32p, _f32p, _f32p, _f32p,
                                    C.c_float, _f32p, C.c_float, C.c_int]
        L.ref_pbf_steps.restype = C.c_int
        L.ref_grid_query.argtypes = [_f32p, C.c_int, C.c_float, _f32p, C.c_float, _i32p, C.c_int]
        L.ref_grid_query.restype = C.c_int
        L.ref_query_all_pairs.argtypes = [_f32p, C.c_int, C.c_float, C.c_float, C.c_void_p,
                                          C.c_int]
        L.ref_query_all_pairs.restype = C.c_int
        L.ref_generate_block.argtypes = [_f32p, _f32p, C.c_float, C.c_void_p, C.c_int]
        L.ref_generate_block.restype = C.c_int
        L.ref_poly6.argtypes = [C.c_float, C.c_float]
        L.ref_poly6.restype = C.c_float
        L.ref_spiky.argtypes = [C.c_float, C.c_float]
        L.ref_spiky.restype = C.c_float
        L.ref_cubic_spline.argtypes = [C.c_float, C.c_float]
        L.ref_cubic_spline.restype = C.c_float
        L.ref_spiky_grad.argtypes = [_f32p, C.c_float, _f32p]
        L.ref_default_settings.argtypes = [C.POINTER(Settings)]
        L.ref_boundary_volumes.argtypes = [C.c_int, _f32p, C.c_float, _f32p]
        L.ref_boundary_volumes.restype = C.c_int
        L.ref_boundary_world_positions.argtypes = [C.c_int, _f32p, _i32p, C.c_int, _f32p, _f32p,
                                                   _f32p]
        L.ref_fluid_world_run.argtypes = [C.POINTER(Settings), _f32p, _f32p, C.c_float, C.c_int,
                                          _i32p, _f32p, _f32p, _f32p, _f32p, C.c_int, C.c_float,
                                          C.c_float, C.c_float, C.c_int, C.c_int, _f32p, _f32p,
                                          _f32p, _f32p, _f32p, _f32p, _f32p, _f32p]
        L.ref_fluid_world_run.restype = C.c_int
        L.ref_fluid_world_run_ex.argtypes = [
            C.POINTER(Settings), _f32p, _f32p, C.c_float, C.c_int, _i32p, _f32p, _f32p, _f32p,
            _f32p, C.c_int, _f32p, C.c_float, C.c_float, _f32p, C.c_float, C.c_int, C.c_int,
            _f32p, _f32p, _f32p, _f32p, _f32p, _f32p, _f32p, _f32p]
        L.ref_fluid_world_run_ex.restype = C.c_int
        L.ref_world_run.argtypes = [C.c_int, _i32p, _f32p, _f32p, _f32p, _f32p, _f32p, _f32p,
                                    C.c_void_p, C.c_void_p, C.c_float, C.c_int, _f32p, _f32p,
                                    _f32p, _f32p]
        L.ref_world_run.restype = C.c_int
        L.ref_sample_box.argtypes = [_f32p, _f32p, _f32p, C.c_float, C.c_void_p, C.c_int]
        L.ref_sample_sphere.argtypes = [C.c_float, _f32p, _f32p, C.c_float, C.c_void_p, C.c_int]
        L.ref_sample_plane.argtypes = [_f32p, C.c_float, C.c_float, C.c_float, C.c_void_p, C.c_int]
        L.ref_collide.argtypes = [_f32p, _f32p, _f32p, _f32p, _f32p, C.c_int, _i32p]
        L.ref_collide.restype = C.c_int
        L.ref_sap.argtypes = [C.c_int, _f32p, _i32p, _i32p, C.c_int]
        L.ref_sap.restype = C.c_int
        L.ref_rigid_world_run.argtypes = [C.c_int, _f32p, C.c_int, _f32p, _f32p, _f32p, _f32p,
                                          _f32p, C.c_float, C.c_int, _f32p, _f32p, _f32p, _f32p,
                                          _i32p, _i32p]
        L.ref_rigid_world_run.restype = C.c_int

    # Shapes are packed as 19 floats (ref_harness.cpp, shape_from); contacts come back as
    # rows of 11: position (3), normal (3), penetration, body_a, body_b,
    # friction, restitution.
    def collide(self, shape_a, pose_a, shape_b, pose_b):
        """collide_shapes on two packed shapes at poses (x, y, z, qw, qx, qy, qz);
        returns (hit, contacts[n, 11])."""
        out = np.zeros((16, 11), np.float32)
        hit = np.zeros(1, np.int32)
        n = self.lib.ref_collide(_f32(shape_a, (19,)), _f32(pose_a, (7,)), _f32(shape_b, (19,)),
                                 _f32(pose_b, (7,)), out, 16, hit)
        return bool(hit[0]), out[:n]

    def sap(self, boxes, fixed):
        """SweepAndPrune pairs of boxes[n, 6] (min, max) with a static mask."""
        boxes = _f32(boxes, (-1, 6))
        fixed = np.ascontiguousarray(fixed, np.int32)
        cap = max(1, len(boxes) * (len(boxes) - 1) // 2)
        pairs = np.zeros((cap, 2), np.int32)
        n = self.lib.ref_sap(len(boxes), boxes, fixed, pairs, cap)
        return pairs[:n]

    def rigid_world(self, bodies, shapes, lin, ang, settings, gravity, dt, nsteps):
        """The reference World (contacts, solver, sleep) after nsteps steps.
        bodies[n, 17] = mass, inertia (9), position, rotation (w, x, y, z);
        shapes[m, 19] packed; settings = (velocity_iterations, baumgarte, slop,
        warm_starting, sleep_enabled, sleep_energy_threshold,
        sleep_time_required, sleep_ema_alpha).  Returns (pos, quat, lin_vel,
        ang_vel, contacts per step, sleeping)."""
        bodies = _f32(bodies, (-1, 17))
        shapes = _f32(shapes, (-1, 19))
        nb = len(bodies)
        out = [np.zeros((nb, 3), np.float32), np.zeros((nb, 4), np.float32),
               np.zeros((nb, 3), np.float32), np.zeros((nb, 3), np.float32),
               np.zeros(max(nsteps, 1), np.int32), np.zeros(max(nb, 1), np.int32)]
        rc = self.lib.ref_rigid_world_run(nb, bodies, len(shapes), shapes, _f32(lin, (-1, 3)),
                                          _f32(ang, (-1, 3)), _f32(settings, (8,)),
                                          _f32(gravity, (3,)), dt, nsteps, *out)
        if rc:
            raise ValueError("the reference World failed")
        out[4] = out[4][:nsteps]
        out[5] = out[5][:nb]
        return tuple(out)

    def boundary_volumes(self, world, h):
        world = _f32(world, (-1, 3))
        psi = np.zeros(len(world), np.float32)
        if self.lib.ref_boundary_volumes(len(world), world, h, psi) != 0:
            raise ValueError("compute_boundary_volumes threw")
        return psi

    def boundary_world_positions(self, local, body, body_pos, body_quat):
        local = _f32(local, (-1, 3))
        body = np.ascontiguousarray(body, dtype=np.int32)
        bp = _f32(body_pos, (-1, 3))
        bq = _f32(body_quat, (-1, 4))
        out = np.zeros_like(local)
        self.lib.ref_boundary_world_positions(len(local), local, body, len(bp), bp, bq, out)
        return out

    def fluid_world(self, settings: Settings, lower, upper, spacing, bodies, plane_y=None,
                    boundary_extent=1.0, dt=1.0 / 60.0, nsteps=1, cap=1 << 20):
        """The reference FluidWorld (fluid_world.cpp with its rigid World) after
        nsteps steps.  bodies: list of (kind, size3, mass, pos3, quat4 (w, x, y,
        z)) with kind "sphere" (size3[0] = radius) or "box" (half extents).
        Returns (x, v, rho, lam, body_pos, body_quat, body_v, body_w)."""
        nb = len(bodies)
        kind = np.array([0 if b[0] == "sphere" else 1 for b in bodies] or [0], np.int32)
        size = _f32([list(b[1]) for b in bodies] or [[0, 0, 0]], (-1, 3))
        mass = _f32([b[2] for b in bodies] or [0])
        pos = _f32([list(b[3]) for b in bodies] or [[0, 0, 0]], (-1, 3))
        quat = _f32([list(b[4]) for b in bodies] or [[1, 0, 0, 0]], (-1, 4))
        x = np.zeros((cap, 3), np.float32)
        v = np.zeros((cap, 3), np.float32)
        rho = np.zeros(cap, np.float32)
        lam = np.zeros(cap, np.float32)
        bp = np.zeros((max(nb, 1), 3), np.float32)
        bq = np.zeros((max(nb, 1), 4), np.float32)
        bv = np.zeros((max(nb, 1), 3), np.float32)
        bw = np.zeros((max(nb, 1), 3), np.float32)
        n = self.lib.ref_fluid_world_run(
            C.byref(settings), _f32(lower, (3,)), _f32(upper, (3,)), spacing, nb, kind, size,
            mass, pos, quat, 0 if plane_y is None else 1, 0.0 if plane_y is None else plane_y,
            boundary_extent, dt, nsteps, cap, x, v, rho, lam, bp, bq, bv, bw)
        if n < 0:
            raise ValueError("the reference FluidWorld failed")
        return x[:n], v[:n], rho[:n], lam[:n], bp[:nb], bq[:nb], bv[:nb], bw[:nb]

    def fluid_world_ex(self, settings: Settings, lower, upper, spacing, bodies, plane=None,
                       gravity=(0.0, -9.81, 0.0), boundary_extent=1.0, dt=1.0 / 60.0, nsteps=1,
                       cap=1 << 20):
        """As fluid_world, with plane = (normal3, offset) or None and the
        world's gravity set to `gravity`."""
        nb = len(bodies)
        kind = np.array([0 if b[0] == "sphere" else 1 for b in bodies] or [0], np.int32)
        size = _f32([list(b[1]) for b in bodies] or [[0, 0, 0]], (-1, 3))
        mass = _f32([b[2] for b in bodies] or [0])
        pos = _f32([list(b[3]) for b in bodies] or [[0, 0, 0]], (-1, 3))
        quat = _f32([list(b[4]) for b in bodies] or [[1, 0, 0, 0]], (-1, 4))
        x = np.zeros((cap, 3), np.float32)
        v = np.zeros((cap, 3), np.float32)
        rho = np.zeros(cap, np.float32)
        lam = np.zeros(cap, np.float32)
        bp = np.zeros((max(nb, 1), 3), np.float32)
        bq = np.zeros((max(nb, 1), 4), np.float32)
        bv = np.zeros((max(nb, 1), 3), np.float32)
        bw = np.zeros((max(nb, 1), 3), np.float32)
        normal = _f32(plane[0] if plane else (0.0, 1.0, 0.0), (3,))
        offset = float(plane[1]) if plane else 0.0
        n = self.lib.ref_fluid_world_run_ex(
            C.byref(settings), _f32(lower, (3,)), _f32(upper, (3,)), spacing, nb, kind, size,
            mass, pos, quat, 1 if plane else 0, normal, offset, boundary_extent,
            _f32(gravity, (3,)), dt, nsteps, cap, x, v, rho, lam, bp, bq, bv, bw)
        if n < 0:
            raise ValueError("the reference FluidWorld failed")
        return x[:n], v[:n], rho[:n], lam[:n], bp[:nb], bq[:nb], bv[:nb], bw[:nb]

    def world(self, bodies, lin, ang, dt, nsteps, force=None, torque=None):
        """The reference rigid World (no ground plane) after nsteps steps of
        free bodies (as fluid_world's bodies) from velocities lin/ang, with
        constant force/torque applied before each step.  Returns
        (pos, quat (w, x, y, z), lin_vel, ang_vel)."""
        nb = len(bodies)
        kind = np.array([0 if b[0] == "sphere" else 1 for b in bodies], np.int32)
        size = _f32([list(b[1]) for b in bodies], (-1, 3))
        mass = _f32([b[2] for b in bodies])
        pos = _f32([list(b[3]) for b in bodies], (-1, 3))
        quat = _f32([list(b[4]) for b in bodies], (-1, 4))
        f = None if force is None else _f32(force, (-1, 3))
        t = None if torque is None else _f32(torque, (-1, 3))
        out = [np.zeros((nb, 3), np.float32), np.zeros((nb, 4), np.float32),
               np.zeros((nb, 3), np.float32), np.zeros((nb, 3), np.float32)]
        rc = self.lib.ref_world_run(nb, kind, size, mass, pos, quat, _f32(lin, (-1, 3)),
                                    _f32(ang, (-1, 3)),
                                    None if f is None else f.ctypes.data,
                                    None if t is None else t.ctypes.data, dt, nsteps, *out)
        if rc:
            raise ValueError("the reference World failed")
        return tuple(out)

    def _sampled(self, fn, *args):
        m = fn(*args, None, 0)
        out = np.zeros((max(m, 1), 3), np.float32)
        fn(*args, out.ctypes.data, m)
        return out[:m]

    def sample_box(self, half, lt_pos=(0, 0, 0), lt_quat=(1, 0, 0, 0), spacing=0.1):
        return self._sampled(self.lib.ref_sample_box, _f32(half, (3,)), _f32(lt_pos, (3,)),
                             _f32(lt_quat, (4,)), spacing)

    def sample_sphere(self, radius, lt_pos=(0, 0, 0), lt_quat=(1, 0, 0, 0), spacing=0.1):
        return self._sampled(self.lib.ref_sample_sphere, radius, _f32(lt_pos, (3,)),
                             _f32(lt_quat, (4,)), spacing)

    def sample_plane(self, normal, offset, spacing, extent):
        return self._sampled(self.lib.ref_sample_plane, _f32(normal, (3,)), offset, spacing,
                             extent)

    def default_settings(self) -> Settings:
        s = Settings()
        self.lib.ref_default_settings(C.byref(s))
        return s

    def steps(self, settings: Settings, x, v, rho, lam, dt, g, mass, nsteps=1):
        x = _f32(x, (-1, 3)).copy()
        v = _f32(v, (-1, 3)).copy()
        rho = _f32(rho).copy()
        lam = _f32(lam).copy()
        self.lib.ref_pbf_steps(C.byref(settings), len(x), x, v, rho, lam, dt, _f32(g, (3,)),
                               mass, nsteps)
        return x, v, rho, lam

    def grid_query(self, pts, cell, q, radius=0.0):
        pts = _f32(pts, (-1, 3))
        out = np.zeros(max(len(pts), 1), np.int32)
        m = self.lib.ref_grid_query(pts, len(pts), cell, _f32(q, (3,)), radius, out, len(out))
        return out[:m].copy()

    def query_all_pairs(self, pts, cell, radius):
        pts = _f32(pts, (-1, 3))
        m = self.lib.ref_query_all_pairs(pts, len(pts), cell, radius, None, 0)
        out = np.zeros((max(m, 1), 2), np.int32)
        self.lib.ref_query_all_pairs(pts, len(pts), cell, radius, out.ctypes.data, m)
        return out[:m]

    def generate_block(self, lower, upper, spacing):
        m = self.lib.ref_generate_block(_f32(lower, (3,)), _f32(upper, (3,)), spacing, None, 0)
        out = np.zeros((max(m, 1), 3), np.float32)
        self.lib.ref_generate_block(_f32(lower, (3,)), _f32(upper, (3,)), spacing,
                                    out.ctypes.data, m)
        return out[:m]

    def poly6(self, r_sq, h):
        return self.lib.ref_poly6(r_sq, h)

    def spiky(self, r, h):
        return self.lib.ref_spiky(r, h)

    def cubic_spline(self, r, h):
        return self.lib.ref_cubic_spline(r, h)

    def spiky_grad(self, r, h):
        out = np.zeros(3, np.float32)
        self.lib.ref_spiky_grad(_f32(r, (3,)), h, out)
        return out
