"""Seeded synthetic dam-break workloads of the PBF step.

All inputs are synthetic (no dataset is involved): a cubic lattice, x
fastest then y then z like generate_fluid_block (src/fluid/particle_state.cpp:
31-58), plus uniform jitter from ``numpy.random.default_rng(seed)``; float32
throughout so every consumer sees identical bytes.

* ``dam_break_8k``  - 20^3 particles, r = 0.025 m, box [0,1]^3, h = 4r,
  4 iterations, dt = 1/120 s (the reference CPU-runnable case).
* ``dam_break_1m``  - 100^3 particles, r = 0.01 m, box [0,4]x[0,2]x[0,2],
  h = 4r, 4 iterations, dt = 1/240 s (the single-GPU throughput case).

Common parameters: rest density 1000, mass rho0 r^3, gravity -9.81 z,
s_corr k = 0.1, n = 4, dq = 0.2 h, XSPH c = 0.01, vorticity eps = 1e-4,
domain clamp on with particle_radius = r/2, block lower corner at r/2 per
axis so that the initial state is inside the clamp.
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np


@dataclass
class Workload:
    name: str
    x: np.ndarray            # (n, 3) float32
    v: np.ndarray            # (n, 3) float32
    settings: dict           # PBFSettings fields (+ extensions)
    dt: float
    gravity: np.ndarray      # (3,) float32
    mass: float
    steps: int
    meta: dict = field(default_factory=dict)

    @property
    def n(self) -> int:
        return len(self.x)


def lattice(counts, spacing, lower) -> np.ndarray:
    """generate_fluid_block order: x fastest; coordinates lower + i * spacing in float32."""
    nx, ny, nz = counts
    sp = np.float32(spacing)
    lo = np.asarray(lower, np.float32)
    iz, iy, ix = np.meshgrid(np.arange(nz, dtype=np.float32), np.arange(ny, dtype=np.float32),
                             np.arange(nx, dtype=np.float32), indexing="ij")
    pts = np.stack([lo[0] + ix.ravel() * sp, lo[1] + iy.ravel() * sp, lo[2] + iz.ravel() * sp],
                   axis=1)
    return np.ascontiguousarray(pts.astype(np.float32))


def dam_break(counts, r, box_upper, h_factor=4.0, iterations=4, dt=1.0 / 120.0, jitter=1e-4,
              seed=0, vorticity=1e-4, steps=120, name="dam_break") -> Workload:
    rng = np.random.default_rng(seed)
    lower = np.full(3, r / 2, np.float32)
    x = lattice(counts, r, lower)
    x = (x + rng.uniform(-jitter, jitter, x.shape)).astype(np.float32)
    h = np.float32(h_factor * r)
    settings = dict(
        rest_density=1000.0, kernel_radius=float(h), particle_radius=float(np.float32(r / 2)),
        solver_iterations=iterations, epsilon=100.0, xsph_viscosity=0.01,
        vorticity_epsilon=vorticity, corr_delta_q=0.2, corr_k=0.1, corr_n=4,
        use_domain_bounds=1, domain_lower=(0.0, 0.0, 0.0), domain_upper=tuple(box_upper),
    )
    mass = float(np.float32(1000.0) * np.float32(r) ** 3)
    return Workload(name=name, x=x, v=np.zeros_like(x), settings=settings, dt=float(np.float32(dt)),
                    gravity=np.array([0.0, 0.0, -9.81], np.float32), mass=mass, steps=steps,
                    meta=dict(r=r, counts=tuple(counts), box=tuple(box_upper), seed=seed,
                              jitter=jitter))


def dam_break_8k(vorticity=1e-4) -> Workload:
    return dam_break((20, 20, 20), 0.025, (1.0, 1.0, 1.0), dt=1.0 / 120.0, jitter=1e-4, seed=0,
                     vorticity=vorticity, steps=120, name="dam_break_8k")


def dam_break_1m(vorticity=1e-4) -> Workload:
    return dam_break((100, 100, 100), 0.01, (4.0, 2.0, 2.0), dt=1.0 / 240.0, jitter=1e-5, seed=1,
                     vorticity=vorticity, steps=200, name="dam_break_1m")


def scaled_dam_break(counts, vorticity=1e-4, seed=1) -> Workload:
    """A block of `counts` at the 1M case's density and box (same per-particle work)."""
    return dam_break(counts, 0.01, (4.0, 2.0, 2.0), dt=1.0 / 240.0, jitter=1e-5, seed=seed,
                     vorticity=vorticity, steps=200, name=f"dam_break_{np.prod(counts)}")


def batched_scenes(nscenes=1024, seed=3, n_lo=2000, n_hi=64000, r=0.02, dt=1.0 / 120.0,
                   steps=100, vorticity=1e-4) -> list[Workload]:
    """Independent dam-break scenes of uneven size for batched stepping.

    Per scene, from ``default_rng(seed)``: a target count N = round(exp(U(ln n_lo,
    ln n_hi))), a block aspect a ~ U(1, 3) as a:1:1 (ny = nz = round((N/a)^(1/3)),
    nx = round(N / (ny nz)), so the actual count follows the lattice), a box of
    U(1.5, 3) x the block extent per axis, solver iterations ~ U{2..6}, a jitter
    seed; r = 0.02 m, h = 4r, the other parameters as ``dam_break``.
    """
    rng = np.random.default_rng(seed)
    out = []
    for k in range(nscenes):
        target = int(round(float(np.exp(rng.uniform(np.log(n_lo), np.log(n_hi))))))
        aspect = float(rng.uniform(1.0, 3.0))
        ny = max(1, int(round((target / aspect) ** (1.0 / 3.0))))
        nx = max(1, int(round(target / (ny * ny))))
        counts = (nx, ny, ny)
        ext = np.array(counts, np.float64) * r
        box = tuple(float(np.float32(e * f + r)) for e, f in zip(ext, rng.uniform(1.5, 3.0, 3)))
        iters = int(rng.integers(2, 7))
        w = dam_break(counts, r, box, iterations=iters, dt=dt, jitter=1e-4,
                      seed=int(rng.integers(0, 2**31)), vorticity=vorticity, steps=steps,
                      name=f"scene_{k}")
        out.append(w)
    return out


def served_scenes(nclients=256, seed=4, n_lo=1000, n_hi=200_000, r=0.02, dt=1.0 / 240.0,
                  vorticity=1e-4) -> list[Workload]:
    """One scene per client of a serving run, from ``default_rng(seed)``: a
    target count N = round(exp(U(ln n_lo, ln n_hi))); half dam breaks (a 1:1:2
    block in the corner of a box 3x its footprint and 1.5x its height), half
    pools (a 2:2:1 block covering the floor of a box 2x its height), with 0-4
    rigid spheres (radius 5r, density U(300, 1500)) above the fluid in
    ``meta["spheres"]`` as (center, radius, density).  h = 4r,
    4 iterations, XSPH 0.01, vorticity 1e-4, and the s_corr defaults of
    PBFSettings (k = 0.001, dq = 0.3 h, n = 4): served scenes run hundreds of
    consecutive steps, and with k = 0.1 the fluid collapses into a few
    overfull cells within ~100 steps."""
    rng = np.random.default_rng(seed)
    out = []
    for k in range(nclients):
        target = int(round(float(np.exp(rng.uniform(np.log(n_lo), np.log(n_hi))))))
        if rng.uniform() < 0.5:
            a = max(1, int(round((target / 2.0) ** (1.0 / 3.0))))
            counts = (a, a, max(1, int(round(target / (a * a)))))
            ext = np.array(counts, np.float64) * r
            box = (3.0 * ext[0] + r, 3.0 * ext[1] + r, 1.5 * ext[2] + r)
            kind = "dam"
        else:
            c = max(1, int(round((target / 4.0) ** (1.0 / 3.0))))
            a = max(1, int(round((target / c) ** 0.5)))
            counts = (a, a, c)
            ext = np.array(counts, np.float64) * r
            box = (ext[0] + r, ext[1] + r, 2.0 * ext[2] + r)
            kind = "pool"
        box = tuple(float(np.float32(b)) for b in box)
        w = dam_break(counts, r, box, iterations=4, dt=dt, jitter=1e-4,
                      seed=int(rng.integers(0, 2**31)), vorticity=vorticity, steps=16,
                      name=f"client_{k}_{kind}")
        w.settings.update(corr_k=0.001, corr_delta_q=0.3)
        # 0-4 Akinci spheres (radius 5r, density U(300, 1500)) above the fluid,
        # spread over the box footprint: (center, radius, density) each.
        spheres = []
        rad = 5.0 * r
        top = float(ext[2] + r / 2)
        for j in range(int(rng.integers(0, 5))):
            cx = float(rng.uniform(rad, box[0] - rad)) if box[0] > 2 * rad else box[0] / 2
            cy = float(rng.uniform(rad, box[1] - rad)) if box[1] > 2 * rad else box[1] / 2
            cz = min(top + 2.0 * rad * (1 + j % 2), box[2] - rad)
            spheres.append(((cx, cy, max(cz, rad)), rad, float(rng.uniform(300.0, 1500.0))))
        w.meta["spheres"] = spheres
        out.append(w)
    return out


def coupled_pool(seed=2, scorr="default") -> dict:
    """The two-way coupled pool: a 50 x 50 x 100 lattice (250,000 particles) at
    r = 0.015 m centred on the floor of a 2 x 2 x 2 m box, 4 boxes (edge 0.2 m)
    and 4 spheres (radius 0.12 m) of density U(300, 1500) from ``default_rng(
    seed)``, dropped from 0.5-1.0 m above the pool at x-y positions in 8 of the
    9 cells (0.25 m) of a 3 x 3 grid over the pool footprint (jittered by up to
    5 mm, so no two bodies overlap), a floor plane (normal +z, offset 0),
    Akinci boundary particles at spacing r over a boundary extent of 1 m; h =
    4r, 4 iterations, dt = 1/240 s, XSPH 0.01, vorticity 1e-4, gravity -9.81 z,
    domain clamp on [0, 2]^3 with particle_radius = r/2.  s_corr: PBFSettings'
    own (k = 0.001, dq = 0.3 h) with scorr="default" (the pool's configuration
    does not set it), or the dam break's k = 0.1, dq = 0.2 h with "config0".

    Returns a dict: block (lower, upper, spacing), bodies as (kind, size3,
    mass, pos3, quat4 (w, x, y, z)) with kind "box" (half extents) or "sphere"
    (size3[0] = radius), plane (normal3, offset), boundary_extent, settings
    (PBFSettings fields), gravity, dt.  Masses and positions are float32."""
    rng = np.random.default_rng(seed)
    r = 0.015
    counts = np.array([50, 50, 100])
    lower = np.array([(2.0 - 50 * r) / 2, (2.0 - 50 * r) / 2, r / 2], np.float32)
    upper = lower + (counts - 0.5).astype(np.float32) * np.float32(r)
    cells = rng.permutation(9)[:8]
    bodies = []
    for k in range(8):
        dens = float(rng.uniform(300.0, 1500.0))
        cx, cy = divmod(int(cells[k]), 3)
        xy = lower[:2] + (np.array([cx, cy]) + 0.5) * 0.25 + rng.uniform(-0.005, 0.005, 2)
        z = float(upper[2] + rng.uniform(0.5, 1.0))
        pos = tuple(float(t) for t in np.array([xy[0], xy[1], z], np.float32))
        if k < 4:
            bodies.append(("box", (0.1, 0.1, 0.1), float(np.float32(dens * 0.2 ** 3)), pos,
                           (1.0, 0.0, 0.0, 0.0)))
        else:
            rad = 0.12
            m = float(np.float32(dens * 4.0 / 3.0 * np.pi * rad ** 3))
            bodies.append(("sphere", (rad, 0.0, 0.0), m, pos, (1.0, 0.0, 0.0, 0.0)))
    settings = dict(
        rest_density=1000.0, kernel_radius=float(np.float32(4 * r)),
        particle_radius=float(np.float32(r / 2)), solver_iterations=4, epsilon=100.0,
        xsph_viscosity=0.01, vorticity_epsilon=1e-4, corr_delta_q=0.3, corr_k=0.001, corr_n=4,
        use_domain_bounds=1, domain_lower=(0.0, 0.0, 0.0), domain_upper=(2.0, 2.0, 2.0))
    if scorr == "config0":
        settings.update(corr_k=0.1, corr_delta_q=0.2)
    return dict(block=(tuple(float(t) for t in lower), tuple(float(t) for t in upper), r),
                bodies=bodies, plane=((0.0, 0.0, 1.0), 0.0), boundary_extent=1.0,
                settings=settings, gravity=np.array([0.0, 0.0, -9.81], np.float32),
                dt=float(np.float32(1.0 / 240.0)), r=r)


def fluid_world_of(spec):
    """The package's FluidWorld of a coupled_pool spec (the native module)."""
    import novaphy_gb300 as nv

    mb = nv.ModelBuilder()
    normal, offset = spec["plane"]
    mb.add_shape(nv.CollisionShape.make_plane(list(normal), offset))
    for kind, size, mass, pos, quat in spec["bodies"]:
        t = nv.Transform.from_translation(list(pos))
        if kind == "box":
            bi = mb.add_body(nv.RigidBody.from_box(mass, list(size)), t)
            mb.add_shape(nv.CollisionShape.make_box(list(size), bi))
        else:
            bi = mb.add_body(nv.RigidBody.from_sphere(mass, size[0]), t)
            mb.add_shape(nv.CollisionShape.make_sphere(size[0], bi))
    lower, upper, spacing = spec["block"]
    blk = nv.FluidBlockDef()
    blk.lower = list(lower)
    blk.upper = list(upper)
    blk.particle_spacing = spacing
    st = nv.PBFSettings()
    for k, v in spec["settings"].items():
        if k == "use_domain_bounds":
            v = bool(v)
        setattr(st, k, list(v) if isinstance(v, tuple) else v)
    world = nv.FluidWorld(mb.build(), [blk], nv.SolverSettings(), st, spec["boundary_extent"])
    world.set_gravity([float(g) for g in spec["gravity"]])
    return world
