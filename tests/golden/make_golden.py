"""Generates the golden fixtures in this directory from the reference itself.

The reference's own PBF sources (src/fluid/*.cpp) are compiled by
oracle/build_oracle.py into oracle/_ref and run here on seeded synthetic
inputs; their outputs become the fixtures.  The script also checks that the
oracle restatement (oracle/pbf_oracle.c) reproduces every fixture bit for
bit, so the fixtures pin the restatement.

Run from the repository root:  python tests/golden/make_golden.py
(fluid_world.npz alone: python tests/golden/make_golden.py fluid_world; the
digests at the benchmarked sizes alone: ... make_golden.py large)
"""
from __future__ import annotations

import hashlib
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from novaphy_gb300 import workloads  # noqa: E402
from oracle.oracle import Port, Ref, Settings  # noqa: E402


def digest(*arrays) -> str:
    h = hashlib.sha256()
    for a in arrays:
        h.update(np.ascontiguousarray(a, np.float32).tobytes())
    return h.hexdigest()


def small_block(seed=0):
    """10^3 lattice at r = 0.025 in [0,1]^3, dam-break parameters, no vorticity."""
    return workloads.dam_break((10, 10, 10), 0.025, (1.0, 1.0, 1.0), dt=1.0 / 120.0, jitter=1e-4,
                               seed=seed, vorticity=0.0, name="block_1k")


def default_scene():
    """The reference tests' PBF scene: 0.3 m block at spacing 0.025, h = 0.1,
    PBFSettings defaults otherwise (no domain clamp), gravity -9.81 y,
    dt = 1/60 (tests/python/test_pbf.py:28-49)."""
    x = workloads.lattice((13, 13, 13), 0.025, (0.0, 0.0, 0.0))
    s = Settings.make(kernel_radius=0.1, solver_iterations=4, epsilon=100.0)
    return x, s, np.float32(1.0 / 60.0), np.array([0, -9.81, 0], np.float32), \
        np.float32(1000.0) * np.float32(0.025) ** 3


def main():
    P, R = Port(), Ref()
    out = {}

    # --- SPH kernels on a sweep of radii, two kernel radii.
    ker = {}
    for h in (0.1, 0.04):
        hf = np.float32(h)
        r = np.linspace(0.0, 1.2 * h, 97, dtype=np.float32)
        ker[f"r_{h}"] = r
        ker[f"poly6_{h}"] = np.array([R.poly6(t * t, hf) for t in r], np.float32)
        ker[f"spiky_{h}"] = np.array([R.spiky(t, hf) for t in r], np.float32)
        ker[f"cubic_{h}"] = np.array([R.cubic_spline(t, hf) for t in r], np.float32)
        dirs = np.random.default_rng(7).normal(size=(97, 3)).astype(np.float32)
        dirs /= np.linalg.norm(dirs, axis=1, keepdims=True)
        vec = (dirs * r[:, None]).astype(np.float32)
        ker[f"gradvec_{h}"] = vec
        ker[f"spiky_grad_{h}"] = np.stack([R.spiky_grad(t, hf) for t in vec]).astype(np.float32)
        for k in ("poly6", "spiky", "cubic"):
            fn = {"poly6": lambda t: P.poly6(t * t, hf), "spiky": lambda t: P.spiky(t, hf),
                  "cubic": lambda t: P.cubic_spline(t, hf)}[k]
            mine = np.array([fn(t) for t in r], np.float32)
            assert np.array_equal(mine, ker[f"{k}_{h}"]), k
        mine = np.stack([P.spiky_grad(t, hf) for t in vec])
        assert np.array_equal(mine, ker[f"spiky_grad_{h}"])
    np.savez_compressed(os.path.join(HERE, "kernels.npz"), **ker)

    # --- Grid candidate lists on a seeded cloud (query order included).
    rng = np.random.default_rng(42)
    cloud = rng.uniform(-0.3, 1.0, size=(600, 3)).astype(np.float32)
    queries = rng.uniform(-0.3, 1.0, size=(16, 3)).astype(np.float32)
    lists = [R.grid_query(cloud, 0.1, q) for q in queries]
    for q, ref_list in zip(queries, lists):
        assert np.array_equal(P.grid_query(cloud, 0.1, q), ref_list)
    offs = np.cumsum([0] + [len(t) for t in lists]).astype(np.int64)
    np.savez_compressed(os.path.join(HERE, "grid.npz"), cloud=cloud, queries=queries,
                        offsets=offs, cand=np.concatenate(lists).astype(np.int32))

    # --- One and five steps of a 1000-particle dam-break block.
    w = small_block()
    s = Settings.make(**w.settings)
    z = np.zeros(w.n, np.float32)
    res = {}
    for k in (1, 5):
        got = R.steps(s, w.x, w.v, z, z, w.dt, w.gravity, w.mass, k)
        mine = P.steps(s, w.x, w.v, z, z, w.dt, w.gravity, w.mass, k)
        for a, b in zip(got, mine):
            assert np.array_equal(a, b), "restatement differs from the reference build"
        for name, a in zip(("x", "v", "rho", "lam"), got):
            res[f"{name}{k}"] = a
    np.savez_compressed(os.path.join(HERE, "block_1k.npz"), x0=w.x, v0=w.v, **res)

    # --- The reference tests' default-settings scene, one step.
    x, s2, dt, g, m = default_scene()
    z = np.zeros(len(x), np.float32)
    got = R.steps(s2, x, np.zeros_like(x), z, z, dt, g, m, 1)
    mine = P.steps(s2, x, np.zeros_like(x), z, z, dt, g, m, 1)
    for a, b in zip(got, mine):
        assert np.array_equal(a, b)
    np.savez_compressed(os.path.join(HERE, "default_scene.npz"), x0=x, x1=got[0], v1=got[1],
                        rho1=got[2], lam1=got[3])

    # --- Digests of the 8,000-particle dam break after 1 and 10 steps.
    w8 = workloads.dam_break_8k(vorticity=0.0)
    s8 = Settings.make(**w8.settings)
    z = np.zeros(w8.n, np.float32)
    for k in (1, 10):
        got = R.steps(s8, w8.x, w8.v, z, z, w8.dt, w8.gravity, w8.mass, k)
        mine = P.steps(s8, w8.x, w8.v, z, z, w8.dt, w8.gravity, w8.mass, k)
        for a, b in zip(got, mine):
            assert np.array_equal(a, b)
        out[f"dam_break_8k_steps{k}"] = digest(*got)
    out["dam_break_8k_input"] = digest(w8.x)
    with open(os.path.join(HERE, "digests.json"), "w") as f:
        json.dump(out, f, indent=1, sort_keys=True)
    print("fixtures written", out)


# The coupled scene of fluid_world.npz: a fluid block over a ground plane, a
# sphere and a rotated box in opposite corners, apart from each other and from
# the plane through these steps (at least 0.2 m between centres, against 0.15
# for a contact), so that the reference's contact solver stays idle; h = 0.2,
# 2 iterations, dt = 1/60, 5 steps.
FLUID_WORLD = dict(
    lower=[0.0, 0.05, 0.0], upper=[0.3, 0.4, 0.3], spacing=0.05, plane_y=0.0,
    boundary_extent=0.5, steps=5,
    bodies=[("sphere", (0.08, 0.0, 0.0), 0.5, (0.06, 0.25, 0.06), (1.0, 0.0, 0.0, 0.0)),
            ("box", (0.04, 0.04, 0.04), 0.8, (0.26, 0.33, 0.26),
             (0.96592583, 0.0, 0.25881904, 0.0))],
)


def fluid_world_fixture():
    """FluidWorld.step of the reference (fluid_world.cpp with its rigid
    World, built from its sources) on the coupled scene, 5 steps."""
    R = Ref()
    c = FLUID_WORLD
    s = Settings.make(kernel_radius=0.2, solver_iterations=2)
    dt = float(np.float32(1 / 60))
    x, v, rho, lam, bp, bq, bv, bw = R.fluid_world(
        s, c["lower"], c["upper"], c["spacing"], c["bodies"], plane_y=c["plane_y"],
        boundary_extent=c["boundary_extent"], dt=dt, nsteps=c["steps"])
    np.savez_compressed(os.path.join(HERE, "fluid_world.npz"), x=x, v=v, rho=rho, lam=lam,
                        body_pos=bp, body_quat=bq, body_v=bv, body_w=bw)
    print("fluid_world.npz written:", len(x), "particles")


# Bodies resting on the ground under a falling fluid block: a sphere pressed
# into the plane, a box standing on an edge (two corner contacts), and from
# the sixth step on the fluid pushes them into each other (box-sphere), so
# the reference's contact solver acts every step.  The scene is stored in the
# fixture with the results.
FLUID_WORLD_CONTACTS = dict(
    lower=[0.0, 0.15, 0.0], upper=[0.3, 0.4, 0.3], spacing=0.05, plane_y=0.0,
    boundary_extent=0.5, steps=8,
    bodies=[("sphere", (0.08, 0.0, 0.0), 0.5, (0.1, 0.075, 0.1), (1.0, 0.0, 0.0, 0.0)),
            ("box", (0.04, 0.04, 0.04), 0.8, (0.22, 0.05, 0.2),
             (0.9238795, 0.0, 0.0, 0.3826834))],
)


def fluid_world_contacts_fixture():
    R = Ref()
    c = FLUID_WORLD_CONTACTS
    s = Settings.make(kernel_radius=0.2, solver_iterations=2)
    dt = float(np.float32(1 / 60))
    x, v, rho, lam, bp, bq, bv, bw = R.fluid_world(
        s, c["lower"], c["upper"], c["spacing"], c["bodies"], plane_y=c["plane_y"],
        boundary_extent=c["boundary_extent"], dt=dt, nsteps=c["steps"])
    b = c["bodies"]
    np.savez_compressed(
        os.path.join(HERE, "fluid_world_contacts.npz"), x=x, v=v, rho=rho, lam=lam,
        body_pos=bp, body_quat=bq, body_v=bv, body_w=bw,
        scene_kind=np.array([0 if k[0] == "sphere" else 1 for k in b], np.int32),
        scene_size=np.array([k[1] for k in b], np.float32),
        scene_mass=np.array([k[2] for k in b], np.float32),
        scene_pos=np.array([k[3] for k in b], np.float32),
        scene_quat=np.array([k[4] for k in b], np.float32),
        scene_block=np.array([c["lower"], c["upper"]], np.float32),
        scene_scalars=np.array([c["spacing"], c["plane_y"], c["boundary_extent"], c["steps"], dt],
                               np.float32))
    print("fluid_world_contacts.npz written:", len(x), "particles")


def field_digests(x, v, rho, lam) -> dict:
    return {"x": digest(x), "v": digest(v), "rho": digest(rho), "lam": digest(lam)}


# The 32 scenes of the batched workload that the large digests cover: every
# 32nd of the 1,024.
BATCH_SUBSET = slice(0, 1024, 32)


def large_digests():
    """Digests at the benchmarked sizes.  The reference has no vorticity
    confinement, so the reference build runs each case with vorticity 0 (the
    restatement must equal it bit for bit there), and the restatement alone
    gives the digests with the configured vorticity (1e-4):
      * one seeded step of the 1M-particle dam break (workloads.dam_break_1m):
        reference build at vorticity 0, restatement at 1e-4;
      * one FluidWorld.step of the coupled pool (workloads.coupled_pool: 250,000
        fluid particles, 8 bodies, a floor plane), fluid state and bodies, from
        the reference build at vorticity 0;
      * one step of each of 32 scenes of workloads.batched_scenes(): reference
        build at vorticity 0, restatement at each scene's own vorticity."""
    R = Ref()
    P = Port()
    P.set_threads(os.cpu_count() or 1)
    out = {}

    def both(sw, vort):
        st = dict(sw.settings, vorticity_epsilon=vort)
        s = Settings.make(**st)
        z = np.zeros(sw.n, np.float32)
        return (R.steps(s, sw.x, sw.v, z, z, sw.dt, sw.gravity, sw.mass, 1),
                P.steps(s, sw.x, sw.v, z, z, sw.dt, sw.gravity, sw.mass, 1))

    def mine_only(sw):
        s = Settings.make(**sw.settings)
        z = np.zeros(sw.n, np.float32)
        return P.steps(s, sw.x, sw.v, z, z, sw.dt, sw.gravity, sw.mass, 1)

    w = workloads.dam_break_1m()
    got, mine = both(w, 0.0)
    for a, b in zip(got, mine):
        assert np.array_equal(a, b), "restatement differs from the reference build (1M)"
    out["dam_break_1m_input"] = digest(w.x)
    out["dam_break_1m_step1_vort0_ref"] = field_digests(*got)
    assert w.settings["vorticity_epsilon"] > 0
    out["dam_break_1m_step1_port"] = field_digests(*mine_only(w))
    print("1M done", flush=True)

    spec = workloads.coupled_pool()
    spec["settings"]["vorticity_epsilon"] = 0.0
    lower, upper, spacing = spec["block"]
    x, v, rho, lam, bp, bq, bv, bw = R.fluid_world_ex(
        Settings.make(**spec["settings"]), lower, upper, spacing, spec["bodies"],
        plane=spec["plane"], gravity=spec["gravity"], boundary_extent=spec["boundary_extent"],
        dt=spec["dt"], nsteps=1)
    d = field_digests(x, v, rho, lam)
    d.update(n=int(len(x)), body_pos=digest(bp), body_quat=digest(bq), body_v=digest(bv),
             body_w=digest(bw))
    out["coupled_pool_step1_vort0_ref"] = d
    print("coupled pool done", len(x), flush=True)

    scenes = workloads.batched_scenes()[BATCH_SUBSET]
    per = []
    for sw in scenes:
        got, mine = both(sw, 0.0)
        for a, b in zip(got, mine):
            assert np.array_equal(a, b), "restatement differs from the reference build (batch)"
        per.append(dict(name=sw.name, n=int(sw.n), vort0_ref=field_digests(*got),
                        port=field_digests(*mine_only(sw))))
    out["batched_subset_step1"] = per
    with open(os.path.join(HERE, "digests_large.json"), "w") as f:
        json.dump(out, f, indent=1, sort_keys=True)
    print("digests_large.json written")


if __name__ == "__main__":
    # With names, only those fixtures: python tests/golden/make_golden.py fluid_world
    names = sys.argv[1:]
    if names:
        if "fluid_world" in names:
            fluid_world_fixture()
        if "fluid_world_contacts" in names:
            fluid_world_contacts_fixture()
        if "large" in names:
            large_digests()
    else:
        main()
        fluid_world_fixture()
        fluid_world_contacts_fixture()
        large_digests()
