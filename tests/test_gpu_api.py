"""The NovaPhy-compatible API on the GPU: PBFSolver and FluidWorld, written
after the reference's tests/python/test_pbf.py, test_coupling.py and
test_performance_monitor.py, plus bit-exact checks against the oracle."""
import json
import os

import numpy as np
import numpy.testing as npt
import pytest

import novaphy_gb300 as novaphy

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def make_pbf_state(spacing=0.025, block_size=0.3):
    b = novaphy.FluidBlockDef()
    b.lower = np.array([0, 0, 0], np.float32)
    b.upper = np.array([block_size] * 3, np.float32)
    b.particle_spacing = spacing
    s = novaphy.PBFSettings()
    s.kernel_radius = spacing * 4.0
    st = novaphy.ParticleState()
    st.init(novaphy.generate_fluid_block(b))
    return st, s, s.particle_mass(spacing)


def test_pbf_step_runs_and_particles_fall():
    st, s, m = make_pbf_state()
    solver = novaphy.PBFSolver(s)
    y0 = np.mean([p[1] for p in st.positions])
    for _ in range(10):
        solver.step(st, 1 / 60, np.array([0, -9.81, 0], np.float32), m)
    assert np.mean([p[1] for p in st.positions]) < y0
    assert max(np.linalg.norm(v) for v in st.velocities) > 0


def test_zero_gravity_com_and_density():
    st, s, m = make_pbf_state()
    solver = novaphy.PBFSolver(s)
    c0 = np.mean(st.positions_array, axis=0)
    for _ in range(5):
        solver.step(st, 1 / 60, [0, 0, 0], m)
    assert np.linalg.norm(np.mean(st.positions_array, axis=0) - c0) < 0.05
    assert np.mean(st.densities) > 0


def test_pbf_solver_is_the_reference_step_bit_for_bit():
    g = np.load(os.path.join(GOLDEN, "default_scene.npz"))
    st = novaphy.ParticleState()
    st.init(g["x0"])
    s = novaphy.PBFSettings()  # defaults: exact arithmetic, reference hash buckets
    novaphy.PBFSolver(s).step(st, float(np.float32(1 / 60)), [0, -9.81, 0],
                              float(np.float32(1000) * np.float32(0.025) ** 3))
    assert np.array_equal(st.positions_array, g["x1"])
    assert np.array_equal(st.velocities_array, g["v1"])
    assert np.array_equal(st.densities_array, g["rho1"])
    assert np.array_equal(np.array(st.lambdas, np.float32), g["lam1"])


def test_settings_edits_are_read_every_step():
    st, s, m = make_pbf_state(block_size=0.15)
    solver = novaphy.PBFSolver(s)
    solver.settings.solver_iterations = 0
    solver.step(st, 1 / 60, [0, -9.81, 0], m)
    assert all(d == 0.0 for d in st.densities)  # no density pass ran
    solver.settings.solver_iterations = 2
    solver.step(st, 1 / 60, [0, -9.81, 0], m)
    assert max(st.densities) > 0


def block(lower, upper, spacing=0.05):
    b = novaphy.FluidBlockDef()
    b.lower = np.array(lower, np.float32)
    b.upper = np.array(upper, np.float32)
    b.particle_spacing = spacing
    return b


def test_fluid_world_basics():
    mb = novaphy.ModelBuilder()
    mb.add_ground_plane(y=0.0)
    pbf = novaphy.PBFSettings()
    pbf.kernel_radius = 0.2
    w = novaphy.FluidWorld(mb.build(), [block([0, 0.1, 0], [0.2, 0.3, 0.2])],
                           novaphy.SolverSettings(), pbf, boundary_extent=0.5)
    assert isinstance(w, novaphy.World)
    assert w.num_boundary_particles > 0 and w.num_particles > 0
    n0 = w.num_particles
    w.step(1 / 60)
    assert w.fluid_state.num_particles == n0
    empty = novaphy.FluidWorld(novaphy.ModelBuilder().build(), [], novaphy.SolverSettings(), pbf)
    empty.step(1 / 60)
    assert empty.num_particles == 0


def sphere_scene(fluid=True, y=0.8, mass=0.5, radius=0.2):
    mb = novaphy.ModelBuilder()
    mb.add_ground_plane(y=0.0)
    idx = mb.add_body(novaphy.RigidBody.from_sphere(mass, radius),
                      novaphy.Transform.from_translation(np.array([0.1, y, 0.1], np.float32)))
    mb.add_shape(novaphy.CollisionShape.make_sphere(radius, idx))
    pbf = novaphy.PBFSettings()
    pbf.kernel_radius = 0.2
    pbf.solver_iterations = 2
    blocks = [block([0, 0.05, 0], [0.3, 0.4, 0.3])] if fluid else []
    return novaphy.FluidWorld(mb.build(), blocks, novaphy.SolverSettings(), pbf,
                              boundary_extent=0.5)


def test_coupled_simulation_runs_and_sphere_falls():
    w = sphere_scene()
    for _ in range(5):
        w.step(1 / 60)
    assert w.state.transforms[0].position[1] < 0.8
    nf = sphere_scene(fluid=False)
    for _ in range(5):
        nf.step(1 / 60)
    assert nf.state.transforms[0].position[1] < 0.8


def test_monitor_reports_fluid_phases_and_metrics(tmp_path):
    w = sphere_scene()
    mon = w.performance_monitor
    mon.enabled = True
    mon.trace_enabled = True
    w.step(1 / 60)
    phases = {p.name: p for p in mon.phase_stats()}
    want = {"fluid.total", "fluid.pbf.total", "fluid.rigid_step", "world.total",
            "fluid.boundary.positions", "fluid.boundary_density", "fluid.coupling.total"}
    want |= {"fluid.pbf." + k for k in ("predict", "grid_build", "neighbor_query",
                                         "iteration.compute_density",
                                         "iteration.compute_delta_position", "xsph_viscosity",
                                         "commit_positions")}
    assert want <= set(phases)
    assert phases["fluid.pbf.iteration.compute_density"].last_ms > 0.0
    assert phases["fluid.coupling.total"].last_ms > 0.0
    metrics = {m.name: m.value for m in mon.last_frame_metrics()}
    assert metrics["fluid_particles"] > 0 and metrics["boundary_particles"] >= 0
    assert metrics["pbf_solver_iterations"] == 2.0
    assert abs(metrics["kernel_radius"] - 0.2) < 1e-6
    assert metrics["bodies"] == 1.0 and metrics["dynamic_bodies"] == 1.0
    assert mon.frame_count == 1
    path = tmp_path / "fluid_trace.json"
    mon.write_trace_json(path)
    ev = json.loads(path.read_text())["traceEvents"]
    assert {e["name"] for e in ev if e["ph"] == "X" and e["tid"] == 1} >= {
        "fluid.pbf.iteration.compute_density", "fluid.coupling.total"}
    assert any(e["ph"] == "C" and e["name"] == "fluid_particles" for e in ev)
    mon.reset()
    assert mon.frame_count == 0 and mon.phase_stats() == []


def test_profiled_fluid_world_steps_like_the_plain_one():
    # The monitor switches to the profiled launch sequence; the state must not move.
    a, b = sphere_scene(), sphere_scene()
    b.performance_monitor.enabled = True
    for _ in range(3):
        a.step(1 / 60)
        b.step(1 / 60)
    for name in ("positions_array", "velocities_array", "densities_array"):
        assert np.array_equal(getattr(a.fluid_state, name), getattr(b.fluid_state, name)), name
    assert np.array_equal(np.asarray(a.fluid_state.lambdas, np.float32),
                          np.asarray(b.fluid_state.lambdas, np.float32))
    pa, pb = a.state.transforms[0].position, b.state.transforms[0].position
    assert np.array_equal(np.asarray(pa, np.float32), np.asarray(pb, np.float32))


def test_fluid_world_step_matches_oracle(port):
    """One FluidWorld step: fluid state = reference PBF step + boundary density;
    the sphere's new velocity comes from the coupling force the oracle gives."""
    from oracle.oracle import Settings

    w = sphere_scene(y=0.25, radius=0.12)
    fs0 = w.fluid_state
    x0 = fs0.positions_array.copy()
    bps = w.boundary_particles
    local = np.stack([b.local_position for b in bps]).astype(np.float32)
    body = np.array([b.body_index for b in bps], np.int32)
    psi = np.array([b.volume for b in bps], np.float32)
    body_pos = np.array([[0.1, 0.25, 0.1]], np.float32)
    world0 = port.boundary_world_positions(local, body, body_pos, [[1, 0, 0, 0]])
    assert np.array_equal(port.boundary_volumes(world0, np.float32(0.2)), psi)
    dt = float(np.float32(1 / 60))
    w.step(dt)
    s = Settings.make(kernel_radius=0.2, solver_iterations=2)
    z = np.zeros(len(x0), np.float32)
    sp = np.float32(0.05)
    m = np.float32(np.float32(np.float32(1000) * sp) * sp) * sp  # particle_mass order
    ox, ov, orho, olam = port.steps(s, x0, np.zeros_like(x0), z, z, dt,
                                    np.array([0, -9.81, 0], np.float32), m, 1)
    fs = w.fluid_state
    assert np.array_equal(fs.positions_array, ox)
    assert np.array_equal(fs.velocities_array, ov)
    orho = port.boundary_density(ox, orho, world0, psi, np.float32(0.2), np.float32(1000))
    assert np.array_equal(fs.densities_array, orho)
    f, _ = port.coupling_forces(ox, orho, m, world0, body, psi, [1], body_pos, np.float32(0.2),
                                np.float32(1000))
    # symplectic Euler of the sphere: v = (g + F / m) dt
    inv_m = np.float32(1) / np.float32(0.5)
    g = np.array([0, -9.81, 0], np.float32)
    v_want = (g + f[0] * inv_m) * np.float32(dt)
    npt.assert_array_equal(np.asarray(w.state.linear_velocities[0], np.float32), v_want)


def test_fluid_world_matches_reference_fixture():
    """Five FluidWorld steps of a coupled scene (fluid block, ground plane, a
    sphere and a rotated box that stay clear of each other and of the plane, so
    the reference's contact solver has nothing to do) against the reference's own FluidWorld built
    from its sources (tests/golden/fluid_world.npz, make_golden.py): fluid
    state with boundary density and the bodies' poses and velocities, bit for
    bit."""
    g = np.load(os.path.join(GOLDEN, "fluid_world.npz"))
    mb = novaphy.ModelBuilder()
    mb.add_ground_plane(y=0.0)
    i = mb.add_body(novaphy.RigidBody.from_sphere(0.5, 0.08),
                    novaphy.Transform(np.array([0.06, 0.25, 0.06], np.float32), [0, 0, 0, 1]))
    mb.add_shape(novaphy.CollisionShape.make_sphere(0.08, i))
    he = np.array([0.04, 0.04, 0.04], np.float32)
    i = mb.add_body(novaphy.RigidBody.from_box(0.8, he),
                    novaphy.Transform(np.array([0.26, 0.33, 0.26], np.float32),
                                      [0.0, 0.25881904, 0.0, 0.96592583]))
    mb.add_shape(novaphy.CollisionShape.make_box(he, i))
    pbf = novaphy.PBFSettings()
    pbf.kernel_radius = 0.2
    pbf.solver_iterations = 2
    blk = novaphy.FluidBlockDef()
    blk.lower = np.array([0.0, 0.05, 0.0], np.float32)
    blk.upper = np.array([0.3, 0.4, 0.3], np.float32)
    blk.particle_spacing = 0.05
    fw = novaphy.FluidWorld(mb.build(), [blk], novaphy.SolverSettings(), pbf,
                            boundary_extent=0.5)
    dt = float(np.float32(1 / 60))
    for _ in range(5):
        fw.step(dt)
    fs = fw.fluid_state
    assert np.array_equal(fs.positions_array, g["x"])
    assert np.array_equal(fs.velocities_array, g["v"])
    assert np.array_equal(fs.densities_array, g["rho"])
    assert np.array_equal(np.asarray(fs.lambdas, np.float32), g["lam"])
    for k in range(2):
        tr = fw.state.transforms[k]
        q = np.asarray(tr.rotation, np.float32)  # x, y, z, w
        assert np.array_equal(np.asarray(tr.position, np.float32), g["body_pos"][k]), k
        assert np.array_equal(np.array([q[3], q[0], q[1], q[2]], np.float32), g["body_quat"][k]), k
        assert np.array_equal(np.asarray(fw.state.linear_velocities[k], np.float32),
                              g["body_v"][k]), k
        assert np.array_equal(np.asarray(fw.state.angular_velocities[k], np.float32),
                              g["body_w"][k]), k


def test_fluid_world_with_contacts_matches_reference_fixture():
    """Eight FluidWorld steps with the host contact pipeline at work every
    step (a sphere pressed into the ground, a box on an edge, then the fluid
    pushing them together) against the reference's own FluidWorld
    (tests/golden/fluid_world_contacts.npz, which stores the scene too): fluid
    state and both bodies, bit for bit."""
    g = np.load(os.path.join(GOLDEN, "fluid_world_contacts.npz"))
    spacing, plane_y, extent, steps, dt = (float(t) for t in g["scene_scalars"])
    mb = novaphy.ModelBuilder()
    mb.add_ground_plane(y=plane_y)
    for kind, size, mass, pos, q in zip(g["scene_kind"], g["scene_size"], g["scene_mass"],
                                        g["scene_pos"], g["scene_quat"]):
        tr = novaphy.Transform(pos, [float(q[1]), float(q[2]), float(q[3]), float(q[0])])
        if kind == 0:
            i = mb.add_body(novaphy.RigidBody.from_sphere(float(mass), float(size[0])), tr)
            mb.add_shape(novaphy.CollisionShape.make_sphere(float(size[0]), i))
        else:
            i = mb.add_body(novaphy.RigidBody.from_box(float(mass), size), tr)
            mb.add_shape(novaphy.CollisionShape.make_box(size, i))
    pbf = novaphy.PBFSettings()
    pbf.kernel_radius = 0.2
    pbf.solver_iterations = 2
    blk = novaphy.FluidBlockDef()
    blk.lower, blk.upper = g["scene_block"][0], g["scene_block"][1]
    blk.particle_spacing = spacing
    fw = novaphy.FluidWorld(mb.build(), [blk], novaphy.SolverSettings(), pbf,
                            boundary_extent=extent)
    kinds = set()
    for _ in range(int(steps)):
        fw.step(dt)
        assert len(fw.contacts) >= 3
        kinds |= {(c.body_a, c.body_b) for c in fw.contacts}
    assert kinds >= {(-1, 0), (-1, 1)} and len(kinds) == 3  # ground-sphere, ground-box, box-sphere
    fs = fw.fluid_state
    assert np.array_equal(fs.positions_array, g["x"])
    assert np.array_equal(fs.velocities_array, g["v"])
    assert np.array_equal(fs.densities_array, g["rho"])
    assert np.array_equal(np.asarray(fs.lambdas, np.float32), g["lam"])
    for k in range(len(g["scene_kind"])):
        tr = fw.state.transforms[k]
        q = np.asarray(tr.rotation, np.float32)  # x, y, z, w
        got = [np.asarray(tr.position, np.float32), np.array([q[3], q[0], q[1], q[2]], np.float32),
               np.asarray(fw.state.linear_velocities[k], np.float32),
               np.asarray(fw.state.angular_velocities[k], np.float32)]
        for name, a in zip(("body_pos", "body_quat", "body_v", "body_w"), got):
            assert np.array_equal(a.view(np.uint32), g[name][k].view(np.uint32)), (name, k)
