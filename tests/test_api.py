"""The NovaPhy-compatible Python API (novaphy_gb300._core) on CPU: kernels,
fluid blocks, particle state, host hash grid, settings and boundary sampling.
Written after the reference's tests/python/test_fluid.py and test_coupling.py;
the host kernels and sampling are also compared bit-for-bit with the oracle."""
import math

import numpy as np
import numpy.testing as npt
import pytest

import novaphy_gb300 as novaphy


def test_kernel_values_and_normalisation():
    h = 0.1
    assert novaphy.SPHKernels.poly6(0.0, h) > 0
    assert abs(novaphy.SPHKernels.poly6(h * h, h)) < 1e-10
    assert novaphy.SPHKernels.poly6(h * h * 1.1, h) == 0.0
    dr = h / 1000
    integral = sum(novaphy.SPHKernels.poly6(((i + 0.5) * dr) ** 2, h) * 4 * math.pi *
                   ((i + 0.5) * dr) ** 2 * dr for i in range(1000))
    npt.assert_allclose(integral, 1.0, atol=0.02)
    assert novaphy.SPHKernels.spiky(0.0, h) > 0 and novaphy.SPHKernels.spiky(h, h) == 0.0
    npt.assert_allclose(novaphy.SPHKernels.spiky_grad(np.array([h, 0, 0], np.float32), h), 0,
                        atol=1e-7)
    assert novaphy.SPHKernels.spiky_grad(np.array([0.05, 0, 0], np.float32), h)[0] < 0
    assert novaphy.SPHKernels.cubic_spline(0.0, h) > 0
    assert novaphy.SPHKernels.cubic_spline(h, h) == 0.0


def test_host_kernels_match_oracle(port):
    rng = np.random.default_rng(3)
    for h in (np.float32(0.1), np.float32(0.04)):
        for r in rng.uniform(0, 1.2 * h, 200).astype(np.float32):
            assert novaphy.SPHKernels.poly6(float(r * r), float(h)) == port.poly6(r * r, h)
            assert novaphy.SPHKernels.spiky(float(r), float(h)) == port.spiky(r, h)
            v = (rng.normal(size=3) * r).astype(np.float32)
            assert np.array_equal(novaphy.SPHKernels.spiky_grad(v, float(h)), port.spiky_grad(v, h))


def test_fluid_block_generation():
    b = novaphy.FluidBlockDef()
    npt.assert_allclose(b.particle_spacing, 0.02, atol=1e-6)
    npt.assert_allclose(b.lower, [0, 0, 0])
    b.lower = np.array([0, 0, 0], np.float32)
    b.upper = np.array([0.1, 0.1, 0.1], np.float32)
    b.particle_spacing = 0.05
    assert len(novaphy.generate_fluid_block(b)) == 27
    b.upper = [0.2, 0.0, 0.0]
    b.particle_spacing = 0.1
    p = novaphy.generate_fluid_block(b)
    assert len(p) == 3
    for a, c in zip(p, p[1:]):
        npt.assert_allclose(np.linalg.norm(c - a), 0.1, atol=1e-5)


def test_particle_state():
    st = novaphy.ParticleState()
    st.init([np.zeros(3, np.float32), [1, 0, 0], (0, 1, 0)])
    assert st.num_particles == 3 and len(st.velocities) == 3 and len(st.densities) == 3
    st.init([[0, 0, 0]], np.array([1.0, 2.0, 3.0], np.float32))
    npt.assert_allclose(st.velocities[0], [1, 2, 3])
    assert st.positions_array.shape == (1, 3)
    st.clear()
    assert st.num_particles == 0


def test_host_hash_grid_matches_reference_order(port):
    g = np.load(__import__("os").path.join(__import__("os").path.dirname(__file__), "golden",
                                           "grid.npz"))
    grid = novaphy.SpatialHashGrid(0.1)
    grid.build(g["cloud"])
    for k, q in enumerate(g["queries"]):
        want = g["cand"][g["offsets"][k]:g["offsets"][k + 1]]
        assert np.array_equal(grid.query_neighbors(q, 0.1), want)
    pts = np.random.default_rng(42).uniform(0, 1, (500, 3)).astype(np.float32)
    grid.build(pts)
    q = np.array([0.5, 0.5, 0.5], np.float32)
    cand = set(grid.query_neighbors(q, 0.1))
    assert {i for i, p in enumerate(pts) if np.linalg.norm(p - q) < 0.1} <= cand
    # known answer: tests/cpp/test_core_span_apis.cpp:42-50
    three = [[0, 0, 0], [0.1, 0, 0], [0.5, 0, 0]]
    grid = novaphy.SpatialHashGrid(0.2)
    grid.build(three)
    assert grid.query_all_pairs(three, 0.2) == [(0, 1)]


def test_settings_defaults_and_mass():
    s = novaphy.PBFSettings()
    npt.assert_allclose(s.rest_density, 1000.0)
    npt.assert_allclose(s.kernel_radius, 0.1, atol=1e-6)
    assert s.solver_iterations == 4 and s.corr_n == 4 and not s.use_domain_bounds
    assert s.exact_arithmetic and s.hash_compat
    # Extensions with no counterpart in the reference are off by default.
    assert not s.boundary_two_way and s.boundary_friction == 0.0
    s.boundary_friction = 0.25
    npt.assert_allclose(s.boundary_friction, 0.25)
    npt.assert_allclose(s.particle_mass(0.05), 0.125, rtol=1e-5)


def test_boundary_sampling_matches_oracle(port):
    mb = novaphy.ModelBuilder()
    half = np.array([0.12, 0.08, 0.1], np.float32)
    b0 = mb.add_body(novaphy.RigidBody.from_box(1.0, half))
    local = novaphy.Transform(np.array([0.01, 0.02, 0.0], np.float32),
                              [0.0, 0.0, math.sin(0.3), math.cos(0.3)])
    mb.add_shape(novaphy.CollisionShape.make_box(half, b0, local))
    b1 = mb.add_body(novaphy.RigidBody.from_sphere(1.0, 0.1))
    mb.add_shape(novaphy.CollisionShape.make_sphere(0.1, b1))
    mb.add_shape(novaphy.CollisionShape.make_plane(np.array([0, 0, 1], np.float32), 0.05))
    model = mb.build()
    got = novaphy.sample_model_boundaries(model, 0.025, plane_extent=0.3)
    q = local.rotation  # [x, y, z, w]
    want = np.concatenate([
        port.sample_box(half, local.position, [q[3], q[0], q[1], q[2]], np.float32(0.025)),
        port.sample_sphere(np.float32(0.1), (0, 0, 0), (1, 0, 0, 0), np.float32(0.025)),
        port.sample_plane(np.array([0, 0, 1], np.float32), np.float32(0.05), np.float32(0.025),
                          np.float32(0.3)),
    ])
    assert len(got) == len(want)
    assert np.array_equal(np.stack([p.local_position for p in got]), want)
    assert [p.body_index for p in got].count(-1) == len(want) - sum(
        1 for p in got if p.body_index >= 0)


def test_reference_sampling_examples():
    mb = novaphy.ModelBuilder()
    half = np.array([0.5, 0.5, 0.5], np.float32)
    idx = mb.add_body(novaphy.RigidBody.from_box(1.0, half))
    mb.add_shape(novaphy.CollisionShape.make_box(half, idx))
    ps = novaphy.sample_model_boundaries(mb.build(), 0.25)
    assert len(ps) > 0 and all(p.body_index == 0 for p in ps)
    mb = novaphy.ModelBuilder()
    idx = mb.add_body(novaphy.RigidBody.from_sphere(1.0, 0.5))
    mb.add_shape(novaphy.CollisionShape.make_sphere(0.5, idx))
    ps = novaphy.sample_model_boundaries(mb.build(), 0.1)
    assert len(ps) > 10
    for p in ps:
        npt.assert_allclose(np.linalg.norm(p.local_position), 0.5, atol=0.01)
    mb = novaphy.ModelBuilder()
    mb.add_ground_plane(y=0.0)
    ps = novaphy.sample_model_boundaries(mb.build(), 0.2, plane_extent=0.5)
    assert len(ps) > 0 and all(abs(p.local_position[1]) < 1e-5 and p.body_index == -1 for p in ps)
    assert len(novaphy.sample_model_boundaries(novaphy.ModelBuilder().build(), 0.1)) == 0
    bp = novaphy.BoundaryParticle()
    npt.assert_allclose(bp.local_position, [0, 0, 0])
    assert bp.body_index == -1 and bp.volume == 0.0


def test_stepping_needs_a_device_and_says_so():
    if novaphy.capi.device_count() > 0:
        pytest.skip("a GPU is visible")
    st = novaphy.ParticleState()
    st.init([[0, 0, 0], [0.02, 0, 0]])
    with pytest.raises(RuntimeError, match="CUDA"):
        novaphy.PBFSolver(novaphy.PBFSettings()).step(st, 1 / 60, [0, -9.81, 0], 0.125)


def _free_body_world():
    mb = novaphy.ModelBuilder()
    mb.add_ground_plane(y=0.0)
    half = np.array([0.5, 0.5, 0.5], np.float32)
    for y in (0.5, 1.5):
        i = mb.add_body(novaphy.RigidBody.from_box(1.0, half),
                        novaphy.Transform.from_translation(np.array([0.0, y, 0.0], np.float32)))
        mb.add_shape(novaphy.CollisionShape.make_box(half, i))
    return novaphy.World(mb.build(), novaphy.SolverSettings())


def test_monitor_is_off_by_default_and_records_nothing():
    w = _free_body_world()
    mon = w.performance_monitor
    assert mon.enabled is False and mon.trace_enabled is False
    w.step(1 / 120)
    assert mon.frame_count == 0 and mon.phase_stats() == [] and mon.last_frame_metrics() == []
    assert mon.last_frame_total_ms == 0.0


def test_monitor_trace_json_and_reset(tmp_path):
    import json

    w = _free_body_world()
    mon = w.performance_monitor
    mon.enabled = True
    mon.trace_enabled = True
    mon.trace_frame_capacity = 2
    for _ in range(3):
        w.step(1 / 120)
    phases = {p.name: p for p in mon.phase_stats()}
    assert {"world.total", "world.integrate_velocity", "world.integrate_position"} <= set(phases)
    assert phases["world.total"].samples == 3 and phases["world.total"].last_ms > 0.0
    metrics = {m.name: m.value for m in mon.last_frame_metrics()}
    assert set(metrics) == {"bodies", "dynamic_bodies", "shapes", "candidate_pairs", "contacts",
                            "solver_iterations"}
    assert (metrics["bodies"], metrics["dynamic_bodies"], metrics["shapes"]) == (2.0, 2.0, 3.0)
    # ground-box, ground-box and box-box overlap; the resting stack touches
    assert metrics["candidate_pairs"] == 3.0 and metrics["contacts"] >= 4.0
    assert metrics["solver_iterations"] == 30.0
    path = tmp_path / "trace.json"
    mon.write_trace_json(path)
    ev = json.loads(path.read_text())["traceEvents"]
    xs = [e for e in ev if e["ph"] == "X"]
    cs = [e for e in ev if e["ph"] == "C"]
    # two frames kept: one world.total each, six counters each
    assert sum(e["name"] == "world.total" for e in xs) == 2 and len(cs) == 12
    assert all(e["dur"] >= 0.0 and e["ts"] >= 0.0 for e in xs)
    tot = [e for e in xs if e["name"] == "world.total"][-1]
    inner = [e for e in xs if e["name"] == "world.integrate_velocity"][-1]
    assert tot["ts"] <= inner["ts"] and inner["ts"] + inner["dur"] <= tot["ts"] + tot["dur"] + 1.0
    mon.reset()
    assert mon.phase_stats() == [] and mon.last_frame_metrics() == [] and mon.frame_count == 0
    mon.write_trace_json(str(path))
    assert json.loads(path.read_text())["traceEvents"] == []


def test_host_world_free_bodies_match_reference_build(ref):
    """The host World's rigid step (free bodies: symplectic Euler with angular
    damping, quaternion update) against the reference's World compiled from
    its sources, bit for bit, with spinning bodies and constant wrenches."""
    bodies = [("sphere", (0.12, 0.0, 0.0), 0.5, (0.0, 1.0, 0.0), (1.0, 0.0, 0.0, 0.0)),
              ("box", (0.1, 0.05, 0.08), 0.8, (2.0, 3.0, -1.0), (0.5, 0.5, 0.5, 0.5))]
    lin = np.array([[0.3, 1.0, -0.2], [-1.0, 0.5, 0.25]], np.float32)
    ang = np.array([[0.0, 2.0, 1.0], [3.0, -1.0, 0.5]], np.float32)
    force = np.array([[0.1, 2.0, 0.0], [0.0, 0.0, -1.5]], np.float32)
    torque = np.array([[0.01, 0.0, -0.02], [0.0, 0.03, 0.01]], np.float32)
    dt, steps = float(np.float32(1 / 120)), 50
    rp, rq, rv, rw = ref.world(bodies, lin, ang, dt, steps, force, torque)

    mb = novaphy.ModelBuilder()
    for kind, size, mass, pos, q in bodies:
        t = novaphy.Transform(np.array(pos, np.float32), [q[1], q[2], q[3], q[0]])
        if kind == "sphere":
            i = mb.add_body(novaphy.RigidBody.from_sphere(mass, size[0]), t)
            mb.add_shape(novaphy.CollisionShape.make_sphere(size[0], i))
        else:
            he = np.array(size, np.float32)
            i = mb.add_body(novaphy.RigidBody.from_box(mass, he), t)
            mb.add_shape(novaphy.CollisionShape.make_box(he, i))
    w = novaphy.World(mb.build(), novaphy.SolverSettings())
    for k in range(2):
        w.state.set_linear_velocity(k, lin[k])
        w.state.set_angular_velocity(k, ang[k])
    for _ in range(steps):
        for k in range(2):
            w.apply_force(k, force[k])
            w.apply_torque(k, torque[k])
        w.step(dt)
    for k in range(2):
        tr = w.state.transforms[k]
        q = np.asarray(tr.rotation, np.float32)  # x, y, z, w
        assert np.array_equal(np.asarray(tr.position, np.float32), rp[k]), k
        assert np.array_equal(np.array([q[3], q[0], q[1], q[2]], np.float32), rq[k]), k
        assert np.array_equal(np.asarray(w.state.linear_velocities[k], np.float32), rv[k]), k
        assert np.array_equal(np.asarray(w.state.angular_velocities[k], np.float32), rw[k]), k


def test_transform_exports_and_batch_vertex_transform():
    mb = novaphy.ModelBuilder()
    q = np.array([0.1, 0.7, -0.2, 0.68], np.float32)  # x, y, z, w
    for k in range(3):
        mb.add_body(novaphy.RigidBody.from_sphere(1.0, 0.1),
                    novaphy.Transform(np.array([k, 2.0 * k, -1.0], np.float32), q))
    w = novaphy.World(mb.build(), novaphy.SolverSettings())
    pos, quat = w.state.get_transforms_numpy()
    assert pos.shape == (3, 3) and quat.shape == (3, 4)
    for k, t in enumerate(w.state.transforms):
        assert np.array_equal(pos[k], np.asarray(t.position, np.float32))
        assert np.array_equal(quat[k], np.asarray(t.rotation, np.float32))
    p2, q2 = np.zeros((3, 3), np.float32), np.zeros((3, 4), np.float32)
    w.state.get_transforms_into(p2, q2)
    assert np.array_equal(p2, pos) and np.array_equal(q2, quat)
    with pytest.raises(ValueError):
        w.state.get_transforms_into(np.zeros((2, 3), np.float32), q2)

    rng = np.random.default_rng(5)
    idx = np.array([2, 0, 2, 1], np.int32)
    local = rng.normal(size=(4, 5, 3)).astype(np.float32)
    out = np.zeros((20, 3), np.float32)
    novaphy.batch_transform_vertices(pos, quat, idx, local, out)
    # the same float operations in numpy float32: rotation from (x, y, z, w),
    # then r0 v0 + r1 v1 + r2 v2 + p left to right
    one, two = np.float32(1), np.float32(2)
    for i, b in enumerate(idx):
        x, y, z, s = quat[b]
        r = np.array([[one - two * (y * y + z * z), two * (x * y - s * z), two * (x * z + s * y)],
                      [two * (x * y + s * z), one - two * (x * x + z * z), two * (y * z - s * x)],
                      [two * (x * z - s * y), two * (y * z + s * x), one - two * (x * x + y * y)]],
                     np.float32)
        for j in range(5):
            v = local[i, j]
            want = [((r[d, 0] * v[0] + r[d, 1] * v[1]) + r[d, 2] * v[2]) + pos[b, d]
                    for d in range(3)]
            assert np.array_equal(out[5 * i + j], np.array(want, np.float32)), (i, j)
    with pytest.raises(IndexError):
        novaphy.batch_transform_vertices(pos, quat, np.array([3], np.int32), local[:1], out)
