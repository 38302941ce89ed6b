"""The serving loop (pbf_server_*): continuous batching over device-resident
scenes, HBM-budget admission, failure isolation.

The equality bar: a scene served among others (its requests coalesced into
batch launches with whatever else is pending, from several client threads)
ends bit for bit where the same sequence of steps leaves it when stepped
alone with pbf_scene_step (exact arithmetic, the default).
"""
import threading
import time

import numpy as np
import pytest

from novaphy_gb300 import capi, workloads

pytestmark = pytest.mark.gpu


def small_scenes(k=6, seed=31, lo=500, hi=4000):
    return workloads.batched_scenes(nscenes=k, seed=seed, n_lo=lo, n_hi=hi)


def settings_of(w, **kw):
    st = dict(w.settings)
    st.update(kw)
    return capi.default_settings(**st)


def alone(w, dts):
    sc = capi.Scene(settings_of(w), w.x, w.v, mass=w.mass)
    sc.set_gravity(w.gravity)
    for dt in dts:
        sc.step(np.float32(dt), 1)
    out = [sc.read(f) for f in (capi.FIELD_POSITIONS, capi.FIELD_VELOCITIES,
                                capi.FIELD_DENSITIES, capi.FIELD_LAMBDAS)]
    sc.close()
    return out


def served(srv, sid, n):
    return [srv.read(sid, f, n) for f in (capi.FIELD_POSITIONS, capi.FIELD_VELOCITIES,
                                          capi.FIELD_DENSITIES, capi.FIELD_LAMBDAS)]


def same(a, b):
    return all(np.array_equal(x.view(np.uint32), y.view(np.uint32)) for x, y in zip(a, b))


@pytest.mark.parametrize("min_step", [1 << 20, 0])
def test_alone_equals_mix_under_concurrent_clients(min_step):
    # min_step=0 lets launches take several steps of the deeper queues.
    ws = small_scenes()
    srv = capi.Server(capi.server_config(min_step_particles=min_step))
    ids = []
    for w in ws:
        sid, st = srv.open_scene(settings_of(w), w.x, w.v, w.mass, w.gravity)
        assert st == capi.SCENE_RESIDENT
        ids.append(sid)
    rng = np.random.default_rng(5)
    plans = [[(float(np.float32(w.dt * rng.choice([1.0, 0.5]))), int(rng.choice([1, 2, 4])))
              for _ in range(4)] for w in ws]

    def client(k):
        r = np.random.default_rng(100 + k)
        reqs = []
        for dt, m in plans[k]:
            time.sleep(float(r.uniform(0, 0.01)))
            reqs.append(srv.submit(ids[k], dt, m))
        for q in reqs:
            assert srv.wait(q) == capi.REQ_DONE

    th = [threading.Thread(target=client, args=(k,)) for k in range(len(ws))]
    for t in th:
        t.start()
    for t in th:
        t.join()
    st = srv.stats()
    assert st["requests_done"] == sum(len(p) for p in plans)
    assert st["steps_done"] == sum(m for p in plans for _, m in p)
    for k, w in enumerate(ws):
        dts = [dt for dt, m in plans[k] for _ in range(m)]
        assert same(served(srv, ids[k], w.n), alone(w, dts)), k
    srv.close()


def test_requests_are_batched_together():
    ws = small_scenes(k=4, seed=7)
    srv = capi.Server()
    ids = [srv.open_scene(settings_of(w), w.x, w.v, w.mass, w.gravity)[0] for w in ws]
    reqs = [srv.submit(sid, ws[0].dt, 16) for sid in ids]
    for q in reqs:
        srv.wait(q)
    st = srv.stats()
    assert st["steps_done"] == 64
    assert st["mean_launch_scenes"] > 1.0, st
    assert st["launches"] < 64
    assert 0.0 < st["step_ms_p50"] <= st["step_ms_p99"]
    assert 0.0 < st["request_ms_p50"] <= st["request_ms_p99"]
    assert st["particle_steps"] == 16 * sum(w.n for w in ws)
    srv.close()


def test_budget_admission_waits_fifo_and_admits_on_close():
    ws = small_scenes(k=3, seed=9, lo=2000, hi=3000)
    probe = capi.Server()
    charges = []
    for w in ws:
        before = probe.stats()["hbm_bytes_charged"]
        probe.open_scene(settings_of(w), w.x, w.v, w.mass, w.gravity)
        charges.append(probe.stats()["hbm_bytes_charged"] - before)
    scratch = probe.stats()["hbm_bytes_scratch"]
    probe.close()
    # The first two fit, the third does not until the first is closed.
    budget = scratch + max(charges[0] + charges[1], charges[1] + charges[2])
    srv = capi.Server(capi.server_config(hbm_budget_bytes=budget))
    a, sa = srv.open_scene(settings_of(ws[0]), ws[0].x, ws[0].v, ws[0].mass, ws[0].gravity)
    b, sb = srv.open_scene(settings_of(ws[1]), ws[1].x, ws[1].v, ws[1].mass, ws[1].gravity)
    c, sc = srv.open_scene(settings_of(ws[2]), ws[2].x, ws[2].v, ws[2].mass, ws[2].gravity)
    assert (sa, sb, sc) == (capi.SCENE_RESIDENT, capi.SCENE_RESIDENT, capi.SCENE_WAITING)
    assert srv.stats()["scenes_waiting"] == 1
    q = srv.submit(c, ws[2].dt, 2)  # queued behind admission
    with pytest.raises(capi.PbfError) as e:
        srv.wait(q, timeout=0.2)
    assert e.value.code == capi.PBF_ERR_TIMEOUT
    srv.close_scene(a)
    assert srv.wait(q, timeout=30.0) == capi.REQ_DONE
    assert srv.scene_state(c) == capi.SCENE_RESIDENT
    assert same(served(srv, c, ws[2].n), alone(ws[2], [ws[2].dt, ws[2].dt]))
    srv.close()


def test_scene_that_never_fits_is_rejected():
    w = small_scenes(k=1, seed=3)[0]
    probe = capi.Server()
    scratch = probe.stats()["hbm_bytes_scratch"]
    probe.close()
    srv = capi.Server(capi.server_config(hbm_budget_bytes=scratch + 1000))
    with pytest.raises(capi.PbfError) as e:
        srv.open_scene(settings_of(w), w.x, w.v, w.mass, w.gravity)
    assert e.value.code == capi.PBF_ERR_CAPACITY
    assert srv.stats()["scenes_rejected"] == 1
    srv.close()


def test_nonfinite_scene_fails_alone():
    ws = small_scenes(k=2, seed=13)
    srv = capi.Server()
    bad_x = ws[0].x.copy()
    bad_x[7] = np.nan
    a, _ = srv.open_scene(settings_of(ws[0]), bad_x, ws[0].v, ws[0].mass, ws[0].gravity)
    b, _ = srv.open_scene(settings_of(ws[1]), ws[1].x, ws[1].v, ws[1].mass, ws[1].gravity)
    qa = srv.submit(a, ws[0].dt, 3)
    qb = srv.submit(b, ws[1].dt, 3)
    with pytest.raises(capi.PbfError) as e:
        srv.wait(qa)
    assert e.value.code == capi.PBF_ERR_NONFINITE
    assert srv.wait(qb) == capi.REQ_DONE
    assert srv.scene_state(a) == capi.SCENE_FAILED
    with pytest.raises(capi.PbfError) as e:
        srv.submit(a, ws[0].dt, 1)
    assert e.value.code == capi.PBF_ERR_NONFINITE
    assert same(served(srv, b, ws[1].n), alone(ws[1], [ws[1].dt] * 3))
    st = srv.stats()
    assert st["scenes_failed"] == 1 and st["requests_failed"] == 1
    srv.close()


def test_close_waits_for_pending_requests():
    w = small_scenes(k=1, seed=17)[0]
    srv = capi.Server()
    sid, _ = srv.open_scene(settings_of(w), w.x, w.v, w.mass, w.gravity)
    qs = [srv.submit(sid, w.dt, 2) for _ in range(3)]
    srv.close_scene(sid)
    for q in qs:
        assert srv.wait(q) == capi.REQ_DONE
    assert srv.stats()["steps_done"] == 6
    srv.close()


def test_batch_reports_nonfinite_scenes():
    ws = small_scenes(k=3, seed=19)
    bad_x = ws[1].x.copy()
    bad_x[0] = np.nan
    scenes = []
    for k, w in enumerate(ws):
        sc = capi.Scene(settings_of(w), bad_x if k == 1 else w.x, w.v, mass=w.mass)
        sc.set_gravity(w.gravity)
        scenes.append(sc)
    b = capi.Batch()
    b.step(scenes, ws[0].dt)
    assert list(b.nonfinite(3)) == [0, 1, 0]


def test_reads_and_closes_while_other_scenes_run():
    """Client threads read and close their scenes while other scenes' launches
    are queued and being captured; every scene still matches its lone run."""
    ws = small_scenes(k=8, seed=41, lo=1000, hi=6000)
    srv = capi.Server()
    ids = [srv.open_scene(settings_of(w), w.x, w.v, w.mass, w.gravity)[0] for w in ws]
    results = {}
    errors = []

    def client(k):
        try:
            w, sid = ws[k], ids[k]
            steps = 0
            for m in (4, 1, 16, 2):
                srv.wait(srv.submit(sid, w.dt, m))
                steps += m
                served(srv, sid, w.n)  # read between requests
            results[k] = (served(srv, sid, w.n), steps)
            if k % 2 == 0:
                srv.close_scene(sid)
        except Exception as e:  # noqa: BLE001
            errors.append(repr(e))

    th = [threading.Thread(target=client, args=(k,)) for k in range(len(ws))]
    for t in th:
        t.start()
    for t in th:
        t.join()
    assert not errors, errors
    st = srv.stats()
    assert st["scenes_failed"] == 0 and st["requests_failed"] == 0
    for k, w in enumerate(ws):
        got, steps = results[k]
        assert same(got, alone(w, [w.dt] * steps)), k
    srv.close()


def test_coupled_served_scene_equals_fluid_world():
    """A served scene with Akinci rigid bodies follows FluidWorld.step bit for
    bit: fluid state (with boundary density) and the bodies' poses and
    velocities after several steps, the PBF step batched with another scene.
    Served bodies are free bodies (the device rigid step has no contacts), so
    the bodies here stay apart and off the ground for the four steps (the
    fluid drives them together from the sixth step on), which the host
    World's contact count confirms every step."""
    import novaphy_gb300 as nv

    mb = nv.ModelBuilder()
    mb.add_ground_plane(y=0.0)
    si = mb.add_body(nv.RigidBody.from_sphere(0.5, 0.12),
                     nv.Transform.from_translation(np.array([0.1, 0.25, 0.1], np.float32)))
    mb.add_shape(nv.CollisionShape.make_sphere(0.12, si))
    bi = mb.add_body(nv.RigidBody.from_box(0.8, np.array([0.05, 0.05, 0.05], np.float32)),
                     nv.Transform(np.array([0.4, 0.3, 0.15], np.float32),
                                  [0.0, 0.25881904, 0.0, 0.96592583]))
    mb.add_shape(nv.CollisionShape.make_box(np.array([0.05, 0.05, 0.05], np.float32), bi))
    model = mb.build()
    pbf = nv.PBFSettings()
    pbf.kernel_radius = 0.2
    pbf.solver_iterations = 2
    blk = nv.FluidBlockDef()
    blk.lower = np.array([0, 0.05, 0], np.float32)
    blk.upper = np.array([0.3, 0.4, 0.3], np.float32)
    blk.particle_spacing = 0.05
    fw = nv.FluidWorld(model, [blk], nv.SolverSettings(), pbf, boundary_extent=0.5)
    x0 = fw.fluid_state.positions_array.copy()
    v0 = fw.fluid_state.velocities_array.copy()
    bps = fw.boundary_particles
    local = np.stack([b.local_position for b in bps]).astype(np.float32)
    body = np.array([b.body_index for b in bps], np.int32)
    psi = np.array([b.volume for b in bps], np.float32)
    bodies = []
    for k, rb in enumerate(model.bodies):
        tr = model.initial_transforms[k]
        q = np.asarray(tr.rotation, np.float32)  # x, y, z, w
        b = capi.RigidBody()
        b.pos[:] = [float(c) for c in tr.position]
        b.quat[:] = [float(q[3]), float(q[0]), float(q[1]), float(q[2])]
        b.inv_mass = rb.inv_mass()
        b.inv_inertia[:] = rb.inv_inertia()
        bodies.append(b)
    st = capi.Settings()
    for name, _ in capi.Settings._fields_:
        val = getattr(fw.pbf_settings, name)
        if name in ("domain_lower", "domain_upper"):
            getattr(st, name)[:] = [float(c) for c in val]
        else:
            setattr(st, name, val)
    mass = fw.pbf_settings.particle_mass(0.05)
    g = [0.0, -9.81, 0.0]
    dt = float(np.float32(1 / 60))
    nsteps = 4

    other = small_scenes(k=1, seed=23)[0]
    # min_step_particles=0: the 4-step requests run as multi-step launches, so
    # the coupling and rigid step also run between steps inside a launch.
    srv = capi.Server(capi.server_config(min_step_particles=0))
    oid, _ = srv.open_scene(settings_of(other), other.x, other.v, other.mass, other.gravity)
    sid, state = srv.open_coupled_scene(st, x0, v0, mass, g, local, body, psi, bodies)
    assert state == capi.SCENE_RESIDENT
    qo = srv.submit(oid, other.dt, nsteps)
    qs = srv.submit(sid, dt, nsteps)
    assert srv.wait(qs) == capi.REQ_DONE and srv.wait(qo) == capi.REQ_DONE
    for _ in range(nsteps):
        fw.step(dt)
        assert len(fw.contacts) == 0
    fs = fw.fluid_state
    for got, want in ((srv.read(sid, capi.FIELD_POSITIONS, len(x0)), fs.positions_array),
                      (srv.read(sid, capi.FIELD_VELOCITIES, len(x0)), fs.velocities_array),
                      (srv.read(sid, capi.FIELD_DENSITIES, len(x0)), fs.densities_array)):
        assert np.array_equal(got.view(np.uint32), np.asarray(want, np.float32).view(np.uint32))
    out = srv.read_bodies(sid, len(bodies))
    for k, b in enumerate(out):
        tr = fw.state.transforms[k]
        q = np.asarray(tr.rotation, np.float32)
        assert np.array_equal(np.array(b.pos, np.float32), np.asarray(tr.position, np.float32)), k
        assert np.array_equal(np.array(b.quat, np.float32), q[[3, 0, 1, 2]]), k
        assert np.array_equal(np.array(b.lin_vel, np.float32),
                              np.asarray(fw.state.linear_velocities[k], np.float32)), k
        assert np.array_equal(np.array(b.ang_vel, np.float32),
                              np.asarray(fw.state.angular_velocities[k], np.float32)), k
    assert out[0].pos[1] != 0.25  # the sphere moved
    srv.close()


def test_finished_request_records_are_bounded():
    # Zero-step requests finish at submission: no device work, only records.
    w = small_scenes(k=1)[0]
    srv = capi.Server()
    sid, _ = srv.open_scene(settings_of(w), w.x, w.v, w.mass, w.gravity)
    kept = 1 << 16
    ids = [srv.submit(sid, w.dt, 0) for _ in range(kept + 10)]
    assert srv.wait(ids[-1]) == capi.REQ_DONE
    assert srv.wait(ids[10]) == capi.REQ_DONE  # the oldest record still kept
    with pytest.raises(capi.PbfError):
        srv.wait(ids[0])  # dropped
    q = srv.submit(sid, w.dt, 2)  # real steps still run and report
    assert srv.wait(q) == capi.REQ_DONE
    st = srv.stats()
    assert st["requests_done"] == kept + 11 and st["steps_done"] == 2
    srv.close_scene(sid)
    srv.close()


def test_deep_queue_runs_several_steps_per_launch():
    # A 16-step request alone: the launch takes further steps of the same
    # scene (up to the particle-step cap), with the same result as 16 steps.
    w = small_scenes(k=1, seed=12)[0]
    srv = capi.Server(capi.server_config(min_step_particles=0))
    sid, _ = srv.open_scene(settings_of(w), w.x, w.v, w.mass, w.gravity)
    q = srv.submit(sid, w.dt, 16)
    assert srv.wait(q) == capi.REQ_DONE
    st = srv.stats()
    assert st["steps_done"] == 16 and st["launches"] < 16, st
    assert 0.0 < st["step_ms_p50"] <= st["step_ms_p99"]
    assert same(served(srv, sid, w.n), alone(w, [w.dt] * 16))
    srv.close()


def served_shapes_of(model):
    """capi.RigidShape for each of a model's sphere and plane shapes, in model order."""
    import novaphy_gb300 as nv

    out = []
    for sh in model.shapes:
        s = capi.RigidShape()
        s.body = sh.body_index
        s.friction = sh.friction
        s.restitution = sh.restitution
        if sh.type == nv.ShapeType.Sphere:
            s.type = capi.SHAPE_SPHERE
            s.radius = sh.sphere_radius
            s.local_pos[:] = [float(c) for c in sh.local_transform.position]
        else:
            assert sh.type == nv.ShapeType.Plane
            s.type = capi.SHAPE_PLANE
            s.normal[:] = [float(c) for c in sh.plane_normal]
            s.offset = sh.plane_offset
        out.append(s)
    return out


def test_served_scene_with_contacts_equals_fluid_world():
    """A served coupled scene whose bodies collide follows FluidWorld.step bit
    for bit: a sphere resting on the ground plane, a second sphere pressed
    against it, fluid falling on both, with contacts at work every step (the
    host World's contact count says so).  The server runs World's rigid
    pipeline on the device for it (pbf_server_open_coupled_scene_contacts);
    a scene of free bodies shares the batch."""
    import novaphy_gb300 as nv

    mb = nv.ModelBuilder()
    mb.add_ground_plane(y=0.0)
    a = mb.add_body(nv.RigidBody.from_sphere(2.0, 0.1),
                    nv.Transform.from_translation(np.array([0.5, 0.098, 0.5], np.float32)))
    mb.add_shape(nv.CollisionShape.make_sphere(0.1, a))
    b = mb.add_body(nv.RigidBody.from_sphere(1.0, 0.08),
                    nv.Transform.from_translation(np.array([0.67, 0.085, 0.52], np.float32)))
    mb.add_shape(nv.CollisionShape.make_sphere(0.08, b))
    model = mb.build()
    pbf = nv.PBFSettings()
    pbf.kernel_radius = 0.2
    pbf.solver_iterations = 2
    blk = nv.FluidBlockDef()
    blk.lower = np.array([0.35, 0.25, 0.35], np.float32)
    blk.upper = np.array([0.75, 0.5, 0.7], np.float32)
    blk.particle_spacing = 0.05
    fw = nv.FluidWorld(model, [blk], nv.SolverSettings(), pbf, boundary_extent=1.0)
    x0 = fw.fluid_state.positions_array.copy()
    v0 = fw.fluid_state.velocities_array.copy()
    bps = fw.boundary_particles
    local = np.stack([bp.local_position for bp in bps]).astype(np.float32)
    body = np.array([bp.body_index for bp in bps], np.int32)
    psi = np.array([bp.volume for bp in bps], np.float32)
    bodies = []
    for k, rb in enumerate(model.bodies):
        tr = model.initial_transforms[k]
        q = np.asarray(tr.rotation, np.float32)  # x, y, z, w
        rbc = capi.RigidBody()
        rbc.pos[:] = [float(c) for c in tr.position]
        rbc.quat[:] = [float(q[3]), float(q[0]), float(q[1]), float(q[2])]
        rbc.inv_mass = rb.inv_mass()
        rbc.inv_inertia[:] = rb.inv_inertia()
        bodies.append(rbc)
    st = capi.Settings()
    for name, _ in capi.Settings._fields_:
        val = getattr(fw.pbf_settings, name)
        if name in ("domain_lower", "domain_upper"):
            getattr(st, name)[:] = [float(c) for c in val]
        else:
            setattr(st, name, val)
    mass = fw.pbf_settings.particle_mass(0.05)
    g = [0.0, -9.81, 0.0]
    dt = float(np.float32(1 / 60))
    nsteps = 6

    other = small_scenes(k=1, seed=29)[0]
    srv = capi.Server(capi.server_config(min_step_particles=0))
    oid, _ = srv.open_scene(settings_of(other), other.x, other.v, other.mass, other.gravity)
    sid, state = srv.open_coupled_scene(st, x0, v0, mass, g, local, body, psi, bodies,
                                        shapes=served_shapes_of(model))
    assert state == capi.SCENE_RESIDENT
    qo = srv.submit(oid, other.dt, nsteps)
    qs = srv.submit(sid, dt, nsteps)
    assert srv.wait(qs) == capi.REQ_DONE and srv.wait(qo) == capi.REQ_DONE
    kinds = set()
    for _ in range(nsteps):
        fw.step(dt)
        cs = fw.contacts
        assert len(cs) >= 2, "the sphere rests on the plane and touches the other sphere"
        kinds |= {(c.body_a, c.body_b) for c in cs}
    assert (-1, 0) in kinds and (0, 1) in kinds
    fs = fw.fluid_state
    for got, want in ((srv.read(sid, capi.FIELD_POSITIONS, len(x0)), fs.positions_array),
                      (srv.read(sid, capi.FIELD_VELOCITIES, len(x0)), fs.velocities_array),
                      (srv.read(sid, capi.FIELD_DENSITIES, len(x0)), fs.densities_array)):
        assert np.array_equal(got.view(np.uint32), np.asarray(want, np.float32).view(np.uint32))
    out = srv.read_bodies(sid, len(bodies))
    for k, rb in enumerate(out):
        tr = fw.state.transforms[k]
        q = np.asarray(tr.rotation, np.float32)
        assert np.array_equal(np.array(rb.pos, np.float32), np.asarray(tr.position, np.float32)), k
        assert np.array_equal(np.array(rb.quat, np.float32), q[[3, 0, 1, 2]]), k
        assert np.array_equal(np.array(rb.lin_vel, np.float32),
                              np.asarray(fw.state.linear_velocities[k], np.float32)), k
        assert np.array_equal(np.array(rb.ang_vel, np.float32),
                              np.asarray(fw.state.angular_velocities[k], np.float32)), k
    # The sphere on the plane stays on it (the contact holds it up).
    assert out[0].pos[1] > 0.09
    srv.close()


def test_served_contacts_reject_unsupported_shapes():
    w = small_scenes(k=1, seed=30)[0]
    rb = capi.RigidBody()
    rb.quat[:] = [1.0, 0.0, 0.0, 0.0]
    rb.inv_mass = 1.0
    rb.inv_inertia[:] = [1, 0, 0, 0, 1, 0, 0, 0, 1]
    bad = capi.RigidShape()
    bad.type = 7
    bad.body = 0
    missing = capi.RigidShape()
    missing.type = capi.SHAPE_SPHERE
    missing.body = 3
    srv = capi.Server()
    for sh in (bad, missing):
        with pytest.raises(capi.PbfError):
            srv.open_coupled_scene(settings_of(w), w.x, w.v, w.mass, w.gravity,
                                   np.zeros((1, 3), np.float32), np.zeros(1, np.int32),
                                   np.ones(1, np.float32), [rb], shapes=[sh])
    srv.close()
