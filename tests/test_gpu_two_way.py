"""Two-way Akinci coupling (pbf_settings.boundary_two_way, off by default): the
boundary particles of a coupled scene enter the fluid's density constraint in
every Jacobi iteration of pbf_scene_step_coupled, so the fluid is held off the
bodies.  The reference has no counterpart (its boundary pushes the bodies and
never the fluid, src/fluid/fluid_world.cpp:68-79), so there is no reference
output to match; the tests pin what the extension must keep:

* with every boundary volume psi at zero the boundary terms are exact zeros,
  and the two-way step equals the reference's one-way step bit for bit (fluid
  state, force and torque): the extension adds nothing but its terms;
* a fluid block dropped on a static box is held off it with two-way
  coupling and falls through it with the reference's one-way coupling;
* it is deterministic;
* batches and the serving loop, which step the fluid without its boundary,
  refuse it;
* boundary friction (pbf_settings.boundary_friction): zero is a no-op; a
  positive coefficient drags the fluid along a moving or spinning body's
  surface and slows fluid sliding over still boundaries.
"""
import numpy as np
import pytest

from novaphy_gb300 import capi, workloads

pytestmark = pytest.mark.gpu

R = 0.025
HALF = np.array([0.2, 0.2, 0.1], np.float32)
BOX_POS = np.array([[0.5, 0.5, 0.15]], np.float32)
IDENT = np.array([1, 0, 0, 0], np.float32)


def box_scene(port, two_way, psi_scale=1.0, **kw):
    """A 8 x 8 x 6 block at spacing R above a static box (half extents HALF) in [0,1]^3."""
    w = workloads.dam_break((8, 8, 6), R, (1.0, 1.0, 1.0), dt=1.0 / 120.0, seed=0, vorticity=0.0)
    w.x = (w.x + np.array([0.4, 0.4, 0.35], np.float32)).astype(np.float32)
    local = port.sample_box(HALF, (0, 0, 0), IDENT, np.float32(R)).astype(np.float32)
    body = np.zeros(len(local), np.int32)
    world0 = port.boundary_world_positions(local, body, BOX_POS, IDENT[None])
    psi = (port.boundary_volumes(world0, np.float32(4 * R)) * np.float32(psi_scale)).astype(np.float32)
    st = dict(w.settings, boundary_two_way=two_way, corr_k=0.001, corr_delta_q=0.3)
    st.update(kw)
    sc = capi.Scene(capi.default_settings(**st), w.x, w.v, mass=w.mass)
    sc.set_gravity(w.gravity)
    sc.set_boundary(local, body, psi)
    sc.set_bodies(BOX_POS, IDENT[None], np.array([0], np.int32))
    return w, sc


def run(sc, w, nsteps):
    f0 = np.zeros((1, 3), np.float32)
    ft = []
    for _ in range(nsteps):
        ft.append(sc.step_coupled(w.dt, f0, f0))
    return sc.state(), ft


def inside_box(x):
    return (np.abs(x - BOX_POS[0]) < HALF - R / 2).all(1)


@pytest.mark.parametrize("exact", [1, 0])
def test_two_way_with_zero_volumes_equals_one_way(port, exact):
    states = []
    for tw in (0, 1):
        w, sc = box_scene(port, tw, psi_scale=0.0, exact_arithmetic=exact)
        states.append(run(sc, w, 6))
        sc.close()
    (a, fa), (b, fb) = states
    for u, v in zip(a, b):
        assert np.array_equal(u.view(np.uint32), v.view(np.uint32))
    for (f1, t1), (f2, t2) in zip(fa, fb):
        assert np.array_equal(f1, f2) and np.array_equal(t1, t2)


def test_two_way_holds_the_fluid_off_a_static_box(port):
    """Sampled every 15 steps over 90: with one-way coupling most of the block
    passes through the box on its way to the floor; with two-way coupling the
    boundary's density term holds it off (the constraint is soft, so a few
    fast particles dip in: at most 8 % at any sample)."""
    peaks = {}
    for tw in (0, 1):
        w, sc = box_scene(port, tw)
        f0 = np.zeros((1, 3), np.float32)
        counts = []
        for k in range(90):
            sc.step_coupled(w.dt, f0, f0)
            if k % 15 == 14:
                x = sc.state()[0]
                assert np.isfinite(x).all()
                counts.append(int(inside_box(x).sum()))
        peaks[tw] = max(counts)
        sc.close()
    assert peaks[0] > w.n // 2, peaks        # one-way: the block falls through the box
    assert peaks[1] <= 0.08 * w.n, peaks     # two-way: held off


def test_two_way_is_deterministic(port):
    runs = []
    for _ in range(2):
        w, sc = box_scene(port, 1)
        runs.append(run(sc, w, 20)[0])
        sc.close()
    for u, v in zip(*runs):
        assert np.array_equal(u.view(np.uint32), v.view(np.uint32))


def test_batches_and_servers_refuse_two_way(port):
    w, sc = box_scene(port, 1)
    b = capi.Batch()
    with pytest.raises(capi.PbfError):
        b.step([sc], [w.dt])
    b.close()
    sc.close()
    srv = capi.Server()
    with pytest.raises(capi.PbfError):
        srv.open_scene(capi.default_settings(**dict(w.settings, boundary_two_way=1)), w.x, w.v,
                       w.mass, w.gravity)
    srv.close()


@pytest.mark.parametrize("monitor", [False, True])
def test_fluid_world_two_way(monitor):
    """PBFSettings.boundary_two_way through FluidWorld: a block dropped on a
    static box is held off it; with the performance monitor on, the world
    still steps through the whole coupled step (the profiled phases cannot
    split a two-way step) and gives the same bits."""
    import novaphy_gb300 as nv

    def world(two_way, mon):
        mb = nv.ModelBuilder()
        bi = mb.add_body(nv.RigidBody.make_static(),
                         nv.Transform.from_translation(np.array([0.5, 0.5, 0.15], np.float32)))
        mb.add_shape(nv.CollisionShape.make_box(np.array([0.2, 0.2, 0.1], np.float32), bi))
        blk = nv.FluidBlockDef()
        blk.lower = np.array([0.4125, 0.4125, 0.3625], np.float32)
        blk.upper = np.array([0.5875, 0.5875, 0.5], np.float32)
        blk.particle_spacing = R
        st = nv.PBFSettings()
        st.kernel_radius = 4 * R
        st.use_domain_bounds = True
        st.domain_lower = [0.0, 0.0, 0.0]
        st.domain_upper = [1.0, 1.0, 1.0]
        st.particle_radius = R / 2
        st.boundary_two_way = two_way
        w = nv.FluidWorld(mb.build(), [blk], nv.SolverSettings(), st, 1.0)
        w.set_gravity([0.0, 0.0, -9.81])
        w.performance_monitor.enabled = mon
        return w

    peaks, finals = {}, {}
    for tw in (False, True):
        w = world(tw, monitor)
        counts = []
        for k in range(90):
            w.step(1.0 / 120.0)
            if k % 15 == 14:
                counts.append(int(inside_box(w.fluid_state.positions_array).sum()))
        peaks[tw] = max(counts)
        finals[tw] = w.fluid_arrays()["positions"].copy()
    n = len(finals[True])
    assert peaks[False] > n // 2, peaks
    assert peaks[True] <= 0.08 * n, peaks
    if monitor:
        w = world(True, False)
        for _ in range(90):
            w.step(1.0 / 120.0)
        assert np.array_equal(w.fluid_arrays()["positions"], finals[True])


# ---- boundary friction (pbf_settings.boundary_friction, two-way steps only) ----

def mean_velocity(sc):
    return sc.state()[1].mean(0)


def test_zero_friction_is_a_no_op(port):
    """boundary_friction = 0 launches nothing: body velocities do not matter."""
    runs = []
    for vel in (False, True):
        w, sc = box_scene(port, 1, boundary_friction=0.0)
        if vel:
            sc.set_body_velocities([[1.0, 0.0, 0.0]], [[0.0, 0.0, 3.0]])
        runs.append(run(sc, w, 20)[0])
        sc.close()
    for u, v in zip(*runs):
        assert np.array_equal(u.view(np.uint32), v.view(np.uint32))


def test_friction_drags_the_fluid_along_a_moving_surface(port):
    """The box stays put but its surface moves at 0.5 m/s in x (a conveyor):
    with friction the block resting on it picks up x momentum, short of the
    surface's speed on average, without it next to none (splashing particles
    move faster than the surface either way, so only means are compared)."""
    mean = {}
    for c in (0.0, 0.5):
        w, sc = box_scene(port, 1, boundary_friction=c)
        sc.set_body_velocities([[0.5, 0.0, 0.0]], [[0.0, 0.0, 0.0]])
        run(sc, w, 40)
        x, v = sc.state()[:2]
        assert np.isfinite(v).all()
        mean[c] = float(v[:, 0].mean())
        sc.close()
    assert abs(mean[0.0]) < 0.05, mean
    assert 0.2 < mean[0.5] < 0.5, mean


def test_friction_spins_the_fluid_on_a_spinning_body(port):
    """A box spinning about z (w = 2 rad/s) drags the fluid on its top into
    rotation: positive angular momentum about the box axis with friction,
    none without."""
    lz = {}
    for c in (0.0, 0.5):
        w, sc = box_scene(port, 1, boundary_friction=c)
        sc.set_body_velocities([[0.0, 0.0, 0.0]], [[0.0, 0.0, 2.0]])
        run(sc, w, 40)
        x, v = sc.state()[:2]
        d = x - BOX_POS[0]
        lz[c] = float((d[:, 0] * v[:, 1] - d[:, 1] * v[:, 0]).mean())
        sc.close()
    assert abs(lz[0.0]) < 5e-3, lz
    assert lz[0.5] > 0.015, lz


def test_friction_against_world_owned_particles(port):
    """World-owned boundary particles (body -1) have zero surface velocity:
    a block sliding over them at 0.5 m/s is slowed by friction."""
    mean = {}
    for c in (0.0, 0.5):
        w = workloads.dam_break((8, 8, 6), R, (1.0, 1.0, 1.0), dt=1.0 / 120.0, seed=0,
                                vorticity=0.0)
        w.x = (w.x + np.array([0.4, 0.4, 0.26], np.float32)).astype(np.float32)
        w.v[:, 0] = 0.5
        local = port.sample_box(HALF, (0, 0, 0), IDENT, np.float32(R)).astype(np.float32)
        world = (local + BOX_POS[0]).astype(np.float32)
        psi = port.boundary_volumes(world, np.float32(4 * R)).astype(np.float32)
        st = dict(w.settings, boundary_two_way=1, boundary_friction=c, corr_k=0.001,
                  corr_delta_q=0.3)
        sc = capi.Scene(capi.default_settings(**st), w.x, w.v, mass=w.mass)
        sc.set_gravity(w.gravity)
        sc.set_boundary(world, np.full(len(world), -1, np.int32), psi)
        f0 = np.zeros((0, 3), np.float32)
        for _ in range(20):
            sc.step_coupled(w.dt, f0, f0)
        v = sc.state()[1]
        assert np.isfinite(v).all()
        mean[c] = float(v[:, 0].mean())
        sc.close()
    assert mean[0.5] < mean[0.0] - 0.02, mean


def test_body_velocities_need_the_boundary_and_every_body(port):
    w = workloads.dam_break((4, 4, 4), R, (1.0, 1.0, 1.0), seed=0, vorticity=0.0)
    sc = capi.Scene(capi.default_settings(**w.settings), w.x, w.v, mass=w.mass)
    with pytest.raises(capi.PbfError):
        sc.set_body_velocities([[0.0, 0.0, 0.0]], [[0.0, 0.0, 0.0]])
    local = np.zeros((2, 3), np.float32)
    sc.set_boundary(local, np.array([0, 1], np.int32), np.ones(2, np.float32))
    with pytest.raises(capi.PbfError):
        sc.set_body_velocities([[0.0, 0.0, 0.0]], [[0.0, 0.0, 0.0]])
    sc.set_body_velocities(np.zeros((2, 3)), np.zeros((2, 3)))
    sc.close()


def test_fluid_world_friction_against_a_static_box():
    """PBFSettings.boundary_friction through FluidWorld: a block thrown over a
    static box at 0.5 m/s in x is slowed by the box's surface."""
    import novaphy_gb300 as nv

    mean = {}
    for c in (0.0, 0.5):
        mb = nv.ModelBuilder()
        bi = mb.add_body(nv.RigidBody.make_static(),
                         nv.Transform.from_translation(np.array([0.5, 0.5, 0.15], np.float32)))
        mb.add_shape(nv.CollisionShape.make_box(np.array([0.2, 0.2, 0.1], np.float32), bi))
        blk = nv.FluidBlockDef()
        blk.lower = np.array([0.4125, 0.4125, 0.2625], np.float32)
        blk.upper = np.array([0.5875, 0.5875, 0.4], np.float32)
        blk.particle_spacing = R
        blk.initial_velocity = np.array([0.5, 0.0, 0.0], np.float32)
        st = nv.PBFSettings()
        st.kernel_radius = 4 * R
        st.use_domain_bounds = True
        st.domain_lower = [0.0, 0.0, 0.0]
        st.domain_upper = [1.0, 1.0, 1.0]
        st.particle_radius = R / 2
        st.boundary_two_way = True
        st.boundary_friction = c
        w = nv.FluidWorld(mb.build(), [blk], nv.SolverSettings(), st, 1.0)
        w.set_gravity([0.0, 0.0, -9.81])
        for _ in range(20):
            w.step(1.0 / 120.0)
        v = w.fluid_arrays()["velocities"]
        assert np.isfinite(v).all()
        mean[c] = float(v[:, 0].mean())
    assert mean[0.5] < mean[0.0] - 0.02, mean
