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
  refuse it.
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
