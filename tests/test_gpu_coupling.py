"""GPU parity of the Akinci rigid-fluid coupling (FluidWorld's fluid part)
against the oracle, bit-exact: boundary world positions, Akinci volumes,
boundary density added to the fluid densities, and the per-body coupling
force / torque accumulated in boundary order onto the caller's totals."""
import numpy as np
import pytest

from novaphy_gb300 import capi, workloads

pytestmark = pytest.mark.gpu


def quat_z(deg):
    a = np.deg2rad(deg) / 2
    return np.array([np.cos(a), 0.0, 0.0, np.sin(a)], np.float32)


def coupled_scene(port):
    """1000-particle block in the corner of [0,1]^3, a submerged dynamic sphere,
    a static rotated box touching the fluid and a world-owned floor plane."""
    w = workloads.dam_break((10, 10, 10), 0.025, (1.0, 1.0, 1.0), dt=1.0 / 120.0, seed=0,
                            vorticity=0.0)
    sp = np.float32(0.025)
    ident = np.array([1, 0, 0, 0], np.float32)
    sph = port.sample_sphere(0.06, (0, 0, 0), ident, sp)
    box = port.sample_box([0.05, 0.05, 0.05], (0, 0, 0), ident, sp)
    pln = port.sample_plane([0, 0, 1], 0.0, sp, 0.5)
    local = np.concatenate([sph, box, pln]).astype(np.float32)
    body = np.concatenate([np.zeros(len(sph)), np.ones(len(box)), -np.ones(len(pln))]).astype(np.int32)
    body_pos = np.array([[0.12, 0.12, 0.12], [0.27, 0.1, 0.1]], np.float32)
    body_quat = np.stack([ident, quat_z(30.0)]).astype(np.float32)
    dynamic = np.array([1, 0], np.int32)
    world0 = port.boundary_world_positions(local, body, body_pos, body_quat)
    psi = port.boundary_volumes(world0, np.float32(w.settings["kernel_radius"]))
    return w, local, body, psi, body_pos, body_quat, dynamic, world0


def test_boundary_volumes_bit_exact(port):
    w, local, body, psi, bp, bq, dyn, world0 = coupled_scene(port)
    got = capi.boundary_volumes(world0, w.settings["kernel_radius"])
    assert np.array_equal(got, psi)


def test_coupled_step_bit_exact(port):
    from oracle.oracle import Settings

    w, local, body, psi, bp, bq, dyn, world0 = coupled_scene(port)
    h = np.float32(w.settings["kernel_radius"])
    f0 = np.array([[0.1, -0.2, 0.3], [0.0, 0.0, 0.0]], np.float32)
    t0 = np.array([[0.01, 0.02, -0.03], [0.0, 0.0, 0.0]], np.float32)
    sc = capi.Scene(capi.default_settings(**w.settings, exact_arithmetic=1), w.x, w.v, mass=w.mass)
    sc.set_gravity(w.gravity)
    sc.set_boundary(local, body, psi)
    sc.set_bodies(bp, bq, dyn)
    f, t = sc.step_coupled(w.dt, f0, t0)
    x, v, rho, lam = sc.state()
    assert np.array_equal(sc.read_boundary(), world0)
    # oracle: PBF step, boundary density on the final x, coupling forces
    z = np.zeros(w.n, np.float32)
    ox, ov, orho, olam = port.steps(Settings.make(**w.settings), w.x, w.v, z, z, w.dt, w.gravity,
                                    w.mass, 1)
    assert np.array_equal(x, ox) and np.array_equal(v, ov) and np.array_equal(lam, olam)
    orho = port.boundary_density(ox, orho, world0, psi, h, np.float32(1000.0))
    assert np.array_equal(rho, orho)
    assert (rho > port.steps(Settings.make(**w.settings), w.x, w.v, z, z, w.dt, w.gravity,
                             w.mass, 1)[2]).any()
    rf, rt = port.coupling_forces(ox, orho, w.mass, world0, body, psi, dyn, bp, h,
                                  np.float32(1000.0))
    assert np.abs(rf[0]).sum() > 0, "the sphere sits in the fluid and must feel a force"
    assert (rf[1] == 0).all(), "static bodies get no coupling force"
    want_f, want_t = port_coupling_accumulated(port, ox, orho, w.mass, world0, body, psi, dyn,
                                               bp, h, f0, t0)
    assert np.array_equal(f, want_f)
    assert np.array_equal(t, want_t)


def port_coupling_accumulated(port, x, rho, mass, bpos, body, psi, dyn, body_pos, h, f0, t0):
    """orc_coupling_forces accumulating onto given totals (like World::apply_force)."""
    import ctypes as C

    f = np.ascontiguousarray(f0, np.float32).copy()
    t = np.ascontiguousarray(t0, np.float32).copy()
    rc = port.lib.orc_coupling_forces(
        len(x), np.ascontiguousarray(x, np.float32), np.ascontiguousarray(rho, np.float32),
        C.c_float(mass), len(bpos), np.ascontiguousarray(bpos, np.float32),
        np.ascontiguousarray(body, np.int32), np.ascontiguousarray(psi, np.float32),
        len(body_pos), np.ascontiguousarray(dyn, np.int32),
        np.ascontiguousarray(body_pos, np.float32), C.c_float(h), C.c_float(1000.0), f, t)
    assert rc == 0
    return f, t


def test_coupled_step_without_boundary_is_plain_step():
    w = workloads.dam_break((8, 8, 8), 0.025, (1.0, 1.0, 1.0), vorticity=0.0)
    a = capi.Scene(capi.default_settings(**w.settings), w.x, w.v, mass=w.mass)
    b = capi.Scene(capi.default_settings(**w.settings), w.x, w.v, mass=w.mass)
    for s in (a, b):
        s.set_gravity(w.gravity)
    a.step(w.dt, 1)
    b.step_coupled(w.dt, np.zeros((0, 3), np.float32), np.zeros((0, 3), np.float32))
    for u, v in zip(a.state(), b.state()):
        assert np.array_equal(u, v)


def test_batched_step_then_couple_equals_coupled_step(port):
    """Coupled worlds stepped together: one batch step of their fluids, then
    each world's coupling (pbf_scene_couple) gives the bits of its own
    pbf_scene_step_coupled, with a plain scene in the same batch."""
    w, local, body, psi, bp, bq, dyn, world0 = coupled_scene(port)
    f0 = np.array([[0.1, -0.2, 0.3], [0.0, 0.0, 0.0]], np.float32)
    t0 = np.array([[0.01, 0.02, -0.03], [0.0, 0.0, 0.0]], np.float32)

    def make():
        sc = capi.Scene(capi.default_settings(**w.settings), w.x, w.v, mass=w.mass)
        sc.set_gravity(w.gravity)
        sc.set_boundary(local, body, psi)
        sc.set_bodies(bp, bq, dyn)
        return sc

    ref = make()
    rf, rt = f0, t0
    for _ in range(2):
        rf, rt = ref.step_coupled(w.dt, rf, rt)
    other_w = workloads.batched_scenes(nscenes=1, seed=4, n_lo=800, n_hi=1200)[0]
    other = capi.Scene(capi.default_settings(**other_w.settings), other_w.x, other_w.v,
                       mass=other_w.mass)
    other.set_gravity(other_w.gravity)
    sc = make()
    b = capi.Batch()
    f, t = f0, t0
    for _ in range(2):
        b.step([other, sc], [other_w.dt, w.dt])
        f, t = sc.couple(w.dt, f, t)
    for a, c in zip(ref.state(), sc.state()):
        assert np.array_equal(a.view(np.uint32), c.view(np.uint32))
    assert np.array_equal(f, rf) and np.array_equal(t, rt)


@pytest.mark.parametrize("radius,spacing", [(0.06, 0.025), (0.1, 0.008)])
def test_fast_build_tree_wrench_within_its_bound(port, radius, spacing):
    """The fast build reduces each body's coupling terms as a deterministic
    segmented tree instead of the reference's serial sum.  Per component the
    two sums of a body's m terms differ by at most 2 (m - 1) 2^-24 sum |term|;
    the terms themselves are the oracle's, one boundary particle at a time.
    The boundary density stays bit-exact, and two runs give the same bits."""
    w = workloads.dam_break((10, 10, 10), 0.025, (1.0, 1.0, 1.0), dt=1.0 / 120.0, seed=0,
                            vorticity=0.0)
    ident = np.array([1, 0, 0, 0], np.float32)
    local = port.sample_sphere(radius, (0, 0, 0), ident, np.float32(spacing)).astype(np.float32)
    body = np.zeros(len(local), np.int32)
    bp = np.array([[0.12, 0.12, 0.12]], np.float32)
    bq = ident[None, :]
    dyn = np.array([1], np.int32)
    h = np.float32(w.settings["kernel_radius"])
    world0 = port.boundary_world_positions(local, body, bp, bq)
    psi = port.boundary_volumes(world0, h)
    f0 = np.array([[0.1, -0.2, 0.3]], np.float32)
    t0 = np.array([[0.01, 0.02, -0.03]], np.float32)
    runs = []
    for _ in range(2):
        sc = capi.Scene(capi.default_settings(**w.settings, exact_arithmetic=0), w.x, w.v,
                        mass=w.mass)
        sc.set_gravity(w.gravity)
        sc.set_boundary(local, body, psi)
        sc.set_bodies(bp, bq, dyn)
        sc.step(w.dt, 1)
        x, _, rho_pre, _ = sc.state()
        f, t = sc.couple(w.dt, f0, t0)
        runs.append((x, rho_pre, sc.state()[2], f, t))
        sc.close()
    x, rho_pre, rho, f, t = runs[0]
    assert all(np.array_equal(a, b) for a, b in zip(runs[0], runs[1])), "not deterministic"
    rho_b = port.boundary_density(x, rho_pre, world0, psi, h, np.float32(1000.0))
    assert np.array_equal(rho, rho_b)
    want_f, want_t = port_coupling_accumulated(port, x, rho_b, w.mass, world0, body, psi, dyn,
                                               bp, h, f0, t0)
    terms_f, terms_t = [], []
    for b in range(len(local)):
        tf, tt = port.coupling_forces(x, rho_b, w.mass, world0[b:b + 1], body[b:b + 1],
                                      psi[b:b + 1], dyn, bp, h, np.float32(1000.0))
        terms_f.append(tf[0])
        terms_t.append(tt[0])
    terms_f, terms_t = np.array(terms_f, np.float64), np.array(terms_t, np.float64)
    m = int((np.abs(terms_f).sum(1) > 0).sum())
    assert m > 10, "the sphere must sit in the fluid"
    u = 2.0 ** -24
    tol_f = 2 * (m + 1) * u * (np.abs(terms_f).sum(0) + np.abs(f0[0]))
    tol_t = 2 * (m + 1) * u * (np.abs(terms_t).sum(0) + np.abs(t0[0]))
    assert (np.abs(f[0].astype(np.float64) - want_f[0]) <= tol_f).all(), (f, want_f, tol_f)
    assert (np.abs(t[0].astype(np.float64) - want_t[0]) <= tol_t).all(), (t, want_t, tol_t)
