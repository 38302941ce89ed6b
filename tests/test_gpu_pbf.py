"""GPU parity of the PBF step through the C ABI, against the oracle.

Bars (all FP32):
  * cell assignments and canonical neighbour sets: bit-exact;
  * exact_arithmetic = 1 (the default): x, v, rho, lambda bit-exact with the
    oracle after 1 and 10 steps (same operation order, no FMA, IEEE div/sqrt);
  * exact_arithmetic = 0 (FMA + rsqrt): after 1 step, per particle
    |dx| <= 1e-5 |x| + 1e-7 and |dv| <= 1e-5 |v| + V_ABS with V_ABS = 1e-4 m/s
    (v = (x* - x)/dt turns one float ulp of x* into ~1e-5 m/s at dt = 1/120);
    after 10 steps max |dx| <= 1e-3 h.  Checked with s_corr off: with the
    configured k = 0.1 a last-bit density change flips the reference's
    s_corr gate (see tests/test_oracle.py::test_configured_scorr_is_ill_conditioned),
    so only the exact build can match the reference there.
"""
import json
import os

import numpy as np
import pytest

from novaphy_gb300 import capi, workloads

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
V_ABS = 1e-4


def settings_of(w, **kw):
    st = dict(w.settings)
    st.update(kw)
    return capi.default_settings(**st)


def scene_of(w, **kw):
    sc = capi.Scene(settings_of(w, **kw), w.x, w.v, mass=w.mass)
    sc.set_gravity(w.gravity)
    return sc


def oracle_steps(port, w, nsteps, **kw):
    from oracle.oracle import Settings

    st = dict(w.settings)
    st.update({k: v for k, v in kw.items() if k not in ("exact_arithmetic", "hash_compat")})
    z = np.zeros(w.n, np.float32)
    return port.steps(Settings.make(**st), w.x, w.v, z, z, w.dt, w.gravity, w.mass, nsteps)


def assert_close_1step(got, want):
    x, v = got[0], want[0]
    dx = np.linalg.norm(got[0] - want[0], axis=1)
    assert (dx <= 1e-5 * np.linalg.norm(want[0], axis=1) + 1e-7).all(), dx.max()
    dv = np.linalg.norm(got[1] - want[1], axis=1)
    assert (dv <= 1e-5 * np.linalg.norm(want[1], axis=1) + V_ABS).all(), dv.max()


@pytest.mark.parametrize("n,bits", [(1, 8), (2047, 10), (2048, 12), (2049, 16), (100_000, 18),
                                    (1_000_003, 24), (300_000, 32)])
def test_sort_is_stable_and_sorted(n, bits):
    rng = np.random.default_rng(n)
    hi = (1 << bits) - 1
    keys = rng.integers(0, hi, n, dtype=np.uint64, endpoint=True).astype(np.uint32)
    if n > 1000:
        keys[: n // 3] = keys[0]  # long runs of equal keys exercise stability
    ko, vo = capi.sort_pairs(keys, bits)
    order = np.argsort(keys, kind="stable")
    assert np.array_equal(vo, order.astype(np.uint32))
    assert np.array_equal(ko, keys[order])


def test_sort_empty_is_noop():
    ko, vo = capi.sort_pairs(np.zeros(0, np.uint32), 8)
    assert len(ko) == 0 and len(vo) == 0


def test_cells_bit_exact(port):
    w = workloads.dam_break_8k()
    sc = scene_of(w)
    got = sc.debug_cells(w.dt)
    xs, _ = port.predict(w.x, w.v, w.dt, w.gravity)
    want = port.cell_coords(xs, np.float32(w.settings["kernel_radius"]))
    assert np.array_equal(got, want)


@pytest.mark.parametrize("hash_compat", [1, 0])
def test_neighbor_sets_bit_exact(port, hash_compat):
    w = workloads.dam_break_8k()
    sc = scene_of(w, hash_compat=hash_compat)
    offs, idx = sc.debug_neighbors(w.dt)
    xs, _ = port.predict(w.x, w.v, w.dt, w.gravity)
    o2, i2 = port.neighbor_sets(xs, np.float32(w.settings["kernel_radius"]))
    assert np.array_equal(offs, o2)
    assert np.array_equal(idx, i2)


@pytest.mark.parametrize("vort", [0.0, 1e-4])
def test_exact_mode_bit_exact_1_and_10_steps(port, vort):
    w = workloads.dam_break_8k(vorticity=vort)
    for nsteps in (1, 10):
        sc = scene_of(w, exact_arithmetic=1)
        sc.step(w.dt, nsteps)
        got = sc.state()
        want = oracle_steps(port, w, nsteps)
        for name, a, b in zip("x v rho lam".split(), got, want):
            assert np.array_equal(a, b), (nsteps, name, np.abs(a - b).max())


def test_exact_mode_matches_reference_fixture():
    g = np.load(os.path.join(GOLDEN, "block_1k.npz"))
    w = workloads.dam_break((10, 10, 10), 0.025, (1.0, 1.0, 1.0), dt=1.0 / 120.0, jitter=1e-4,
                            seed=0, vorticity=0.0)
    for k in (1, 5):
        sc = scene_of(w, exact_arithmetic=1)
        sc.step(w.dt, k)
        for name, a in zip(("x", "v", "rho", "lam"), sc.state()):
            assert np.array_equal(a, g[f"{name}{k}"]), (k, name)


def test_exact_mode_default_settings_fixture():
    # The reference tests' scene: PBFSettings defaults, no clamp, gravity -y.
    g = np.load(os.path.join(GOLDEN, "default_scene.npz"))
    s = capi.default_settings(exact_arithmetic=1)
    sc = capi.Scene(s, g["x0"], None, mass=float(np.float32(1000) * np.float32(0.025) ** 3))
    sc.set_gravity([0, -9.81, 0])
    sc.step(float(np.float32(1 / 60)), 1)
    for name, a in zip(("x1", "v1", "rho1", "lam1"), sc.state()):
        assert np.array_equal(a, g[name]), name


@pytest.mark.parametrize("vort", [0.0, 1e-4])
def test_fast_mode_tolerances(port, vort):
    w = workloads.dam_break_8k(vorticity=vort)
    w.settings["corr_k"] = 0.0
    sc = scene_of(w, exact_arithmetic=0)
    sc.step(w.dt, 1)
    assert_close_1step(sc.state(), oracle_steps(port, w, 1))
    sc = scene_of(w, exact_arithmetic=0)
    sc.step(w.dt, 10)
    want = oracle_steps(port, w, 10)
    h = w.settings["kernel_radius"]
    assert np.linalg.norm(sc.read(capi.FIELD_POSITIONS) - want[0], axis=1).max() <= 1e-3 * h


@pytest.mark.parametrize("kw", [
    dict(solver_iterations=0), dict(solver_iterations=1), dict(xsph_viscosity=0.0),
    dict(corr_n=2), dict(corr_k=0.0), dict(use_domain_bounds=0), dict(epsilon=1.0),
    dict(vorticity_epsilon=1e-3, xsph_viscosity=0.0),
])
def test_settings_variants_bit_exact(port, kw):
    w = workloads.dam_break((9, 7, 8), 0.025, (1.0, 1.0, 1.0), dt=1.0 / 120.0, seed=11,
                            vorticity=0.0)
    sc = scene_of(w, exact_arithmetic=1, **kw)
    sc.step(w.dt, 3)
    want = oracle_steps(port, w, 3, **kw)
    for name, a, b in zip("x v rho lam".split(), sc.state(), want):
        assert np.array_equal(a, b), (kw, name)


def test_far_from_axes_needs_no_slow_path(port):
    # Shifted block: no hash collisions, so hash_compat on/off agree exactly.
    w = workloads.dam_break((8, 8, 8), 0.025, (1.0, 1.0, 1.0), vorticity=0.0)
    shift = np.array([3.0, 5.0, 7.0], np.float32)
    w.x = (w.x + shift).astype(np.float32)
    w.settings["domain_lower"] = tuple(shift)
    w.settings["domain_upper"] = tuple(shift + 1.0)
    assert port.hash_collisions(w.x, np.float32(0.1)) == 0
    a = scene_of(w, exact_arithmetic=1, hash_compat=1)
    b = scene_of(w, exact_arithmetic=1, hash_compat=0)
    a.step(w.dt, 3)
    b.step(w.dt, 3)
    for u, t in zip(a.state(), b.state()):
        assert np.array_equal(u, t)


def test_tiny_and_empty_scenes(port):
    s = capi.default_settings(exact_arithmetic=1)
    sc = capi.Scene(s, np.zeros((0, 3), np.float32), None, mass=1.0)
    sc.step(0.01, 3)
    assert sc.n == 0
    x = np.array([[0.5, 0.5, 0.5]], np.float32)
    sc = capi.Scene(s, x, None, mass=0.125)
    sc.set_gravity([0, -9.81, 0])
    sc.step(np.float32(1 / 60), 2)
    from oracle.oracle import Settings

    z = np.zeros(1, np.float32)
    want = port.steps(Settings.make(), x, np.zeros_like(x), z, z, np.float32(1 / 60),
                      np.array([0, -9.81, 0], np.float32), 0.125, 2)
    for a, b in zip(sc.state(), want):
        assert np.array_equal(a, b)


def test_exact_mode_tracks_oracle_many_steps(port):
    # 30 consecutive steps of the configured (exploding) 8k dam break.
    w = workloads.dam_break_8k(vorticity=1e-4)
    sc = scene_of(w, exact_arithmetic=1)
    sc.step(w.dt, 30)
    want = oracle_steps(port, w, 30)
    for name, a, b in zip("x v rho lam".split(), sc.state(), want):
        assert np.array_equal(a, b), name


def test_solver_step_host_equals_scene_step():
    w = workloads.dam_break_8k()
    sc = scene_of(w)
    sc.step(w.dt, 1)
    ref = sc.state()
    drop = capi.Scene(settings_of(w), np.zeros((1, 3), np.float32), None, mass=w.mass)
    z = np.zeros(w.n, np.float32)
    got = drop.solver_step_host(w.x, w.v, z, z, w.dt, w.gravity, w.mass)
    for a, b in zip(got, ref):
        assert np.array_equal(a, b)


def test_deterministic_and_graph_replay_equal():
    w = workloads.dam_break_8k()
    a = scene_of(w)
    b = scene_of(w)
    a.step(w.dt, 5)
    for _ in range(5):
        b.step(w.dt, 1)
    for u, t in zip(a.state(), b.state()):
        assert np.array_equal(u, t)


def test_profiled_step_equals_plain_step():
    w = workloads.dam_break_8k()
    a = scene_of(w)
    b = scene_of(w)
    a.step(w.dt, 1)
    ph = b.step_profiled(w.dt)
    assert set(ph) >= {"fluid.pbf.predict", "fluid.pbf.iteration.compute_density"}
    assert ph["fluid.pbf.iteration.compute_delta_position"][1] >= 4
    for u, t in zip(a.state(), b.state()):
        assert np.array_equal(u, t)


@pytest.mark.parametrize("exact", [1, 0])
def test_million_particle_properties(exact):
    # Size-independent properties at the full 1M size: determinism (two runs
    # bit-identical), clamp bounds, finiteness; with s_corr off the fluid
    # falls under gravity.
    w = workloads.dam_break_1m()
    a = scene_of(w, exact_arithmetic=exact)
    b = scene_of(w, exact_arithmetic=exact)
    a.step(w.dt, 3)
    b.step(w.dt, 3)
    xa, xb = a.read(capi.FIELD_POSITIONS), b.read(capi.FIELD_POSITIONS)
    assert np.array_equal(xa, xb)
    assert a.check_finite() == capi.PBF_OK
    lo = np.float32(w.settings["particle_radius"])
    hi = np.array(w.settings["domain_upper"], np.float32) - lo
    assert (xa >= lo).all() and (xa <= hi).all()
    rho = a.read(capi.FIELD_DENSITIES)
    assert np.isfinite(rho).all() and rho.max() > 500.0
    w.settings["corr_k"] = 0.0
    c = scene_of(w, exact_arithmetic=exact)
    c.step(w.dt, 3)
    assert c.read(capi.FIELD_POSITIONS)[:, 2].mean() < w.x[:, 2].mean()


def test_nonfinite_input_is_detected():
    w = workloads.dam_break((4, 4, 4), 0.025, (1.0, 1.0, 1.0))
    x = w.x.copy()
    x[5, 1] = np.nan
    sc = capi.Scene(settings_of(w), x, None, mass=w.mass)
    assert sc.check_finite() == capi.PBF_ERR_NONFINITE


def test_snapshot_resume_is_bit_identical():
    # k steps, snapshot, m steps == k + m steps (checkpoint / resume).
    w = workloads.dam_break_8k()
    a = scene_of(w)
    a.step(w.dt, 7)
    b = scene_of(w)
    b.step(w.dt, 3)
    snap = b.snapshot()
    b.step(w.dt, 2)           # diverge, then resume from the snapshot
    b.restore(snap)
    b.step(w.dt, 4)
    for u, t in zip(a.state(), b.state()):
        assert np.array_equal(u, t)
    # restoring into a fresh scene of another size resizes it
    c = capi.Scene(settings_of(w), np.zeros((5, 3), np.float32), None, mass=1.0)
    c.restore(snap)
    assert c.n == w.n
    c.step(w.dt, 4)
    for u, t in zip(a.state(), c.state()):
        assert np.array_equal(u, t)


def test_replay_timed_restores_each_step():
    w = workloads.dam_break_8k()
    a = scene_of(w)
    seed = a.snapshot()
    ms = a.replay_timed(seed, w.dt, 3)
    assert ms > 0
    b = scene_of(w)
    b.step(w.dt, 1)
    for u, t in zip(a.state(), b.state()):
        assert np.array_equal(u, t)


def test_solver_step_host_on_page_locked_arrays():
    """pbf_solver_step_host on page-locked arrays (capi.pinned_empty, updated in
    place) gives the bits of the same call on pageable arrays, for sizes that
    are not a multiple of the block and across changes of n."""
    for counts in ((20, 20, 20), (12, 11, 7), (13, 11, 7)):
        w = workloads.dam_break(counts, 0.025, (1.0, 1.0, 1.0), seed=3)
        drop = capi.Scene(settings_of(w), np.zeros((1, 3), np.float32), None, mass=w.mass)
        z = np.zeros(w.n, np.float32)
        want = drop.solver_step_host(w.x, w.v, z, z, w.dt, w.gravity, w.mass)
        hx, hv = capi.pinned_empty((w.n, 3)), capi.pinned_empty((w.n, 3))
        hr, hl = capi.pinned_empty((w.n,)), capi.pinned_empty((w.n,))
        for _ in range(2):
            hx[:] = w.x
            hv[:] = w.v
            hr[:] = 0
            hl[:] = 0
            capi.solver_step_host_inplace(drop, hx, hv, hr, hl, w.dt, w.gravity, w.mass)
            for a, b in zip((hx, hv, hr, hl), want):
                assert np.array_equal(a.view(np.uint32), b.view(np.uint32))
        drop.close()
