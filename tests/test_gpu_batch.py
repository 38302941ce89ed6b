"""Batched stepping (pbf_batch_*) against stepping each scene alone.

A scene stepped inside a batch must end bit for bit where pbf_scene_step
leaves it (same sorts, candidate order and arithmetic; per-scene settings,
gravity, mass, dt and iteration counts from the batch's table), whatever else
is in the batch.  The single-scene path is itself bit-exact with the oracle
(tests/test_gpu_pbf.py), and one scene is checked against the oracle here
directly.  The fast build (exact_arithmetic = 0) may contract the batched
and single-scene kernel instances differently, so it is held to 1e-3 h after
two steps with s_corr off (with the configured k = 0.1 the step is
ill-conditioned; see tests/test_oracle.py).
"""
import numpy as np
import pytest

from novaphy_gb300 import capi, workloads

pytestmark = pytest.mark.gpu


def make_scene(w, **kw):
    st = dict(w.settings)
    st.update(kw)
    sc = capi.Scene(capi.default_settings(**st), w.x, w.v, mass=w.mass)
    sc.set_gravity(w.gravity)
    return sc


def state(sc):
    return [sc.read(f) for f in (capi.FIELD_POSITIONS, capi.FIELD_VELOCITIES,
                                 capi.FIELD_DENSITIES, capi.FIELD_LAMBDAS)]


def assert_same(a, b, what=""):
    for k, (x, y) in enumerate(zip(a, b)):
        assert np.array_equal(x.view(np.uint32), y.view(np.uint32)), (what, k,
                                                                      np.abs(x - y).max())


def mixed_scenes():
    """Small scenes with different sizes, settings, gravity and dt."""
    ws = workloads.batched_scenes(nscenes=6, seed=11, n_lo=300, n_hi=4000)
    variants = [
        dict(),
        dict(solver_iterations=0),
        dict(vorticity_epsilon=0.0, xsph_viscosity=0.0),
        dict(hash_compat=0),
        dict(use_domain_bounds=0, corr_k=0.0),
        dict(solver_iterations=7, corr_n=2),
    ]
    return ws, variants


def test_batch_equals_scenes_alone():
    ws, variants = mixed_scenes()
    dts = [w.dt * (1.0 + 0.25 * k) for k, w in enumerate(ws)]
    alone = [make_scene(w, **kw) for w, kw in zip(ws, variants)]
    inbatch = [make_scene(w, **kw) for w, kw in zip(ws, variants)]
    alone[0].set_gravity([0.0, -9.81, 0.0])
    inbatch[0].set_gravity([0.0, -9.81, 0.0])
    for sc, dt in zip(alone, dts):
        sc.step(np.float32(dt), 3)
    b = capi.Batch()
    for _ in range(3):
        b.step(inbatch, np.asarray(dts, np.float32))
    for k, (a, c) in enumerate(zip(alone, inbatch)):
        assert_same(state(a), state(c), f"scene {k} {variants[k]}")


def test_batch_matches_oracle(port):
    from oracle.oracle import Settings

    ws = workloads.batched_scenes(nscenes=3, seed=5, n_lo=500, n_hi=3000)
    scenes = [make_scene(w) for w in ws]
    b = capi.Batch()
    b.step(scenes, ws[0].dt, nsteps=2)
    for w, sc in zip(ws, scenes):
        z = np.zeros(w.n, np.float32)
        want = port.steps(Settings.make(**w.settings), w.x, w.v, z, z, w.dt, w.gravity, w.mass, 2)
        got = state(sc)
        for k in range(4):
            assert np.array_equal(got[k].view(np.uint32), np.asarray(want[k], np.float32).view(
                np.uint32)), (w.name, k)


def test_per_scene_step_counts_and_empty_scenes():
    ws, variants = mixed_scenes()
    steps = [0, 1, 2, 3, 1, 2]
    alone = [make_scene(w, **kw) for w, kw in zip(ws, variants)]
    inbatch = [make_scene(w, **kw) for w, kw in zip(ws, variants)]
    empty = capi.Scene(capi.default_settings(), np.zeros((0, 3), np.float32))
    for sc, m, w in zip(alone, steps, ws):
        sc.step(w.dt, m)
    b = capi.Batch()
    b.step(inbatch + [empty], [w.dt for w in ws] + [ws[0].dt], nsteps=steps + [5])
    for k, (a, c) in enumerate(zip(alone, inbatch)):
        assert_same(state(a), state(c), f"scene {k}")


def test_result_independent_of_batch_composition():
    ws = workloads.batched_scenes(nscenes=5, seed=21, n_lo=500, n_hi=5000)
    b = capi.Batch()
    solo = make_scene(ws[2])
    b.step([solo], ws[2].dt, nsteps=2)
    mix = [make_scene(w) for w in ws]
    b.step(list(reversed(mix)), ws[0].dt, nsteps=2)
    assert_same(state(solo), state(mix[2]))


def test_fast_build_batched_equals_alone():
    ws, variants = mixed_scenes()
    variants = [dict(kw, corr_k=0.0) for kw in variants]
    alone = [make_scene(w, exact_arithmetic=0, **kw) for w, kw in zip(ws, variants)]
    inbatch = [make_scene(w, exact_arithmetic=0, **kw) for w, kw in zip(ws, variants)]
    for sc, w in zip(alone, ws):
        sc.step(w.dt, 2)
    b = capi.Batch()
    b.step(inbatch, [w.dt for w in ws], nsteps=2)
    for k, (a, c) in enumerate(zip(alone, inbatch)):
        x0, x1 = state(a)[0], state(c)[0]
        assert np.abs(x0 - x1).max() <= 1e-3 * ws[k].settings["kernel_radius"], k


def test_mixed_exact_and_fast_scenes():
    ws, _ = mixed_scenes()
    flags = [1, 0, 1, 0, 1, 0]
    alone = [make_scene(w, exact_arithmetic=f) for w, f in zip(ws, flags)]
    inbatch = [make_scene(w, exact_arithmetic=f) for w, f in zip(ws, flags)]
    for sc, w in zip(alone, ws):
        sc.step(w.dt, 2)
    b = capi.Batch()
    b.step(inbatch, [w.dt for w in ws], nsteps=2)
    for k in range(len(ws)):
        if flags[k]:
            assert_same(state(alone[k]), state(inbatch[k]), f"scene {k}")


def test_scene_ops_are_ordered_after_the_batch():
    w = workloads.batched_scenes(nscenes=1, seed=8, n_lo=2000, n_hi=2001)[0]
    a, c = make_scene(w), make_scene(w)
    b = capi.Batch()
    b.step([c], w.dt, sync=False)  # no host wait: the read must still see the step
    c.step(w.dt, 1, sync=False)
    a.step(w.dt, 2)
    assert_same(state(a), state(c))


def test_replay_timed_and_graph_reuse():
    ws = workloads.batched_scenes(nscenes=4, seed=2, n_lo=1000, n_hi=4000)
    scenes = [make_scene(w) for w in ws]
    seeds = [sc.snapshot() for sc in scenes]
    ref = [make_scene(w) for w in ws]
    for sc, w in zip(ref, ws):
        sc.step(w.dt, 1)
    b = capi.Batch()
    ms = b.replay_timed(scenes, seeds, ws[0].dt, 3)
    assert ms > 0.0
    for a, c in zip(ref, scenes):
        assert_same(state(a), state(c))
    assert b.device_bytes() > 0


def test_invalid_batches():
    w = workloads.batched_scenes(nscenes=1, seed=8, n_lo=500, n_hi=501)[0]
    sc = make_scene(w)
    b = capi.Batch()
    with pytest.raises(capi.PbfError) as e:
        b.step([sc, sc], w.dt)
    assert e.value.code == capi.PBF_ERR_INVALID_ARG
    with pytest.raises(capi.PbfError) as e:
        b.step([sc], 0.0)
    assert e.value.code == capi.PBF_ERR_INVALID_ARG
    with pytest.raises(capi.PbfError) as e:
        b.step([sc], w.dt, nsteps=[-1])
    assert e.value.code == capi.PBF_ERR_INVALID_ARG
    b.step([], w.dt)  # nothing to do


def test_persistent_loop_equals_per_pass_launches():
    """The Jacobi loop as one cooperative launch (grid-stride, bounded grid
    barrier) gives the same bits as one launch per pass, with scenes of
    different iteration counts (0 to 7) in one batch."""
    ws, variants = mixed_scenes()
    alone = [make_scene(w, **kw) for w, kw in zip(ws, variants)]
    inbatch = [make_scene(w, **kw) for w, kw in zip(ws, variants)]
    for sc, w in zip(alone, ws):
        sc.step(w.dt, 3)
    b = capi.Batch()
    b.set_persistent(True)
    for _ in range(3):
        b.step(inbatch, [w.dt for w in ws])
    b.sync()
    for k, (a, c) in enumerate(zip(alone, inbatch)):
        assert_same(state(a), state(c), f"scene {k} {variants[k]}")


def test_persistent_loop_on_a_large_batch():
    ws = workloads.batched_scenes(nscenes=24, seed=6, n_lo=2000, n_hi=64000)
    a = [make_scene(w) for w in ws]
    c = [make_scene(w) for w in ws]
    b1, b2 = capi.Batch(), capi.Batch()
    b2.set_persistent(True)
    b1.step(a, ws[0].dt, nsteps=2)
    b2.step(c, ws[0].dt, nsteps=2)
    b2.sync()
    for k in range(len(ws)):
        assert_same(state(a[k]), state(c[k]), f"scene {k}")


def test_autotuner_keeps_results_and_caches_its_choice(tmp_path, monkeypatch):
    """Autotuning tries four choices on the first steps of a batch shape
    (block size 128/64/256, persistent loop) without changing any result,
    then keeps the fastest and records it; a new batch reads it back."""
    cache = tmp_path / "autotune.jsonl"
    monkeypatch.setenv("PBF_AUTOTUNE_CACHE", str(cache))
    ws, variants = mixed_scenes()
    alone = [make_scene(w, **kw) for w, kw in zip(ws, variants)]
    inbatch = [make_scene(w, **kw) for w, kw in zip(ws, variants)]
    nsteps = 6
    for sc, w in zip(alone, ws):
        sc.step(w.dt, nsteps)
    b = capi.Batch()
    b.set_autotune(True)
    seen = set()
    for _ in range(nsteps):
        b.step(inbatch, [w.dt for w in ws])
        seen.add(b.tuning())
    assert {(128, 0), (64, 0), (256, 0), (128, 1)} <= seen
    for k, (a, c) in enumerate(zip(alone, inbatch)):
        assert_same(state(a), state(c), f"scene {k}")
    lines = cache.read_text().splitlines()
    assert len(lines) >= 1 and '"block": ' in lines[0]
    best = b.tuning()
    b2 = capi.Batch()
    b2.set_autotune(True)
    b2.step(inbatch, [w.dt for w in ws])
    assert b2.tuning() == best
