#!/usr/bin/env python
"""Throughput of the GB300 PBF step (particle-steps/s) on the 1M-particle dam break.

A step is one full PBF step (predict, cell sort, reference hash buckets,
4 Jacobi density iterations with s_corr, velocity update, XSPH, vorticity
confinement, domain clamp, commit) over one batch of synthetic input: the
seeded 1,000,000-particle dam break (100^3 lattice at r = 0.01 m in a
4x2x2 m box, h = 4r, dt = 1/240 s; novaphy_gb300/workloads.py).  Every step
starts from that seeded state (restored from a device-resident snapshot by a
device-to-device copy inside the timed region): with the configured s_corr
k = 0.1 the reference's own step explodes within a step or two and
consecutive steps pile the fluid onto the walls and into the box corners, so
a run of consecutive steps measures that degenerate state instead (reported
separately as `consecutive`, and in the summary).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

ours: `value` is device throughput with the scene resident in HBM (CUDA
events on the scene's stream around K {restore; graph-replayed step}; the
per-step working set, ~300 MB, exceeds the 129 MB L2).  Arithmetic is the
default exact build (bit-identical to the reference); `fast` repeats the
measurement with the FMA build.  `e2e` is the same metric through the
drop-in host-array call pbf_solver_step_host (the C ABI of PBFSolver::step):
each call uploads x, v, densities, lambdas from pinned host memory, steps
and reads them back; the host arrays are re-seeded between calls outside the
timed calls.  Under torchrun each rank runs an independent replica on its own
GPU (the single-scene path does not shard); `value` sums the ranks'
particle-steps over the slowest rank's time.

reference: the reference's CPU PBF step on the same 1M workload and config,
each step from the seeded state.  What runs is the oracle's C restatement,
which the tests pin bit for bit to the reference's own sources built from its
tree (the tree is absent on the GPU host), with its per-particle loops spread
over every host thread.  This arm imports no native code of the package.
"""
from __future__ import annotations

import argparse
import faulthandler
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

from novaphy_gb300 import shard, workloads  # noqa: E402

METRIC = "particle-steps/sec"
UNIT = "particle-steps/s"
# Algorithmic (compulsory) HBM bytes per particle per launch of the two
# constraint kernels: density+lambda reads x* (12 B) and writes rho, lambda
# (8 B); delta reads x*, lambda (16 B) and writes x*' (12 B).
ALG_BYTES = {"fluid.pbf.iteration.compute_density": 20.0,
             "fluid.pbf.iteration.compute_delta_position": 28.0}
KERNEL_OF_PHASE = {"fluid.pbf.iteration.compute_density": "k_density_lambda",
                   "fluid.pbf.iteration.compute_delta_position": "k_delta"}


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def measured_peak_hbm():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        d = json.load(open(p))
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def profile_value(kernel: str, key: str = "traffic_bytes_per_launch"):
    """A per-launch figure of `kernel` (DRAM bytes, warp instructions) from the
    committed ncu summary of the 1M case, if any."""
    p = os.path.join(ROOT, "profiles", f"{kernel}_dam_break_1m.md")
    if not os.path.exists(p):
        return None
    for line in open(p):
        if line.strip().startswith(key + ":"):
            try:
                return float(line.split(":", 1)[1].strip())
            except ValueError:
                return None
    return None


def issue_roof(inst_per_launch, launch_ms, sm_mhz, kernel, sms=152):
    """Third roof, the one that binds: warp instructions issued per cycle per SM
    (4 schedulers, one instruction each per cycle).  Instructions per launch
    come from the ncu capture of the same kernel on the same workload; the
    launch time and SM clock are this run's."""
    if not inst_per_launch or not launch_ms or not sm_mhz:
        return None
    ipc = inst_per_launch / (launch_ms / 1e3 * sm_mhz * 1e6 * sms)
    return {"achieved": ipc, "peak": 4.0, "unit": "warp inst/cycle/SM", "frac": ipc / 4.0,
            "inst_per_launch": inst_per_launch,
            "source": f"smsp__inst_executed.sum of profiles/{kernel}_dam_break_1m.md"}


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.path = None

    def __enter__(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.device}", f"--query-gpu={self.Q}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        if self.proc is None or not self.path or not os.path.exists(self.path):
            return None
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            f = [t.strip() for t in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax = float(f[2])
            except ValueError:
                continue
            for nm, val in zip(names, f[5:9]):
                if val.lower() == "active":
                    reasons.add(nm)
        os.unlink(self.path)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": smax, "reasons": sorted(reasons),
                "samples": len(sm)}


def cpu_port(threads=None):
    """The oracle restatement (bit-identical to the reference build, which is
    pinned against it by the tests) with `threads` host threads on its
    per-particle loops (default: every host core)."""
    from oracle.oracle import Port

    port = Port()
    used = port.set_threads(threads or os.cpu_count() or 1)
    return port, used


CPU_KIND_NOTE = ("the oracle's C restatement of the reference's PBF step, bit-identical to "
                 "the reference's own sources built from its tree (the tests pin it); the "
                 "reference tree is absent on the GPU host, so the restatement is what runs, "
                 "with its per-particle loops spread over the host threads (the reference "
                 "itself is single-threaded)")


def time_cpu_1m(nsteps, warmup, vorticity):
    """Reference CPU steps of the full 1M dam break, each from the seeded state
    (the copy of the seeded arrays is inside the timed step)."""
    from oracle.oracle import Settings

    port, threads = cpu_port()
    w = workloads.dam_break_1m(vorticity=vorticity)
    s = Settings.make(**w.settings)
    z = np.zeros(w.n, np.float32)
    for _ in range(warmup):
        port.steps(s, w.x, w.v, z, z, w.dt, w.gravity, w.mass, 1)
    el = 0.0
    for _ in range(nsteps):
        t0 = time.perf_counter()
        port.steps(s, w.x, w.v, z, z, w.dt, w.gravity, w.mass, 1)
        el += time.perf_counter() - t0
    return w, w.n * nsteps / el, threads, el


def headline_config(w, ws, vorticity):
    """The `config` of the headline line, the same for both arms."""
    return {"workload": "dam_break_1m", "particles": w.n, "lattice": "100x100x100",
            "r": 0.01, "h": w.settings["kernel_radius"],
            "iterations": w.settings["solver_iterations"], "dt": w.dt,
            "vorticity_epsilon": vorticity,
            "arithmetic": "f32, the reference's operation order (bit-identical)",
            "hash_compat": 1,
            "step": "one PBF step from the seeded state (state restored inside the timed "
                    "region)",
            "l2": "per-step working set ~300 MB > 129 MB L2",
            "parallelism": f"replicas x{ws}" if ws > 1 else "one scene"}


def run_reference(args, ws, rank):
    if rank != 0:
        return 0
    w, val, threads, el = time_cpu_1m(args.steps, args.warmup, args.vorticity)
    line = {
        "impl": "reference", "metric": METRIC, "value": val, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": el * 1e3 / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic",
        "config": headline_config(w, ws, args.vorticity),
        "cpu_baseline": {"value": val, "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": f"the full workload: {w.n} particles x {args.steps} steps, "
                                   f"each from the seeded state, {threads} host threads",
                         "kind_note": CPU_KIND_NOTE},
        "e2e": {"value": val, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def percentile(xs, q):
    return float(np.percentile(np.asarray(xs, np.float64), q)) if len(xs) else None


def _cpu_scene_step(item):
    """One reference CPU step of one scene from its seeded state (pool worker)."""
    from oracle.oracle import Port, Settings

    settings, x, v, dt, g, mass = item
    port = Port()
    z = np.zeros(len(x), np.float32)
    t0 = time.perf_counter()
    port.steps(Settings.make(**settings), x, v, z, z, dt, g, mass, 1)
    return len(x), time.perf_counter() - t0


def cpu_scene_pool(sample):
    """Reference CPU throughput for independent scenes, one process per host
    core (spawned), each running one seeded step of a scene of `sample`.
    Returns particle-steps/s per core (scene-weighted) and that figure times
    the core count, the aggregate of a host running one scene per core."""
    import multiprocessing as mp

    cores = os.cpu_count() or 1
    items = [(w.settings, w.x, w.v, w.dt, w.gravity, w.mass) for w in sample]
    with mp.get_context("spawn").Pool(cores) as pool:
        res = pool.map(_cpu_scene_step, items, chunksize=1)
    n = sum(r[0] for r in res)
    busy = sum(r[1] for r in res)
    per_core = n / busy
    return {"value": per_core * cores, "unit": UNIT, "cores": cores, "kind": "port",
            "per_core": per_core,
            "sample": f"one seeded step of each of {len(sample)} scenes of the workload "
                      f"({n} particles), one spawned process per core; value = per-core "
                      f"throughput x {cores} cores"}


def run_batched(args, device, ws=1, rank=0, dist=None):
    """Independent dam-break scenes of uneven size (workloads.batched_scenes:
    1,024 scenes, 2,000-64,000 particles log-uniform, 2-6 iterations) stepped
    (a) as one batch per step (pbf_batch_step: one sort and one launch per
    phase for all scenes) and (b) by the plain drop-in path, one
    pbf_scene_step per scene on its own stream, all issued before one wait.
    Both arms run the same consecutive steps from the same seeded states
    (bit-identical trajectories), timed on the host clock from the first call
    to the end of the last step; the batch arm also reports the device time
    of seeded batch steps and per-step latency percentiles."""
    from novaphy_gb300 import capi

    wl = workloads.batched_scenes(nscenes=args.batched_scenes)
    if ws > 1:  # this rank's share of the scenes, dealt by particle count
        wl = [wl[i] for i in shard.rank_scenes([w.n for w in wl], ws, rank)]
    total = int(sum(w.n for w in wl))

    def barrier():
        if dist is not None:
            dist.barrier()
    scenes = []
    for w in wl:
        sc = capi.Scene(capi.default_settings(**w.settings), w.x, w.v, mass=w.mass, device=device)
        sc.set_gravity(w.gravity)
        scenes.append(sc)
    seeds = [sc.snapshot() for sc in scenes]
    dts = np.array([w.dt for w in wl], np.float32)
    k = max(1, args.batched_steps)

    def reseed():
        for sc, sd in zip(scenes, seeds):
            sc.restore(sd)

    progress(f"batched: {len(wl)} scenes created")
    # Batched arm, autotuned: the warm-up steps try the block sizes and the
    # persistent loop, the timed steps run the fastest.
    b = capi.Batch(device)
    b.set_autotune(True)
    for _ in range(5):
        reseed()
        b.step(scenes, dts)
    tuning = b.tuning()
    reseed()
    lat = []
    barrier()
    t0 = time.perf_counter()
    for _ in range(k):
        lat.append(b.step_timed(scenes, dts))
    t_batch = time.perf_counter() - t0
    job_units, job_batch = shard.job_throughput(total * k, t_batch, dist)
    reseed()
    dev_ms = b.replay_timed(scenes, seeds, dts, k)
    # The same with the Jacobi loop as one persistent cooperative launch.
    b.set_autotune(False)
    b.set_persistent(True)
    reseed()
    b.step(scenes, dts)  # graph with the persistent loop
    reseed()
    t0 = time.perf_counter()
    for _ in range(k):
        b.step(scenes, dts, sync=False)
    b.sync()
    t_persist = time.perf_counter() - t0
    b.set_persistent(False)

    t_plain = t_plain_sync = ks = None
    if not args.no_batched_plain:
        # Plain per-scene arm.
        progress("batched: plain arm")
        reseed()
        for sc, dt in zip(scenes, dts):  # warm-up: per-scene scratch and graphs
            sc.step(float(dt), 1, sync=False)
        for sc in scenes:
            sc.sync()
        reseed()
        t0 = time.perf_counter()
        for _ in range(k):
            for sc, dt in zip(scenes, dts):
                sc.step(float(dt), 1, sync=False)
        for sc in scenes:
            sc.sync()
        t_plain = time.perf_counter() - t0

        # Plain per-scene arm, synchronous: each scene's step returns after it is
        # done, as a loop over worlds calling the drop-in step does.
        progress("batched: plain synchronous arm")
        reseed()
        ks = min(k, 2)
        t0 = time.perf_counter()
        for _ in range(ks):
            for sc, dt in zip(scenes, dts):
                sc.step(float(dt), 1)
        t_plain_sync = time.perf_counter() - t0


    out = {
        "workload": f"batched_scenes: {len(wl)} dam-break scenes, {total} particles "
                    f"({min(w.n for w in wl)}-{max(w.n for w in wl)} per scene), r = 0.02, "
                    f"h = 4r, 2-6 iterations, dt = 1/120",
        "particles": total, "scenes": len(wl), "steps": k,
        "value": job_units / job_batch, "unit": UNIT,
        "ranks": ws, "rank0_particles": total,
        "plain_value": total * k / t_plain if t_plain else None,
        "speedup_vs_plain": t_plain / t_batch if t_plain else None,
        "plain_sync_value": total * ks / t_plain_sync if t_plain_sync else None,
        "plain_sync_steps": ks,
        "speedup_vs_plain_sync": (t_plain_sync / ks) / (t_batch / k) if t_plain_sync else None,
        "step_ms_p50": percentile(lat, 50), "step_ms_p99": percentile(lat, 99),
        "seeded_device_value": total * k / (dev_ms / 1e3),
        "persistent_value": total * k / t_persist,
        "autotuned": {"block": tuning[0], "persistent": bool(tuning[1])},
        "batch_scratch_bytes": b.device_bytes(),
        "timing": "host clock over k consecutive steps from the seeded states, both arms",
    }
    b.close()
    for sd in seeds:
        sd.close()
    for sc in scenes:
        sc.close()
    if not args.no_cpu_baseline and not args.no_batched_plain:
        progress("batched: cpu baseline")
        if rank == 0:
            out["cpu_baseline"] = cpu_scene_pool(
                wl[:: max(1, len(wl) // (2 * (os.cpu_count() or 1)))])
    return out


def sphere_boundary(w, device=0):
    """Akinci boundary of a workload's rigid spheres (workloads.served_scenes):
    body-frame samples at spacing r from the host sampler, psi from their
    initial world positions on the device, and the bodies as RigidBody."""
    import novaphy_gb300 as nv
    from novaphy_gb300 import capi

    sph = w.meta.get("spheres", [])
    if not sph:
        return None
    r = w.meta["r"]
    mb = nv.ModelBuilder()
    bodies = []
    for (c, rad, dens) in sph:
        m = float(np.float32(dens) * np.float32(4.0 / 3.0 * np.pi) * np.float32(rad) ** 3)
        rb = nv.RigidBody.from_sphere(m, rad)
        bi = mb.add_body(rb, nv.Transform.from_translation(np.array(c, np.float32)))
        mb.add_shape(nv.CollisionShape.make_sphere(rad, bi))
        b = capi.RigidBody()
        b.pos[:] = [float(v) for v in np.array(c, np.float32)]
        b.quat[:] = [1.0, 0.0, 0.0, 0.0]
        b.inv_mass = rb.inv_mass()
        b.inv_inertia[:] = rb.inv_inertia()
        bodies.append(b)
    bps = nv.sample_model_boundaries(mb.build(), r, 1.0)
    local = np.stack([b.local_position for b in bps]).astype(np.float32)
    body = np.array([b.body_index for b in bps], np.int32)
    centers = np.array([c for (c, _, _) in sph], np.float32)
    world = (local + centers[body]).astype(np.float32)
    psi = capi.boundary_volumes(world, w.settings["kernel_radius"], device)
    return local, body, psi, bodies


def rigid_step_np(state, f, t, g, dt):
    """Host rigid step of free bodies in numpy (float32), for the plain arm:
    the same semi-implicit Euler as the library's (timing only)."""
    dt = np.float32(dt)
    for k, b in enumerate(state):
        if b["inv_mass"] == 0:
            continue
        b["v"] += (g + f[k] * b["inv_mass"]) * dt
        b["w"] = (b["w"] + (b["ii"] @ t[k]) * dt) * np.float32(0.999)
        b["p"] += b["v"] * dt
        qw, qx, qy, qz = b["q"]
        w = b["w"]
        dq = np.float32(0.5) * np.array([-w[0] * qx - w[1] * qy - w[2] * qz,
                                         w[0] * qw + w[2] * qy - w[1] * qz,
                                         w[1] * qw - w[2] * qx + w[0] * qz,
                                         w[2] * qw + w[1] * qx - w[0] * qy], np.float32)
        q = b["q"] + dq * dt
        b["q"] = (q / np.sqrt((q * q).sum())).astype(np.float32)


def run_served(args, device, ws=1, rank=0, dist=None):
    """Serving run over workloads.served_scenes (256 clients, 1k-200k particles
    log-uniform, dam breaks and pools, dt = 1/240).  Each client draws request
    arrivals from its own Poisson process with mean 512 ms (so 2 ms for all
    clients together) and asks for k in {1, 4, 16} steps.

    served: requests go to the serving loop (pbf_server_*, continuous
    batching).  Run at the full HBM budget; again with arrivals thinned to
    about half of the throughput the first run measured (latency without an
    overload's backlog); and at a reduced budget sized to
    half of the scenes' charged bytes, where client sessions of 8 requests
    on average close their scene and open a fresh one so that waiting scenes
    get admitted.  plain: each client steps its own scene with the drop-in
    call (pbf_scene_step on the scene's stream, then wait) from its own
    thread, requests queued per client.  Latency = arrival to completion."""
    import threading

    from novaphy_gb300 import capi

    wl = workloads.served_scenes()
    if ws > 1:  # this rank's clients, dealt by particle count; one server per GPU
        wl = [wl[i] for i in shard.rank_scenes([w.n for w in wl], ws, rank)]
    dt = np.float32(wl[0].dt)
    T = float(args.serve_seconds)
    T_side = float(args.serve_side_seconds)

    def make_plans(mean_s, seed, T=T):
        rng = np.random.default_rng(seed)
        out = []
        for k in range(len(wl)):
            t, p = 0.0, []
            while True:
                t += float(rng.exponential(mean_s))
                if t >= T:
                    break
                p.append((t, int(rng.choice([1, 4, 16]))))
            out.append(p)
        return out

    def demand_of(pl):
        return sum(wl[k].n * m for k in range(len(wl)) for _, m in pl[k])

    plans = make_plans(0.512, 44)
    demand = demand_of(plans)
    coupled = [sphere_boundary(w, device) for w in wl]

    # Both arms stop waiting for stragglers 30 s after the last arrival; a
    # run's value is the particle-steps it completed over its wall time.
    drain_s = 30.0

    def served_run(budget=None, session_mean=None, max_batch=16 << 20, plans=plans, T=T):
        deadline_after = T + drain_s
        cfg = capi.server_config(max_batch_particles=max_batch)
        if budget is not None:
            cfg.hbm_budget_bytes = int(budget)
        srv = capi.Server(cfg, device)
        errors = []
        lock = threading.Lock()
        t0 = time.perf_counter() + 0.5
        deadline = t0 + deadline_after

        def wait_all(reqs):
            for q in reqs:
                srv.wait(q, timeout=max(0.0, deadline - time.perf_counter()))

        def client(k):
            w = wl[k]
            st = capi.default_settings(**w.settings)
            r = np.random.default_rng(1000 + k)
            cp = coupled[k]

            def open_():
                if cp is None:
                    return srv.open_scene(st, w.x, w.v, w.mass, w.gravity)[0]
                return srv.open_coupled_scene(st, w.x, w.v, w.mass, w.gravity, *cp)[0]

            try:
                sid = open_()
                left = int(r.geometric(1.0 / session_mean)) if session_mean else -1
                mine = []
                for (ta, m) in plans[k]:
                    d = t0 + ta - time.perf_counter()
                    if d > 0:
                        time.sleep(d)
                    if left == 0:
                        wait_all(mine)
                        mine = []
                        srv.close_scene(sid)
                        sid = open_()
                        left = int(r.geometric(1.0 / session_mean))
                    mine.append(srv.submit(sid, float(dt), m))
                    left -= 1
                wait_all(mine)
                srv.close_scene(sid)
            except capi.PbfError as e:
                with lock:
                    errors.append(str(e))

        th = [threading.Thread(target=client, args=(k,)) for k in range(len(wl))]
        for t in th:
            t.start()
        for t in th:
            t.join()
        el = time.perf_counter() - t0
        stats = srv.stats()
        srv.close()
        job_units, job_el = shard.job_throughput(stats["particle_steps"], el, dist)
        return {"value": job_units / job_el, "unit": UNIT, "wall_s": el,
                "particle_steps": stats["particle_steps"],
                "step_ms_p50": stats["step_ms_p50"], "step_ms_p99": stats["step_ms_p99"],
                "request_ms_p50": stats["request_ms_p50"],
                "request_ms_p99": stats["request_ms_p99"],
                "requests_done": stats["requests_done"],
                "requests_failed": stats["requests_failed"],
                "scenes_failed": stats["scenes_failed"],
                "client_errors": len(errors),
                "errors": dict(__import__("collections").Counter(errors).most_common(3)),
                "launches": stats["launches"], "mean_launch_scenes": stats["mean_launch_scenes"],
                "issue_ms_mean": stats["issue_ms_mean"],
                "graph_captures": stats["graph_captures"], "graph_updates": stats["graph_updates"],
                "graph_instantiations": stats["graph_instantiations"],
                "launches_direct": stats["launches_direct"],
                "post_ms_mean": stats["post_ms_mean"],
                "mean_launch_particles": stats["mean_launch_particles"],
                "scenes_rejected": stats["scenes_rejected"],
                "hbm_bytes_scratch": stats["hbm_bytes_scratch"],
                "budget_bytes": int(cfg.hbm_budget_bytes)}

    def plain_run(T=T):
        deadline_after = T + drain_s
        scenes, rigid = [], []
        for k, w in enumerate(wl):
            sc = capi.Scene(capi.default_settings(**w.settings), w.x, w.v, mass=w.mass,
                            device=device)
            sc.set_gravity(w.gravity)
            sc.step(float(dt), 1)  # warm-up: scratch and the step graph
            sc.reset(w.x, w.v)
            cp = coupled[k]
            st_b = None
            if cp is not None:
                local, body, psi, bodies = cp
                sc.set_boundary(local, body, psi)
                st_b = [{"p": np.array(b.pos, np.float32), "q": np.array(b.quat, np.float32),
                         "v": np.zeros(3, np.float32), "w": np.zeros(3, np.float32),
                         "inv_mass": np.float32(b.inv_mass),
                         "ii": np.array(b.inv_inertia, np.float32).reshape(3, 3)} for b in bodies]
            scenes.append(sc)
            rigid.append(st_b)

        def plain_step(k):
            sc, st_b = scenes[k], rigid[k]
            if st_b is None:
                sc.step(float(dt), 1)
                return
            nb = len(st_b)
            sc.set_bodies(np.stack([b["p"] for b in st_b]), np.stack([b["q"] for b in st_b]),
                          np.array([1 if b["inv_mass"] > 0 else 0 for b in st_b], np.int32))
            f, t = sc.step_coupled(float(dt), np.zeros((nb, 3), np.float32),
                                   np.zeros((nb, 3), np.float32))
            rigid_step_np(st_b, f, t, np.asarray(wl[k].gravity, np.float32), dt)
        lat_step, lat_req = [], []
        done = [0]
        lock = threading.Lock()
        t0 = time.perf_counter() + 0.5
        deadline = t0 + deadline_after

        def client(k):
            sc = scenes[k]
            for (ta, m) in plans[k]:
                d = t0 + ta - time.perf_counter()
                if d > 0:
                    time.sleep(d)
                if time.perf_counter() > deadline:
                    break
                prev = max(t0 + ta, time.perf_counter())
                steps = []
                for _ in range(m):
                    plain_step(k)
                    now = time.perf_counter()
                    steps.append((now - prev) * 1e3)
                    prev = now
                with lock:
                    lat_step.extend(steps)
                    lat_req.append((time.perf_counter() - (t0 + ta)) * 1e3)
                    done[0] += wl[k].n * m

        th = [threading.Thread(target=client, args=(k,)) for k in range(len(wl))]
        for t in th:
            t.start()
        for t in th:
            t.join()
        el = time.perf_counter() - t0
        for sc in scenes:
            sc.close()
        job_units, job_el = shard.job_throughput(done[0], el, dist)
        return {"value": job_units / job_el, "unit": UNIT, "wall_s": el, "particle_steps": done[0],
                "step_ms_p50": percentile(lat_step, 50), "step_ms_p99": percentile(lat_step, 99),
                "request_ms_p50": percentile(lat_req, 50),
                "request_ms_p99": percentile(lat_req, 99)}

    progress("served: full budget")
    full = served_run(max_batch=args.served_max_batch)
    # The same clients at about half of this rank's measured throughput, so
    # that latencies show service time rather than the backlog of an overload.
    own_rate = full["particle_steps"] / max(full["wall_s"], 1e-9)
    mean_half = 0.512 * (demand / T) / max(0.5 * own_rate, 1.0)
    plans_half = make_plans(mean_half, 45, T=T_side)
    progress("served: half load")
    half = served_run(max_batch=args.served_max_batch, plans=plans_half, T=T_side)
    half["arrivals"] = (f"per-client Poisson, mean {mean_half * 1e3:.0f} ms over {T_side:.0f} s, "
                        f"{sum(len(p) for p in plans_half)} requests")
    half["offered_fraction_of_capacity"] = demand_of(plans_half) / T_side / max(own_rate, 1.0)
    if args.served_full_only:
        return {"value": full["value"], "unit": UNIT, "full_budget": full, "half_load": half,
                "max_batch_particles": args.served_max_batch}
    total_charge = sum(w.n for w in wl) * capi.state_bytes_per_particle()
    small_batch = 1 << 20
    probe = capi.Server(capi.server_config(max_batch_particles=small_batch), device)
    scratch = probe.stats()["hbm_bytes_scratch"]
    probe.close()
    progress("served: reduced budget")
    reduced = served_run(budget=scratch + total_charge // 2, session_mean=8,
                         max_batch=small_batch, plans=make_plans(0.512, 46, T=T_side), T=T_side)
    reduced["arrivals"] = f"per-client Poisson, mean 512 ms over {T_side:.0f} s"
    progress("served: plain")
    plain = plain_run()
    cpu = None
    if not args.no_cpu_baseline and rank == 0:
        progress("served: cpu baseline")
        cpu = cpu_scene_pool(wl[:: max(1, len(wl) // (2 * (os.cpu_count() or 1)))])
    return {
        "workload": f"served_scenes: {len(wl)} clients, {sum(w.n for w in wl)} particles "
                    f"({min(w.n for w in wl)}-{max(w.n for w in wl)} per scene), dam breaks "
                    f"and pools with {sum(len(w.meta['spheres']) for w in wl)} Akinci spheres in "
                    f"{sum(1 for c in coupled if c is not None)} of them, r = 0.02, h = 4r, "
                    f"4 iterations, dt = 1/240, "
                    f"s_corr k = 0.001 (PBFSettings default)",
        "arrivals": f"per-client Poisson, mean 512 ms (2 ms aggregate) over {T:.0f} s; "
                    f"k in {{1, 4, 16}}; {sum(len(p) for p in plans)} requests, "
                    f"{demand} particle-steps offered",
        "state_bytes_per_particle": capi.state_bytes_per_particle(),
        "value": full["value"], "unit": UNIT, "seconds": T,
        "step_ms_p50": full["step_ms_p50"], "step_ms_p99": full["step_ms_p99"],
        "request_ms_p50": full["request_ms_p50"], "request_ms_p99": full["request_ms_p99"],
        "speedup_vs_plain": full["value"] / plain["value"],
        "full_budget": full, "half_load": half, "reduced_budget": reduced, "plain": plain,
        "cpu_baseline": cpu,
    }


def run_coupled(args, device):
    """Two-way rigid-fluid coupling through the drop-in FluidWorld: a
    250,000-particle pool (50 x 50 x 100 lattice at r = 0.015 centred on the
    floor of a 2 x 2 x 2 m box), 4 boxes (edge 0.2 m) and 4 spheres (radius
    0.12 m) of density U(300, 1500) dropped from 0.5-1.0 m above the pool, at
    x-y positions in 8 of the 9 cells of a 3 x 3 grid over the pool (seed 2),
    a floor plane; Akinci boundary particles at spacing r; h = 4r, 4
    iterations, dt = 1/240, PBFSettings' s_corr (k = 0.001, dq = 0.3h), XSPH
    0.01, vorticity 1e-4.  One step = FluidWorld.step: the PBF step, boundary
    density, coupling forces and torques reduced per body on the device, the
    host rigid step.  Timed on the host clock over consecutive steps after
    warm-up."""
    spec = workloads.coupled_pool(scorr=args.coupled_scorr)
    world = workloads.fluid_world_of(spec)
    st = world.pbf_settings
    dt = float(np.float32(1.0 / 240.0))
    for _ in range(2):
        world.step(dt)
    k = max(1, args.coupled_steps)
    marks = []
    t0 = time.perf_counter()
    for i in range(k):
        world.step(dt)
        if (i + 1) % max(1, k // 4) == 0:
            marks.append(time.perf_counter())
    el = time.perf_counter() - t0
    seg = k // 4 if k >= 4 else 1
    quarters = [round((b - a) * 1e3 / seg, 3) for a, b in zip([t0] + marks[:-1], marks)][:4]
    n, nb = world.num_particles, world.num_boundary_particles
    # Device time of every phase over 3 more steps (the monitor runs the same
    # step as separate launches with CUDA events between the phases).
    mon = world.performance_monitor
    mon.reset()
    mon.enabled = True
    for _ in range(3):
        world.step(dt)
    mon.enabled = False
    phases = {p.name: p.avg_ms for p in mon.phase_stats()}
    iters = 4
    dom = max(ALG_BYTES, key=lambda q: phases.get(q, 0.0))
    launch_ms = phases[dom] / iters
    peak, peak_kind = measured_peak_hbm()
    achieved = ALG_BYTES[dom] * n / (launch_ms / 1e3) / 1e9
    return {"workload": f"coupled pool: {n} fluid + {nb} boundary particles, 8 bodies "
                        f"(4 boxes, 4 spheres) and a floor plane, r = 0.015, h = 4r, "
                        f"4 iterations, dt = 1/240",
            "value": n * k / el, "unit": UNIT, "steps": k, "ms_per_step": el * 1e3 / k,
            "fluid_particles": n, "boundary_particles": nb,
            "step": "FluidWorld.step: PBF step, boundary density, coupling forces/torques "
                    "(device, per-body serial reduction), host rigid step",
            "timing": f"host clock over {k} consecutive steps after 2 warm-up steps",
            "ms_per_step_by_quarter": quarters,
            "s_corr": {"k": float(st.corr_k), "delta_q": float(st.corr_delta_q),
                       "source": "PBFSettings default" if args.coupled_scorr != "config0"
                       else "the 8k dam break's"},
            "roofline": {"bound": "hbm", "kernel": KERNEL_OF_PHASE[dom], "achieved": achieved,
                         "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                         "alg_bytes_per_launch": ALG_BYTES[dom] * n, "launch_ms": launch_ms,
                         "peak_source": f"{peak_kind} (MEASURED_PEAKS.json hbm_gbs)",
                         "timing": "monitor device phases, 3 steps after the timed ones"},
            "phases_ms": {q: round(v, 4) for q, v in sorted(phases.items())}}


# FP32 (non-tensor) issue peak of a GB300: 152 SMs x 128 FP32 lanes x 2 FLOP
# (fused multiply-add) x 2.07 GHz.  Nominal: no measured FP32 peak exists.
FP32_PEAK_TFLOPS_NOMINAL = 152 * 128 * 2 * 2.07e9 / 1e12


def fp32_roof(particle_steps_per_s, iters, candidates=1728, neighbours=250):
    """Second roof: algorithmic FP32 work of a particle-step at h = 4r.  Every
    candidate of the 27 cells is tested in each of the 2I + 3 neighbour passes
    (3 subtractions + 5 for the squared norm = 8 FLOP), and each of the ~250
    neighbours costs density+lambda 30, delta+s_corr 40 (per iteration), XSPH
    20, omega 22 and confinement 20 FLOP."""
    passes = 2 * iters + 3
    flop = 8 * candidates * passes + neighbours * (70 * iters + 62)
    achieved = particle_steps_per_s * flop / 1e12
    return {"achieved": achieved, "peak": FP32_PEAK_TFLOPS_NOMINAL, "unit": "TFLOP/s",
            "frac": achieved / FP32_PEAK_TFLOPS_NOMINAL, "flop_per_particle_step": flop,
            "peak_source": "nominal (152 SMs x 128 lanes x 2 x 2.07 GHz)"}


def summary_of(value, e2e, fast, roofline, coupled, batched, served, consecutive=None):
    """The headline figures of every section in a few short keys."""
    def r(x, nd=4):
        return None if x is None else float(f"{x:.{nd}g}")

    def get(d, *ks):
        for k in ks:
            if not isinstance(d, dict) or d.get(k) is None:
                return None
            d = d[k]
        return d

    out = {"1m": {"exact": r(value), "e2e": r(get(e2e, "value")), "fast": r(get(fast, "value")),
                  "hbm_frac": r(roofline["frac"], 3),
                  "issue_frac": r(get(roofline, "issue", "frac"), 3),
                  "consecutive": r(get(consecutive, "value"))}}
    if coupled:
        out["coupled"] = {"value": r(get(coupled, "value")), "steps": get(coupled, "steps"),
                          "hbm_frac": r(get(coupled, "roofline", "frac"), 3),
                          "error": get(coupled, "error")}
    if batched:
        out["batched"] = {"value": r(get(batched, "value")),
                          "plain_async": r(get(batched, "plain_value")),
                          "x_plain_async": r(get(batched, "speedup_vs_plain"), 3),
                          "plain_sync": r(get(batched, "plain_sync_value")),
                          "x_plain_sync": r(get(batched, "speedup_vs_plain_sync"), 3),
                          "p50_ms": r(get(batched, "step_ms_p50")),
                          "p99_ms": r(get(batched, "step_ms_p99")),
                          "error": get(batched, "error")}
    if served:
        out["served"] = {"value": r(get(served, "value")),
                         "seconds": get(served, "seconds"),
                         "plain": r(get(served, "plain", "value")),
                         "x_plain": r(get(served, "speedup_vs_plain"), 3),
                         "step_p50_ms": r(get(served, "step_ms_p50")),
                         "step_p99_ms": r(get(served, "step_ms_p99")),
                         "req_p50_ms": r(get(served, "request_ms_p50")),
                         "req_p99_ms": r(get(served, "request_ms_p99")),
                         "half_load": {"value": r(get(served, "half_load", "value")),
                                       "step_p50_ms": r(get(served, "half_load", "step_ms_p50")),
                                       "step_p99_ms": r(get(served, "half_load", "step_ms_p99"))},
                         "error": get(served, "error")}
    for sec in out.values():
        if isinstance(sec, dict) and sec.get("error") is None:
            sec.pop("error", None)
    out["plain_arm"] = ("plain = the drop-in per-scene call on each scene's own stream, all "
                        "issued before one wait (asynchronous); plain_sync waits for each step")
    return out


def side_section(ws, fn):
    """Runs one of the sections beside the headline (batched, coupled,
    served).  On one rank, a failure is reported in that section's place
    instead of losing the whole line; with several ranks it propagates, since
    the other ranks would wait in a collective."""
    if ws > 1:
        return fn()
    try:
        return fn()
    except Exception as e:  # noqa: BLE001 - reported in the JSON line
        import traceback

        traceback.print_exc()
        return {"error": f"{type(e).__name__}: {e}"}


def run_ours(args, ws, rank, local):
    from novaphy_gb300 import capi

    capi.load()
    dist = None
    if ws > 1:
        import torch.distributed as dist  # noqa: F811

        dist.init_process_group("gloo")
    device = local
    w = workloads.dam_break_1m(vorticity=args.vorticity)
    s = capi.default_settings(**w.settings, exact_arithmetic=1)
    sc = capi.Scene(s, w.x, w.v, mass=w.mass, device=device)
    sc.set_gravity(w.gravity)
    seed = sc.snapshot()

    def barrier():
        if dist is not None:
            dist.barrier()

    def max_over_ranks(x):
        if dist is None:
            return x
        import torch

        t = torch.tensor([x], dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        return float(t.item())

    progress("single scene: warm-up")
    sc.replay_timed(seed, w.dt, max(args.warmup, 1))  # warm-up (captures the step graph)
    barrier()
    with ClockSampler(device) as clk:
        ms = sc.replay_timed(seed, w.dt, args.steps)
    barrier()
    clocks = clk.summary()
    sec = max_over_ranks(ms / 1e3)
    value = w.n * args.steps * ws / sec

    # Per-phase device times (one non-graph step from the seed each).
    phases, launches = {}, {}
    reps = 3
    for _ in range(reps):
        sc.restore(seed)
        for k, (t_ms, nl) in sc.step_profiled(w.dt).items():
            phases[k] = phases.get(k, 0.0) + t_ms / reps
            launches[k] = nl
    launches_per_step = sum(launches.values())
    dom = max(ALG_BYTES, key=lambda k: phases.get(k, 0.0))
    iters = w.settings["solver_iterations"]
    launch_ms = phases[dom] / iters
    alg = ALG_BYTES[dom] * w.n
    achieved = alg / (launch_ms / 1e3) / 1e9
    peak, peak_kind = measured_peak_hbm()
    kern = KERNEL_OF_PHASE[dom]
    traffic = profile_value(kern)
    roofline = {"bound": "hbm", "kernel": kern, "achieved": achieved, "peak": peak,
                "unit": "GB/s", "frac": achieved / peak, "traffic": traffic,
                "alg_bytes_per_launch": alg, "launch_ms": launch_ms,
                "peak_source": f"{peak_kind} (MEASURED_PEAKS.json hbm_gbs)",
                "fp32": fp32_roof(value / ws, iters),
                "issue": issue_roof(profile_value(kern, "warp_instructions_per_launch"), launch_ms,
                                    clocks.get("sm_mhz") if clocks else None, kern)}

    progress("single scene: fast build")
    # The FMA build on the same batch.
    fast = None
    if not args.no_fast:
        sf = capi.default_settings(**w.settings, exact_arithmetic=0)
        fs = capi.Scene(sf, w.x, w.v, mass=w.mass, device=device)
        fs.set_gravity(w.gravity)
        fseed = fs.snapshot()
        fs.replay_timed(fseed, w.dt, max(args.warmup, 1))
        barrier()
        fsec = max_over_ranks(fs.replay_timed(fseed, w.dt, args.steps) / 1e3)
        fast = {"value": w.n * args.steps * ws / fsec, "unit": UNIT,
                "ms_per_step": fsec * 1e3 / args.steps, "arithmetic": "FMA, rsqrt, approximate division"}
        fseed.close()
        fs.close()

    # Consecutive steps of the configured trajectory from the seed.
    consecutive = None
    if not args.no_consecutive:
        ksteps = min(args.steps, 10)
        sc.restore(seed)
        cms = sc.step_timed(w.dt, ksteps)
        consecutive = {"value": w.n * ksteps / (cms / 1e3), "unit": UNIT, "steps": ksteps,
                       "note": "steps 1..k of the seeded dam break; the configured s_corr "
                               "makes it explode, and the domain clamp piles fluid into the "
                               "box corners"}

    progress("single scene: end to end")
    # End to end through the host-array drop-in call.
    e2e = None
    if not args.no_e2e:
        try:
            import torch

            def pinned(shape):
                return torch.empty(shape, dtype=torch.float32).pin_memory().numpy()
        except Exception:  # pragma: no cover
            def pinned(shape):
                return np.empty(shape, np.float32)
        hx, hv = pinned((w.n, 3)), pinned((w.n, 3))
        hr, hl = pinned((w.n,)), pinned((w.n,))
        drop = capi.Scene(s, w.x[:1], None, mass=w.mass, device=device)
        L = capi.load()
        import ctypes as C

        g = np.ascontiguousarray(w.gravity, np.float32)
        gp = g.ctypes.data_as(C.POINTER(C.c_float))

        def reseed():
            hx[:] = w.x
            hv[:] = w.v
            hr[:] = 0
            hl[:] = 0

        def call():
            capi.check(L.pbf_solver_step_host(drop.handle, w.n, capi._ptr(hx), capi._ptr(hv),
                                              capi._ptr(hr), capi._ptr(hl), w.dt, gp, w.mass))

        for _ in range(max(args.warmup, 1)):
            reseed()
            call()
        barrier()
        el = 0.0
        for _ in range(args.steps):
            reseed()
            t0 = time.perf_counter()
            call()
            el += time.perf_counter() - t0
        barrier()
        el = max_over_ranks(el)
        per = w.n * (12 + 12 + 4 + 4)
        e2e = {"value": w.n * args.steps * ws / el, "unit": UNIT, "h2d_bytes_per_step": per,
               "d2h_bytes_per_step": per,
               "call": "pbf_solver_step_host: pinned host x, v, densities, lambdas in and out"}
        drop.close()

    batched = None
    if not args.no_batched:
        progress("batched scenes")
        batched = side_section(ws, lambda: run_batched(args, device, ws, rank, dist))
    coupled = None
    if not args.no_coupled:
        progress("coupled scene")
        coupled = side_section(ws, lambda: run_coupled(args, device))
    served = None
    if not args.no_served:
        progress("served scenes")
        served = side_section(ws, lambda: run_served(args, device, ws, rank, dist))

    cpu = None
    if rank == 0 and ws == 1 and not args.no_cpu_baseline:
        progress("cpu baseline")
        _, val, threads, el = time_cpu_1m(1, 0, args.vorticity)
        cpu = {"value": val, "unit": UNIT, "cores": threads, "kind": "port",
               "sample": f"one step of the full workload ({w.n} particles) from the seeded "
                         f"state, {threads} host threads ({el:.1f} s)",
               "kind_note": CPU_KIND_NOTE}

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": sec * 1e3 / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic",
            "config": headline_config(w, ws, args.vorticity),
            "roofline": roofline,
            "cpu_baseline": cpu,
            "e2e": e2e,
            "gpu_launches": launches_per_step * args.steps,
            "clocks": clocks,
            "phases_ms": {k: round(v, 4) for k, v in phases.items()},
            "fast": fast,
            "consecutive": consecutive,
            "coupled": coupled,
            "batched": batched,
            "served": served,
            # Last, so that a reader of the line's tail sees it whole.
            "summary": summary_of(value, e2e, fast, roofline, coupled, batched, served,
                                  consecutive),
        }
        print(json.dumps(line), flush=True)
    seed.close()
    sc.close()
    if dist is not None:
        dist.destroy_process_group()
    return 0


def progress(msg):
    print(f"[bench {time.strftime('%H:%M:%S')}] {msg}", file=sys.stderr, flush=True)


def main():
    faulthandler.enable()
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--vorticity", type=float, default=1e-4)
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-fast", action="store_true")
    ap.add_argument("--no-consecutive", action="store_true")
    ap.add_argument("--no-batched", action="store_true")
    ap.add_argument("--batched-scenes", type=int, default=1024)
    ap.add_argument("--batched-steps", type=int, default=10)
    ap.add_argument("--no-batched-plain", action="store_true",
                    help="skip the plain per-scene arms and CPU pool of the batched run")
    ap.add_argument("--no-served", action="store_true")
    ap.add_argument("--no-coupled", action="store_true")
    ap.add_argument("--coupled-steps", type=int, default=300)
    ap.add_argument("--coupled-scorr", choices=["default", "config0"], default="default",
                    help="s_corr of the coupled pool: PBFSettings' own or the dam break's k = 0.1")
    ap.add_argument("--serve-seconds", type=float, default=60.0,
                    help="arrival window of the full-budget served run and its plain arm")
    ap.add_argument("--serve-side-seconds", type=float, default=10.0,
                    help="arrival window of the half-load and reduced-budget served runs")
    ap.add_argument("--served-max-batch", type=int, default=16 << 20,
                    help="particles per launch of the full-budget serving run")
    ap.add_argument("--served-full-only", action="store_true",
                    help="run only the full-budget serving arm")
    args = ap.parse_args()
    if args.warmup < 3 and args.impl == "ours":
        print("warning: fewer than 3 warm-up steps", file=sys.stderr)
    ws, rank, local = dist_env()
    if args.impl == "reference":
        return run_reference(args, ws, rank)
    return run_ours(args, ws, rank, local)


if __name__ == "__main__":
    sys.exit(main())
