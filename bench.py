"""Benchmark: cloth vertex-steps/s on one GB300 (large plain cloth).

Workload: the 1024 x 1024 plain cloth (1,048,576 vertices, 5,230,601 struts,
2,093,058 triangles; per-strut stiffness within +-10%, N(0, 1e-3) position
noise, top row pinned, wind, drag/lift, plane + UV-sphere colliders,
explicit Euler at dt = 1/600 s) built by feriphys_gb300.workloads.c1 on
synthetic seeded data.  A "step" is one Simulation::step of that cloth.
Rollouts restart from the initial state every --rollout steps outside the
timed region: 30 by default.  Explicit Euler at the configured dt is
unstable on this cloth: from step ~36 the largest speed doubles every two
steps and the state is non-finite at step 62 (bench.py --probe); from step
~45 the exploding vertices' segments cross the whole sphere, so the exact
first-hit search tests every obstacle face for them and a step costs ~3.5x
more.  Rollouts of 30 keep every timed step on the physical part of the
trajectory (each one a complete step of the configuration).

Timing: W warm-up steps, then K steps; L2 is flushed (a 256 MB write) before
every timed step and each step is timed with CUDA events on the stream the
kernel runs on; ms_per_step is their mean.  `e2e` repeats the metric through
the C ABI with host buffers every step: set_points (H2D of the Stateful
points from pinned memory) + step + get_points (D2H).  `cpu_baseline` times
the oracle (a single-threaded C++ restatement of the reference's step, like
the reference) on a bounded sample of the same workload.

`--impl reference` times that CPU implementation alone (the Rust reference
cannot be built here: no cargo/rustc) and prints the reference line.
Multi-GPU: the path does not shard, so `--gpus N` runs N independent
replicas under torchrun (one cloth per rank, no collective).
"""
from __future__ import annotations

import argparse
import json
import os
import platform
import re
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "cloth vertex-steps/s"
UNIT = "vertex-steps/s"
KERNEL_PROFILE = os.path.join(ROOT, "profiles", "step_grid_c1.md")
GENERAL_PROFILE = os.path.join(ROOT, "profiles", "step_general_c1.md")


def algorithmic_bytes_per_vertex_step(n_vertices: int, n_struts: int) -> float:
    """Read pos+vel (32 B), write pos+vel (32 B), mass/pin (4 B) and each
    strut's (k, c, L) once (12 B per strut)."""
    return 64.0 + 4.0 + 12.0 * n_struts / n_vertices


def host_cpu():
    model = platform.processor() or platform.machine()
    try:
        for line in open("/proc/cpuinfo"):
            if line.lower().startswith(("model name", "cpu model")):
                model = line.split(":", 1)[1].strip()
                break
    except OSError:
        pass
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True).stdout
        m = re.search(r"Model name:\s*(.+)", out)
        if m:
            model = m.group(1).strip()
    except OSError:
        pass
    return model, os.cpu_count()


def profile_figure(path, key):
    """A `key: value` line of a committed ncu summary, or None."""
    try:
        m = re.search(r"^%s:\s*([0-9.eE+-]+)" % re.escape(key), open(path).read(), re.M)
    except OSError:
        return None
    return float(m.group(1)) if m else None


def profile_traffic(path=KERNEL_PROFILE, key="dram_bytes_per_launch"):
    """DRAM bytes per launch of the step kernel from the committed ncu summary."""
    try:
        txt = open(path).read()
    except OSError:
        return None
    m = re.search(key + r":\s*([0-9.eE+]+)", txt)
    return float(m.group(1)) if m else None


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.path = os.path.join("/tmp", "fgb_clocks_%d_%d.csv" % (os.getpid(), gpu_index))

    def __enter__(self):
        try:
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.FIELDS,
                                          "--format=csv,noheader,nounits", "-lms", "100"], stdout=self.f,
                                         stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
            self.f.close()

    def summary(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"], "samples": 0}
        rows = []
        for line in open(self.path):
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 9:
                rows.append(parts)
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = set()
        sm, smax = [], []
        for r in rows:
            try:
                sm.append(float(r[1]))
                smax.append(float(r[2]))
            except ValueError:
                continue
            for name, v in zip(names, r[5:9]):
                if v.lower() == "active":
                    reasons.add(name)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def time_cpu_reference(scene_fn, target_s: float, max_steps: int, warmup: int = 1, keep_points: bool = False):
    """Single-threaded oracle on a bounded sample of the workload: full steps
    of the same cloth until max_steps or target_s seconds are reached.  With
    keep_points (and no warm-up steps), the oracle's points after the timed
    steps from the initial state are returned as a second value."""
    import oracle
    from feriphys_gb300 import workloads as W

    scene = scene_fn()
    sim, mesh, _ = W.build(scene, oracle)
    for _ in range(max(0, warmup)):
        sim.step(1)  # page-in
    steps, t0 = 0, time.perf_counter()
    while steps < max(1, max_steps) and (steps == 0 or (time.perf_counter() - t0) < target_s):
        sim.step(1)
        steps += 1
    dt = time.perf_counter() - t0
    n = scene.n_vertices
    res = {"value": n * steps / dt, "unit": UNIT, "cores": 1, "kind": "port",
           "sample": "%d full steps of the %s cloth (%d vertices) on one host core (%s), %.1f s; the "
                     "reference's step is single-threaded (springy/simulation.rs:28)"
                     % (steps, scene.name, n, host_cpu()[0], dt),
           "seconds": dt, "steps": steps}
    if keep_points:
        return res, (mesh.get_points() if warmup <= 0 else None)
    return res


def time_cpu_batch_sample(batch, target_s: float, steps_per_cloth: int = 10, seed: int = 777):
    """The oracle on a bounded sample of a batch: seeded random cloths, each
    in a Simulation of its own (the reference's wind is global per
    Simulation, springy/config.rs:13), `steps_per_cloth` full steps each,
    until target_s seconds of stepping."""
    import oracle

    order = np.random.default_rng(seed).permutation(len(batch.cloths))
    c = batch.config
    vsteps, secs, used = 0, 0.0, 0
    for i in order:
        args, pins, wind = batch.cloths[int(i)]
        mesh = oracle.SpringyMesh.cloth(*args, pins)
        obstacles = [oracle.CollidableMesh(p, q) for p, q in batch.obstacles]
        sim = oracle.Simulation([mesh], obstacles)
        sim.set_config(oracle.Config.make(c["integration"], c["dt"], c["gravity"], wind, c["lift_coefficient"],
                                          c["drag_coefficient"], c["coefficient_of_restitution"],
                                          c["coefficient_of_friction"]))
        t0 = time.perf_counter()
        sim.step(steps_per_cloth)
        secs += time.perf_counter() - t0
        vsteps += args[0] * args[1] * steps_per_cloth
        used += 1
        if secs >= target_s:
            break
    return {"value": vsteps / secs, "unit": UNIT, "cores": 1, "kind": "port",
            "sample": "%d full steps of each of %d seeded random cloths of the batch (%d vertex-steps) on one host "
                      "core (%s), %.1f s; the reference steps its meshes one after another on one thread "
                      "(springy/simulation.rs:28)" % (steps_per_cloth, used, vsteps, host_cpu()[0], secs),
            "seconds": secs}


def rel_pos_error(a, b):
    """max |a - b| / max |b| over the positions of two Stateful point arrays."""
    a = np.asarray(a, np.float64)[:, 1:4]
    b = np.asarray(b, np.float64)[:, 1:4]
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-30))


def gpu_rollout(mesh, sim, init_points, checkpoints):
    """Points after each of the (ascending) step counts, from init_points."""
    mesh.set_points(init_points)
    out, done = {}, 0
    for c in checkpoints:
        sim.step(c - done)
        done = c
        out[c] = mesh.get_points()
    return out


def c1_workload(n: int, rollout: int) -> str:
    """The headline workload's name, identical in both arms (the counts are
    Cloth::new's: 3(n-1)^2 + 2(n-1) triangle struts, 2(n-2)^2 binding struts,
    2(n-1)^2 triangles)."""
    struts = 3 * (n - 1) ** 2 + 2 * (n - 1) + 2 * max(n - 2, 0) ** 2
    return ("c1 plain cloth %dx%d: %d vertices, %d struts, %d triangles; dt=1/600 Euler; plane + UV sphere "
            "(32x16); rollouts of %d steps from the initial state" % (n, n, n * n, struts, 2 * (n - 1) ** 2, rollout))


def run_reference(args, rank, world):
    """The reference arm: rank 0 times the reference's step on the host CPU
    (the oracle, a single-threaded C++ restatement: the reference itself is
    Rust and cannot be built here).  W warm-up steps, then exactly K timed
    steps, each one full step of the same cloth; rollouts restart from the
    initial state every --rollout steps outside the timed region, as in the
    GPU arm."""
    import oracle
    from feriphys_gb300 import workloads as W

    if rank != 0:
        return
    scene = W.c1(n=args.n)
    sim, mesh, _ = W.build(scene, oracle)
    init = mesh.get_points()
    for _ in range(args.warmup):
        sim.step(1)
    mesh.set_points(init)
    secs, since_reset = 0.0, 0
    for _ in range(args.steps):
        if since_reset == args.rollout:
            mesh.set_points(init)
            since_reset = 0
        t0 = time.perf_counter()
        sim.step(1)
        secs += time.perf_counter() - t0
        since_reset += 1
    n = scene.n_vertices
    value = n * args.steps / secs
    res = {"value": value, "unit": UNIT, "cores": 1, "kind": "port",
           "sample": "%d full steps of the %s cloth (%d vertices) on one host core (%s), %.1f s; the reference's "
                     "step is single-threaded (springy/simulation.rs:28)" % (args.steps, scene.name, n, host_cpu()[0],
                                                                              secs),
           "seconds": secs, "steps": args.steps}
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * secs / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded)",
            "config": {"workload": c1_workload(args.n, args.rollout), "cpu_threads": 1},
            "cpu_baseline": res,
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "note": "Rust reference not buildable here (no cargo/rustc); timed: the oracle's C++ restatement of the "
                    "reference's step, one thread like the reference"}
    print(json.dumps(line), flush=True)


def kernels_per_step(mesh, args):
    """Launches of this library's kernels per step (every step form is one)."""
    return 1


def run_batched(args, rank, world, dist, torch, fgb, W, emit=True):
    """4096 uneven cloths advanced together: rollouts of --rollout steps (100
    by default here) captured once as a CUDA graph and replayed; each rollout
    restarts from the initial state outside the timed region.  The working set
    (~3 GB) is far larger than L2, so no flush is needed."""
    rollout = args.rollout if args.rollout != 30 else 100
    t0 = time.perf_counter()
    batch = W.c2(n_cloths=args.cloths, seed=rank)
    sim, meshes, _ = W.build_batch(batch, fgb)
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    sim.set_stream(stream.cuda_stream)
    sim.step(0)  # device upload, batch build, autotune
    init = [m.get_points() for m in meshes]
    build_s = time.perf_counter() - t0
    n_vert = batch.n_vertices

    def reset():
        for m, p in zip(meshes, init):
            m.set_points(p)

    sim.step(rollout)  # graph capture + warm-up
    for _ in range(max(0, args.warmup - 1)):
        reset()
        sim.step(rollout)
    torch.cuda.synchronize()
    n_roll = max(1, args.steps // rollout)
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(n_roll)]
    nonfinite = 0
    if dist:
        dist.barrier()
    with ClockSampler(int(os.environ.get("LOCAL_RANK", "0"))) as clk:
        wall0 = time.perf_counter()
        for i in range(n_roll):
            reset()
            ev[i][0].record(stream)
            sim.step(rollout)
            ev[i][1].record(stream)
            torch.cuda.synchronize()
            nonfinite += int(sim.synchronize())
        wall = time.perf_counter() - wall0
    ms = float(np.mean([a.elapsed_time(b) for a, b in ev])) / rollout
    if dist:
        t = torch.tensor([ms], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
    value = world * n_vert / (ms * 1e-3)
    info = sim.batch_info()
    dt = batch.config["dt"]
    S = sum(int(m.counts()[1]) for m in meshes)
    B = algorithmic_bytes_per_vertex_step(n_vert, S)
    peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json"))) if os.path.exists(
        os.path.join(ROOT, "MEASURED_PEAKS.json")) else None
    peak = peaks["hbm_gbs"] if peaks else 6800.0
    achieved = B * n_vert / (ms * 1e-3) / 1e9
    parity = batch_fp64_parity(batch, fgb, W, [1, 10, rollout]) if rank == 0 else None
    cpu = time_cpu_batch_sample(batch, args.cpu_seconds / 2) if rank == 0 and world == 1 and not args.no_cpu else None
    line = None
    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": n_roll * rollout,
            "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded)",
            "config": {"workload": "c2 batched plain: %d cloths, side U{16..128} (%d vertices, %d struts), k x U(0.5,2), "
                                   "per-cloth wind, plane; dt=1/600 Euler; %d-step rollouts as one CUDA graph"
                                   % (len(meshes), n_vert, S, rollout),
                       "l2": "working set (%.1f GB) larger than L2, not flushed" % (B * n_vert / 1e9),
                       "launch": {"cloths": info[0], "tiles": info[1], "mode": ["per-tile CTAs", "persistent"][info[2]],
                                  "ctas": info[3], "tile": "32x%d" % info[4], "chosen_by": "autotuner"}},
            "simulated_seconds_per_s": world * dt / (ms * 1e-3),
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                         "traffic": profile_figure(os.path.join(ROOT, "profiles", "step_batched_c2.md"),
                                                   "dram_bytes_per_launch") if args.cloths == 4096 else None,
                         "algorithmic_bytes_per_launch": B * n_vert},
            "cpu_baseline": cpu, "e2e": None, "gpu_launches": n_roll * rollout, "parity": parity,
            "clocks": clk.summary(), "wall_s_timed": wall, "nonfinite_rollouts": nonfinite,
            "setup_s": build_s, "device": torch.cuda.get_device_name()}
        if emit:
            print(json.dumps(line), flush=True)
    del sim, meshes
    return line


def batch_fp64_parity(batch, fgb, W, checkpoints, n_sample=16, seed=12345):
    """A seeded sample of the batch's cloths advanced as a batch of their own
    (f32, the batched kernel: each cloth's result equals its result in the
    full batch) and each alone in f64 on the GPU, from the same initial state;
    the relative position error per cloth after each checkpoint."""
    rs = np.random.default_rng(seed)
    pick = sorted(rs.choice(len(batch.cloths), size=min(n_sample, len(batch.cloths)), replace=False).tolist())
    sub = W.Batch(batch.name + "-sample", batch.config, [batch.cloths[i] for i in pick], batch.obstacles)
    s32, m32, _ = W.build_batch(sub, fgb)
    s64, m64, _ = W.build_batch(sub, fgb)
    for m in m64:
        m.set_precision(64)
    out, done = {}, 0
    for c in sorted(set(checkpoints)):
        s32.step(c - done)
        s64.step(c - done)
        done = c
        errs, bad = [], 0
        for a, b in zip(m32, m64):
            pa, pb = a.get_points(), b.get_points_f64()
            if np.isfinite(pa).all() and np.isfinite(pb).all():
                errs.append(rel_pos_error(pa, pb))
            else:
                bad += 1
        out[str(c)] = {"median": float(np.median(errs)) if errs else None, "max": float(max(errs)) if errs else None,
                       "nonfinite_cloths": bad}
    return {"vs_fp64_gpu": {"cloths": len(pick), "rel_pos_err_after_steps": out,
                            "how": "a seeded sample of the cloths, batched f32 against each stepped alone in f64 on "
                                   "the GPU; max |x32 - x64| / max |x64| over positions, per cloth; cloths that go "
                                   "non-finite under the reference's Euler at dt = 1/600 are counted, not compared"}}


def rollout_error(p, f):
    """RMS position difference over the RMS spread of the reference positions."""
    p, f = p[:, 1:4].astype(np.float64), f[:, 1:4].astype(np.float64)
    return float(np.sqrt(((p - f) ** 2).sum(1).mean()) / np.sqrt(((f - f.mean(0)) ** 2).sum(1).mean()))


SURROGATE_FLOPS_PER_VERTEX = 2 * (54 * 128 + 128 * 128 + 128 * 3)  # 47,360 algorithmic
SURROGATE_MMA_FLOPS_PER_VERTEX = 2 * (64 * 128 + 128 * 128 + 128 * 16)  # as issued (padded K and N)


def run_surrogate(args, rank, world, dist, torch, fgb, W, emit=True):
    """c3: the learned surrogate on the 1024^2 cloth; c4: on 4096 uneven cloths.

    The reference's explicit Euler is unstable at dt = 1/600 s on these cloths
    (the 1024^2 cloth goes non-finite at step 62; at 1/6000 s after ~3,600
    steps, at any position noise), so the fine solver that generates the
    training data and measures the surrogate runs at --fine-dt (1/30000 s by
    default: finite through the whole evaluation; at 1/6000 s some of the
    uneven cloths also go non-finite within 3000 steps), and one coarse step
    is `ratio` (10) fine steps.
    Training data: seeded cloths of the evaluated kind (c3: 256^2 cloths with
    the large cloth's spacing, stiffness jitter and noise; c4: a 256-cloth
    batch of the uneven kind), one snapshot every --collect-skip coarse
    steps, into the device ring.  Then Adam on batches of 65,536 rows.  The
    evaluation rolls the surrogate out for --coarse-steps coarse steps (with
    the energy/strain checks and per-cloth fine-step fallback) next to the
    fine solver over the same simulated time, from the same initial state."""
    ratio = args.ratio
    if args.train_steps <= 0:
        args.train_steps = 3000 if args.workload == "c3" else 20000
    if args.ring <= 0:
        args.ring = (16 if args.workload == "c3" else 32) * 1024 * 1024
    if args.collect_skip <= 0:
        args.collect_skip = 60 if args.workload == "c3" else max(1, args.coarse_steps // 20)
    dt_f = args.fine_dt if args.fine_dt > 0 else 1.0 / 30000.0
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    t_setup = time.perf_counter()
    sur = fgb.Surrogate.new(1234 + rank)
    if args.workload == "c3":
        n = args.n
        train_side = min(args.train_side, n)
        ring = args.ring
        sur.reserve(ring)
        per_cloth = max(1, ring // (args.train_cloths * train_side * train_side))
        for k in range(args.train_cloths):
            sc = W.c1(n=train_side, side=(train_side - 1) / (n - 1), dt=dt_f, seed=1000 + k)
            tsim, _, _ = W.build(sc, fgb)
            for _ in range(per_cloth):
                sur.collect(tsim, ratio, 1)
                tsim.step(ratio * args.collect_skip)
            del tsim
        eval_scene = W.c1(n=n, dt=dt_f, seed=rank)

        def build_eval():
            sim, mesh, _ = W.build(eval_scene, fgb)
            return sim, [mesh]

        workload = ("c3 surrogate: %dx%d cloth (the plain large config), fine dt=%.3g s Euler, coarse step = %d fine "
                    "steps; trained on %d seeded %dx%d cloths of the same spacing" % (n, n, dt_f, ratio,
                                                                                    args.train_cloths, train_side,
                                                                                    train_side))
    else:
        tb = W.c2(n_cloths=args.train_cloths * 64, seed=1000, dt=dt_f)
        tsim, tmeshes, _ = W.build_batch(tb, fgb)
        ring = args.ring
        sur.reserve(ring)
        per = max(1, ring // tb.n_vertices)
        noise_rng = np.random.default_rng(4242)
        perturb = args.train_noise_p > 0 or args.train_noise_v > 0
        for snap in range(per):
            if perturb and snap % 2 == 1:
                # every other snapshot is taken from a perturbed copy of the state (free vertices: positions
                # + N(0, noise_p h), velocities + N(0, noise_v h / T)), so the network also learns the
                # dynamics just off the trajectory, where its own steps drift; the clean state is then
                # restored and the trajectory continues from it
                saved = [m.get_points() for m in tmeshes]
                for m, pts, (cargs, pins, _) in zip(tmeshes, saved, tb.cloths):
                    h = cargs[2]
                    q = pts.copy()
                    free = np.ones(len(q), bool)
                    free[np.asarray(pins, np.int64)] = False
                    q[free, 1:4] += noise_rng.normal(0.0, args.train_noise_p * h, (int(free.sum()), 3))
                    q[free, 4:7] += noise_rng.normal(0.0, args.train_noise_v * h / (ratio * dt_f),
                                                     (int(free.sum()), 3))
                    m.set_points(q)
                sur.collect(tsim, ratio, 1)
                for m, pts in zip(tmeshes, saved):
                    m.set_points(pts)
                tsim.step(ratio * (args.collect_skip + 1))
            else:
                sur.collect(tsim, ratio, 1)
                tsim.step(ratio * args.collect_skip)
        del tsim, tmeshes
        eb = W.c2(n_cloths=args.cloths, seed=rank, dt=dt_f)

        def build_eval():
            sim, meshes, _ = W.build_batch(eb, fgb)
            return sim, meshes

        workload = ("c4 batched surrogate: %d uneven cloths (side U{16..128}), fine dt=%.3g s Euler, coarse step = "
                    "%d fine steps; trained on a %d-cloth batch of the same kind" % (args.cloths, dt_f, ratio,
                                                                                    args.train_cloths * 64))
    rows, _ = sur.dataset_info()
    sur.fit_normalization()
    collect_s = time.perf_counter() - t_setup
    torch.cuda.synchronize()
    t1 = time.perf_counter()
    a = int(args.train_steps * 2 // 3)
    losses = np.concatenate([sur.train(a, 65536, 3e-3, seed=1), sur.train(args.train_steps - a, 65536, 1e-3, seed=2)])
    torch.cuda.synchronize()
    train_s = time.perf_counter() - t1

    # fine reference over the same simulated time (timed: one event pair around each coarse interval)
    psim, pmeshes = build_eval()
    psim.set_stream(stream.cuda_stream)
    psim.step(0)
    n_vert = sum(m.n_points for m in pmeshes)
    checkpoints = sorted({c for c in (1, 10, 100, 300, args.coarse_steps) if c <= args.coarse_steps})
    refs, plain_cum = {}, {}
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    done = 0
    plain_ms = 0.0
    for c in checkpoints:
        e0.record(stream)
        psim.step(ratio * (c - done))
        e1.record(stream)
        torch.cuda.synchronize()
        plain_ms += e0.elapsed_time(e1)
        plain_cum[c] = plain_ms
        done = c
        refs[c] = [m.get_points() for m in pmeshes]
    plain_fine_ms = plain_ms / (ratio * args.coarse_steps)
    del psim, pmeshes

    # FP64 rerun of the fine solver on the GPU (c3: the cloth; c4: a seeded sample of 16 cloths), the
    # oracle both the f32 fine solver and the surrogate are measured against below
    if args.workload == "c3":
        pick = [0]
        sim64, meshes64 = build_eval()
    else:
        rs = np.random.default_rng(12345)
        pick = sorted(rs.choice(len(eb.cloths), size=min(16, len(eb.cloths)), replace=False).tolist())
        sim64, meshes64, _ = W.build_batch(W.Batch(eb.name + "-sample", eb.config, [eb.cloths[i] for i in pick],
                                                   eb.obstacles), fgb)
    for m in meshes64:
        m.set_precision(64)
    ref64, done = {}, 0
    for c in checkpoints:
        sim64.step(ratio * (c - done))
        done = c
        ref64[c] = [m.get_points_f64() for m in meshes64]
    del sim64, meshes64

    # surrogate: kernel-only timing (no checks), then the checked rollout
    ssim, smeshes = build_eval()
    ssim.set_stream(stream.cuda_stream)
    ssim.step(0)
    init = [m.get_points() for m in smeshes]

    def reset():
        for m, p in zip(smeshes, init):
            m.set_points(p)

    k_kernel = 50
    ssim.step_surrogate(sur, ratio, 5)
    reset()
    e0.record(stream)
    ssim.step_surrogate(sur, ratio, k_kernel)
    e1.record(stream)
    torch.cuda.synchronize()
    kernel_ms = e0.elapsed_time(e1) / k_kernel
    reset()
    chk = fgb.SurrogateCheck.make(energy_growth=args.energy_growth, energy_abs=1e-3, max_strain=args.max_strain)
    errors, errors64, fallbacks, done, sur_ms = {}, {}, 0, 0, 0.0
    n_cloths_eval = len(smeshes)
    horizon = {}
    with ClockSampler(int(os.environ.get("LOCAL_RANK", "0"))) as clk:
        for c in checkpoints:
            e0.record(stream)
            fallbacks += ssim.step_surrogate(sur, ratio, c - done, chk)
            e1.record(stream)
            torch.cuda.synchronize()
            sur_ms += e0.elapsed_time(e1)
            done = c
            # over the first c coarse steps: the same simulated time c*T in both solvers
            horizon[c] = {"speedup_vs_plain": plain_cum[c] / sur_ms,
                          "fallback_fraction": fallbacks / float(n_cloths_eval * c)}
            pts = [m.get_points() for m in smeshes]
            ref_ok = np.array([np.isfinite(f).all() for f in refs[c]])
            sur_ok = np.array([np.isfinite(p).all() for p in pts])
            per_cloth = np.array([rollout_error(p, f) if a and b else np.nan
                                  for p, f, a, b in zip(pts, refs[c], sur_ok, ref_ok)])
            fin = per_cloth[np.isfinite(per_cloth)]
            errors[c] = {"mean": float(fin.mean()) if fin.size else None, "max": float(fin.max()) if fin.size else None,
                         "median": float(np.median(fin)) if fin.size else None,
                         "nonfinite_fine": int((~ref_ok).sum()), "nonfinite_surrogate": int((~sur_ok).sum())}
            e_fine, e_sur = [], []
            for k, i in enumerate(pick):
                r64 = ref64[c][k]
                if not np.isfinite(r64).all():
                    continue
                if ref_ok[i]:
                    e_fine.append(rollout_error(refs[c][i], r64))
                if sur_ok[i]:
                    e_sur.append(rollout_error(pts[i], r64))
            errors64[c] = {"fine_f32": float(np.median(e_fine)) if e_fine else None,
                           "surrogate": float(np.median(e_sur)) if e_sur else None}
            horizon[c]["median_rel_pos_err"] = errors[c]["median"]
            horizon[c]["max_rel_pos_err"] = errors[c]["max"]
    coarse_ms = sur_ms / args.coarse_steps
    T = ratio * np.float32(dt_f)
    value = world * n_vert * ratio / (coarse_ms * 1e-3)
    plain_value = world * n_vert / (plain_fine_ms * 1e-3)
    peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json"))) if os.path.exists(
        os.path.join(ROOT, "MEASURED_PEAKS.json")) else None
    peak = peaks["bf16_tflops"] if peaks else 1900.0
    achieved = SURROGATE_FLOPS_PER_VERTEX * n_vert / (kernel_ms * 1e-3) / 1e12
    line = None
    if rank == 0:
        line = {
            "metric": "cloth vertex-steps/s (fine-step equivalents) with the learned surrogate", "value": value,
            "unit": UNIT, "n_gpus": world, "steps": args.coarse_steps, "warmup": 5,
            "ms_per_step": coarse_ms, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "bf16 (MLP, f32 accumulate) / f32 (state)", "data": "synthetic (seeded)",
            "config": {"workload": workload, "vertices": n_vert, "ratio": ratio, "coarse_dt": float(T),
                       "fine_dt": dt_f, "checks": {"energy_growth": args.energy_growth, "max_strain": args.max_strain},
                       "l2": "working set larger than L2 (c4) / one cloth of 1M vertices (c3): not flushed"},
            "error_vs_fine": {str(k): v for k, v in errors.items()},
            "error_vs_fp64_fine": {"after_coarse_steps": {str(k): v for k, v in errors64.items()},
                                   "cloths": len(pick),
                                   "how": "the fine solver rerun in f64 on the GPU from the same initial state; "
                                          "median over the compared cloths of the same relative RMS position "
                                          "error as error_vs_fine, for the f32 fine solver and for the surrogate"},
            "fallbacks": fallbacks,
            "fallback_fraction": fallbacks / float(n_cloths_eval * args.coarse_steps),
            "by_horizon": {str(k): v for k, v in horizon.items()},
            "target": ">= 5x the simulated seconds per second of the plain solver at <= 1e-2 relative "
                      "position error after 1000 coarse steps; by_horizon gives the speed-up over the first c "
                      "coarse steps and the error after them",
            "simulated_seconds_per_s": {"surrogate": float(T) / (coarse_ms * 1e-3),
                                        "plain_fine": dt_f / (plain_fine_ms * 1e-3),
                                        "ratio": (float(T) / coarse_ms) / (dt_f / plain_fine_ms)},
            "plain_fine_vertex_steps_per_s": plain_value,
            "roofline": {"bound": "tensor", "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                         "frac": achieved / peak, "traffic": None,
                         "algorithmic_flops_per_launch": SURROGATE_FLOPS_PER_VERTEX * n_vert,
                         "kernel_ms": kernel_ms,
                         "mma_issued_tflops": SURROGATE_MMA_FLOPS_PER_VERTEX * n_vert / (kernel_ms * 1e-3) / 1e12,
                         "tensor_pipe_active_pct": profile_figure(os.path.join(ROOT, "profiles", "surrogate_step_c3.md"),
                                                                  "tensor_pipe_active_pct"),
                         "note": "k_sur_step: features + 3 MMA layers + GELU epilogues + integration in one launch; "
                                 "achieved and mma_issued_tflops measured in this run (CUDA events, the padded "
                                 "K = 64 / N = 16 MMA shapes for the latter); tensor_pipe_active_pct is "
                                 "sm__pipe_tensor_cycles_active from the committed ncu summary "
                                 "profiles/surrogate_step_c3.md"},
            "training": {"rows": rows, "collect_and_setup_s": collect_s, "steps": int(args.train_steps),
                         "batch": 65536, "seconds": train_s, "samples_per_s": args.train_steps * 65536 / train_s,
                         "loss_first": float(losses[0]), "loss_last": float(losses[-1])},
            "cpu_baseline": None, "e2e": None, "gpu_launches": None,
            "clocks": clk.summary(), "device": torch.cuda.get_device_name()}
        if emit:
            print(json.dumps(line), flush=True)
    del ssim, smeshes, sur
    return line


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=2000)
    ap.add_argument("--warmup", type=int, default=20)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--n", "--side", dest="n", type=int, default=1024, help="cloth side in vertices")
    ap.add_argument("--rollout", type=int, default=30)
    ap.add_argument("--e2e-steps", type=int, default=50)
    ap.add_argument("--cpu-seconds", type=float, default=20.0)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-extras", action="store_true",
                    help="c1 only: leave out the batched (c2) and batched-surrogate (c4) results of the line")
    ap.add_argument("--path", type=int, default=0,
                    help="0 auto, 1 general gather, 2 tiled grid, 3 untiled grid, 4 general gather (plain lists)")
    ap.add_argument("--probe", action="store_true", help="report the first step whose state is non-finite")
    ap.add_argument("--workload", default="c1", choices=["c1", "c2", "c3", "c4"],
                    help="c1: one 1024x1024 cloth (default); c2: 4096 uneven cloths, one launch per step; "
                         "c3/c4: the learned surrogate on c1/c2")
    ap.add_argument("--cloths", type=int, default=4096)
    ap.add_argument("--ratio", type=int, default=10, help="fine steps per surrogate coarse step")
    ap.add_argument("--coarse-steps", type=int, default=1000)
    ap.add_argument("--fine-dt", type=float, default=0.0, help="fine step of the surrogate workloads (0: default)")
    ap.add_argument("--train-steps", type=int, default=0, help="Adam steps (0: c3 3000, c4 20000)")
    ap.add_argument("--train-cloths", type=int, default=4)
    ap.add_argument("--train-side", type=int, default=256, help="c3: side of the training cloths")
    ap.add_argument("--ring", type=int, default=0, help="dataset ring rows (0: c3 16M, c4 32M)")
    ap.add_argument("--collect-skip", type=int, default=0,
                    help="coarse steps between collected snapshots (0: c3 60; c4 coarse-steps/20, so that the "
                         "snapshots span the evaluated horizon)")
    ap.add_argument("--train-noise-p", type=float, default=0.0,
                    help="c4: position noise (fraction of the rest spacing) of every other training snapshot")
    ap.add_argument("--train-noise-v", type=float, default=0.0,
                    help="c4: velocity noise (fraction of spacing per coarse step) of every other training snapshot")
    ap.add_argument("--energy-growth", type=float, default=0.05)
    ap.add_argument("--max-strain", type=float, default=1000.0)
    args = ap.parse_args()

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))

    if args.impl == "reference":
        if world > 1:
            import torch.distributed as dist

            dist.init_process_group("gloo")
        run_reference(args, rank, world)
        if world > 1:
            dist.barrier()
            dist.destroy_process_group()
        return

    import torch

    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl", device_id=torch.device("cuda", local))

    import feriphys_gb300 as fgb
    from feriphys_gb300 import workloads as W

    if args.workload in ("c2", "c3", "c4"):
        (run_batched if args.workload == "c2" else run_surrogate)(args, rank, world, dist, torch, fgb, W)
        if dist:
            dist.barrier()
            dist.destroy_process_group()
        return

    scene = W.c1(n=args.n, seed=rank)
    sim, mesh, _ = W.build(scene, fgb)
    mesh.set_path(args.path)
    stream = torch.cuda.Stream()  # a real stream handle (the legacy default stream's is 0)
    torch.cuda.set_stream(stream)
    sim.set_stream(stream.cuda_stream)
    n_vert, n_struts, n_faces, _ = mesh.counts()
    init_points = mesh.get_points()

    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")

    if args.probe:
        mesh.set_points(init_points)
        first = None
        for i in range(1, args.steps + 1):
            sim.step(1)
            if sim.synchronize():
                first = i
                break
        print(json.dumps({"probe": scene.name, "first_nonfinite_step": first, "checked_steps": args.steps}))
        return

    def reset():
        mesh.set_points(init_points)

    # warm-up
    reset()
    for i in range(args.warmup):
        sim.step(1)
    torch.cuda.synchronize()
    reset()

    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    nonfinite_steps = 0
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    with ClockSampler(local) as clk:
        wall0 = time.perf_counter()
        done = 0
        while done < args.steps:
            chunk = min(args.rollout, args.steps - done)
            for j in range(chunk):
                flush.zero_()
                starts[done + j].record(stream)
                sim.step(1)
                ends[done + j].record(stream)
            done += chunk
            torch.cuda.synchronize()
            if sim.synchronize():
                nonfinite_steps += 1
            if done < args.steps:
                reset()  # next rollout from the initial state (outside the events)
        torch.cuda.synchronize()
        wall = time.perf_counter() - wall0
    if dist:
        dist.barrier()
    times = np.array([s.elapsed_time(e) for s, e in zip(starts, ends)], np.float64)  # ms
    ms_step = float(times.mean())
    ms_median = float(np.median(times))
    if dist:
        t = torch.tensor([ms_step], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms_step = float(t.item())
    value = world * n_vert / (ms_step * 1e-3)

    # end to end through the C ABI with host buffers
    pinned = torch.empty((n_vert, 10), dtype=torch.float32, pin_memory=True)
    pinned.numpy()[:] = init_points
    host = pinned.numpy()
    sim.set_stream(None)
    for _ in range(3):
        mesh.set_points(host)
        sim.step(1)
        mesh.get_points(out=host)
    pinned.numpy()[:] = init_points
    t0 = time.perf_counter()
    for i in range(args.e2e_steps):
        mesh.set_points(host)
        sim.step(1)
        mesh.get_points(out=host)
    e2e_s = (time.perf_counter() - t0) / args.e2e_steps
    if dist:
        t = torch.tensor([e2e_s], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        e2e_s = float(t.item())
    e2e = {"value": world * n_vert / e2e_s, "unit": UNIT, "h2d_bytes_per_step": 40 * n_vert,
           "d2h_bytes_per_step": 40 * n_vert, "ms_per_step": 1e3 * e2e_s,
           "path": "fgb_mesh_set_points + fgb_sim_step + fgb_mesh_get_points, pinned host buffers"}

    # end to end in the shape of the reference's render loop (demos/cloth.rs:107-138): the state stays on
    # the GPU, every step is followed by a read of the positions only (12 B per vertex) into pinned memory;
    # rollouts restart from the initial state every --rollout steps outside the timed region
    pos_pinned = torch.empty((n_vert, 3), dtype=torch.float32, pin_memory=True)
    pos_host = pos_pinned.numpy()
    mesh.set_points(init_points)
    for _ in range(3):
        sim.step(1)
        mesh.get_positions(out=pos_host)
    mesh.set_points(init_points)
    pos_s, since = 0.0, 0
    for i in range(args.e2e_steps):
        if since == args.rollout:
            mesh.set_points(init_points)
            since = 0
        t0 = time.perf_counter()
        sim.step(1)
        mesh.get_positions(out=pos_host)
        pos_s += time.perf_counter() - t0
        since += 1
    pos_s /= args.e2e_steps
    if dist:
        t = torch.tensor([pos_s], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        pos_s = float(t.item())
    e2e_positions = {"value": world * n_vert / pos_s, "unit": UNIT, "h2d_bytes_per_step": 0,
                     "d2h_bytes_per_step": 12 * n_vert, "ms_per_step": 1e3 * pos_s,
                     "path": "fgb_sim_step + fgb_mesh_get_positions into a pinned host buffer (state resident on "
                             "the GPU, positions read back every step, as a render loop does)"}
    del pos_pinned, pos_host

    peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json"))) if os.path.exists(
        os.path.join(ROOT, "MEASURED_PEAKS.json")) else None
    peak = peaks["hbm_gbs"] if peaks else 6800.0
    B = algorithmic_bytes_per_vertex_step(n_vert, n_struts)
    achieved = B * n_vert / (ms_step * 1e-3) / 1e9
    # DRAM bytes per launch of the 1024^2 step from the committed ncu summaries
    path_used = args.path if args.path in (3, 4) else mesh.get_path()
    traffic = {2: profile_traffic(), 1: profile_traffic(GENERAL_PROFILE),
               4: profile_traffic(GENERAL_PROFILE, "dram_bytes_per_launch_plain")}.get(path_used) if args.n == 1024 else None
    roofline = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                "traffic": traffic, "algorithmic_bytes_per_launch": B * n_vert,
                "peak_source": "MEASURED_PEAKS.json hbm_gbs (measured)" if peaks else "fallback 6.8 TB/s"}

    # error of the timed f32 step against an FP64 rerun of the same step on the GPU and against the
    # reference's CPU step (the oracle restatement), from the same initial state
    parity = None
    cpu = None
    if rank == 0:
        cps = sorted({c for c in (1, 2, 5, 10, 20, args.rollout) if 1 <= c <= max(1, args.rollout)})
        p32 = gpu_rollout(mesh, sim, init_points, cps)
        sim64, mesh64, _ = W.build(scene, fgb)
        mesh64.set_precision(64)
        p64 = gpu_rollout(mesh64, sim64, init_points, cps)
        del sim64, mesh64
        parity = {"vs_fp64_gpu": {"rel_pos_err_after_steps": {str(c): rel_pos_error(p32[c], p64[c]) for c in cps},
                                  "how": "the same cloth stepped in f64 on the GPU (general gather path) from the "
                                         "same initial state, max |x32 - x64| / max |x64| over positions; at this "
                                         "dt the reference's Euler diverges on this cloth (non-finite at step 62), "
                                         "which amplifies rounding differences from step ~20 on"}}
        if world == 1 and not args.no_cpu:
            cpu, ref_pts = time_cpu_reference(lambda: W.c1(n=args.n), args.cpu_seconds, 60, warmup=0,
                                              keep_points=True)
            g_pts = gpu_rollout(mesh, sim, init_points, [cpu["steps"]])[cpu["steps"]]
            parity["vs_cpu_reference"] = {"steps": cpu["steps"], "rel_pos_err": rel_pos_error(g_pts, ref_pts),
                                          "kind": "port",
                                          "how": "the oracle's points after the CPU baseline's timed steps"}

    # the rows either side of the step: SpringyMesh::new's strut de-duplication on the host and on the
    # GPU (the same mesh), and the ColoredVertex render export from the device state
    around = None
    if rank == 0:
        t0 = time.perf_counter()
        m_host = fgb.SpringyMesh.new(scene.positions, scene.indices, scene.mass, 1.0, 1.0)
        host_s = time.perf_counter() - t0
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        m_dev = fgb.SpringyMesh.new(scene.positions, scene.indices, scene.mass, 1.0, 1.0, build_on_device=True)
        torch.cuda.synchronize()
        dev_s = time.perf_counter() - t0
        (kh, ah), (kd, ad) = m_host.get_struts(), m_dev.get_struts()
        same = bool(np.array_equal(ah, ad) and kh.tobytes() == kd.tobytes())
        n_tri_struts = len(ah)
        del m_host, m_dev
        buf = torch.empty(n_vert * 9, dtype=torch.float32, device="cuda")
        mesh.export_vertices(buf.data_ptr(), stream_handle=stream.cuda_stream)  # the first call uploads its face lists
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(20):
            mesh.export_vertices(buf.data_ptr(), stream_handle=stream.cuda_stream)
        e1.record(stream)
        torch.cuda.synchronize()
        exp_ms = e0.elapsed_time(e1) / 20
        around = {"mesh_build": {"host_s": host_s, "device_s": dev_s, "identical": same,
                                 "how": "SpringyMesh::new of this cloth's positions and triangles (%d struts "
                                        "de-duplicated from the triangle edges) through fgb_mesh_new and "
                                        "fgb_mesh_new_device, wall clock" % n_tri_struts},
                  "render_export": {"ms": exp_ms, "vertices": n_vert, "bytes_written": 36 * n_vert,
                                    "how": "fgb_mesh_export_vertices: ColoredVertex (position, color, normal "
                                           "summed over the vertex's faces) into a device buffer, CUDA events"}}
        del buf

    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded)",
                "config": {"workload": c1_workload(args.n, args.rollout),
                           "l2": "flushed (256 MB write) before every timed step",
                           "parallelism": "replicas" if world > 1 else "single GPU",
                           "path": {1: "general gather", 2: "tiled grid stencil", 3: "untiled grid stencil",
                                    4: "general gather (plain lists)"}[path_used]},
                "ms_per_step_median": ms_median,
                "roofline": roofline, "cpu_baseline": cpu, "e2e": e2e, "e2e_positions": e2e_positions,
                "parity": parity, "around_the_step": around,
                "gpu_launches": args.steps * kernels_per_step(mesh, args),
                "clocks": clk.summary(), "wall_s_timed": wall, "nonfinite_rollouts": nonfinite_steps,
                "device": torch.cuda.get_device_name()}
    # the other half of the metric: the uneven-cloth batch, plain and with the learned surrogate
    # (each its own timed region, after the headline's)
    extras = [] if args.no_extras else ["batched", "surrogate"]
    if extras:
        del sim, mesh, flush
        torch.cuda.synchronize()
        sub = argparse.Namespace(**vars(args))
        sub.rollout = 100
        sub.steps = max(args.steps, 100)
        sub.workload = "c2"
        b = run_batched(sub, rank, world, dist, torch, fgb, W, emit=False)
        torch.cuda.synchronize()
        sub = argparse.Namespace(**vars(args))
        sub.workload = "c4"
        su = run_surrogate(sub, rank, world, dist, torch, fgb, W, emit=False)
        if rank == 0:
            line["batched"] = b
            line["surrogate"] = su
    if rank == 0:
        print(json.dumps(line), flush=True)
    if dist:
        dist.barrier()
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
