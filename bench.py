"""Benchmark: cloth vertex-steps/s on one GB300 (large plain cloth).

Workload: the 1024 x 1024 plain cloth (1,048,576 vertices, 5,230,601 struts,
2,093,058 triangles; per-strut stiffness within +-10%, N(0, 1e-3) position
noise, top row pinned, wind, drag/lift, plane + UV-sphere colliders,
explicit Euler at dt = 1/600 s) built by feriphys_gb300.workloads.c1 on
synthetic seeded data.  A "step" is one Simulation::step of that cloth.
Rollouts restart from the initial state every --rollout steps outside the
timed region: 50 by default, because explicit Euler at the configured dt
makes this cloth's state non-finite at step 62 (bench.py --probe), and every
timed step should run on finite data.

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


def profile_traffic():
    """DRAM bytes per launch of the step kernel from the committed ncu summary."""
    try:
        txt = open(KERNEL_PROFILE).read()
    except OSError:
        return None
    m = re.search(r"dram_bytes_per_launch:\s*([0-9.eE+]+)", txt)
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


def time_cpu_reference(scene_fn, target_s: float, max_steps: int, warmup: int = 1):
    """Single-threaded oracle on a bounded sample of the workload: full steps
    of the same cloth until max_steps or target_s seconds are reached."""
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
    return {"value": n * steps / dt, "unit": UNIT, "cores": 1, "kind": "port",
            "sample": "%d full steps of the %s cloth (%d vertices) on one host core (%s), %.1f s; the "
                      "reference's step is single-threaded (springy/simulation.rs:28)"
                      % (steps, scene.name, n, host_cpu()[0], dt),
            "seconds": dt, "steps": steps}


def run_reference(args, rank, world):
    """The reference arm: rank 0 times the CPU implementation; each of the K
    steps is one full step of the same cloth, capped by --cpu-seconds overall
    so that any --steps/--warmup finishes within a few minutes."""
    from feriphys_gb300 import workloads as W

    if rank != 0:
        return
    res = time_cpu_reference(lambda: W.c1(n=args.n), args.cpu_seconds, args.steps, warmup=min(args.warmup, 1))
    value = res["value"]
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * res["seconds"] / res["steps"],
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded)",
            "config": {"workload": "c1 plain cloth %dx%d (%d vertices), dt=1/600, Euler, plane+sphere"
                                   % (args.n, args.n, args.n * args.n), "cpu_threads": 1,
                       "timed_steps": res["steps"]},
            "cpu_baseline": res,
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "note": "Rust reference not buildable here (no cargo/rustc); timed: the oracle's C++ restatement"}
    print(json.dumps(line), flush=True)


def kernels_per_step(mesh, args):
    """Launches of this library's kernels per step (every step form is one)."""
    return 1


def run_batched(args, rank, world, dist, torch, fgb, W):
    """4096 uneven cloths advanced together: rollouts of --rollout steps (100
    by default here) captured once as a CUDA graph and replayed; each rollout
    restarts from the initial state outside the timed region.  The working set
    (~3 GB) is far larger than L2, so no flush is needed."""
    rollout = args.rollout if args.rollout != 50 else 100
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
    if rank == 0:
        print(json.dumps({
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": n_roll * rollout,
            "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded)",
            "config": {"workload": "c2 batched plain: %d cloths, side U{16..128} (%d vertices, %d struts), k x U(0.5,2), "
                                   "per-cloth wind, plane; dt=1/600 Euler; %d-step rollouts as one CUDA graph"
                                   % (len(meshes), n_vert, S, rollout),
                       "l2": "working set (%.1f GB) larger than L2, not flushed" % (B * n_vert / 1e9),
                       "launch": {"cloths": info[0], "tiles": info[1], "mode": ["per-tile CTAs", "persistent"][info[2]],
                                  "ctas": info[3]}},
            "simulated_seconds_per_s": world * dt / (ms * 1e-3),
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                         "traffic": None, "algorithmic_bytes_per_launch": B * n_vert},
            "cpu_baseline": None, "e2e": None, "gpu_launches": n_roll * rollout,
            "clocks": clk.summary(), "wall_s_timed": wall, "nonfinite_rollouts": nonfinite,
            "setup_s": build_s, "device": torch.cuda.get_device_name()}), flush=True)
    if dist:
        dist.barrier()
        dist.destroy_process_group()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=2000)
    ap.add_argument("--warmup", type=int, default=20)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--n", type=int, default=1024, help="cloth side in vertices")
    ap.add_argument("--rollout", type=int, default=50)
    ap.add_argument("--e2e-steps", type=int, default=50)
    ap.add_argument("--cpu-seconds", type=float, default=20.0)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--path", type=int, default=0, help="0 auto, 1 general gather, 2 tiled grid, 3 untiled grid")
    ap.add_argument("--probe", action="store_true", help="report the first step whose state is non-finite")
    ap.add_argument("--workload", default="c1", choices=["c1", "c2"],
                    help="c1: one 1024x1024 cloth (default); c2: 4096 uneven cloths, one launch per step")
    ap.add_argument("--cloths", type=int, default=4096)
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

    if args.workload == "c2":
        return run_batched(args, rank, world, dist, torch, fgb, W)

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

    peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json"))) if os.path.exists(
        os.path.join(ROOT, "MEASURED_PEAKS.json")) else None
    peak = peaks["hbm_gbs"] if peaks else 6800.0
    B = algorithmic_bytes_per_vertex_step(n_vert, n_struts)
    achieved = B * n_vert / (ms_step * 1e-3) / 1e9
    traffic = profile_traffic()
    roofline = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                "traffic": traffic, "algorithmic_bytes_per_launch": B * n_vert,
                "peak_source": "MEASURED_PEAKS.json hbm_gbs (measured)" if peaks else "fallback 6.8 TB/s"}

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        cpu = time_cpu_reference(lambda: W.c1(n=args.n), args.cpu_seconds, 60, warmup=0)

    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded)",
                "config": {"workload": "c1 plain cloth %dx%d: %d vertices, %d struts, %d triangles; dt=1/600 "
                                       "Euler; plane + UV sphere (32x16); rollouts of %d steps from the "
                                       "initial state" % (args.n, args.n, n_vert, n_struts, n_faces, args.rollout),
                           "l2": "flushed (256 MB write) before every timed step",
                           "parallelism": "replicas" if world > 1 else "single GPU",
                           "path": {1: "general gather", 2: "tiled grid stencil", 3: "untiled grid stencil"}[3 if args.path == 3 else mesh.get_path()]},
                "roofline": roofline, "cpu_baseline": cpu, "e2e": e2e,
                "gpu_launches": args.steps * kernels_per_step(mesh, args),
                "clocks": clk.summary(), "wall_s_timed": wall, "nonfinite_rollouts": nonfinite_steps,
                "device": torch.cuda.get_device_name()}
        print(json.dumps(line), flush=True)
    if dist:
        dist.barrier()
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
