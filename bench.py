#!/usr/bin/env python3
"""Throughput of the MPS time step on one GB300: particle-steps/s.

Default workload: the 1M-particle 2-D dam break (water column 0.5 x 1.0 m,
l0 = 0.5/707 m so the column is 707 x 1414 = 999,698 fluid particles, tank
2.0 x 1.2 m with 2 wall and 2 dummy layers, dt = 5e-5 s, the reference's
physics with radii 3.1/3.1/2.1 l0), synthetic and seeded, solved with the
mixed-precision PPE solver (FP32 Krylov iterations, FP64 dot products and
FP64 residual refinement to 1e-10).  The same steps are also timed with the
plain FP64 solver (the reference's Jacobi-CG at machine-epsilon tolerance).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

One JSON line on stdout (rank 0).  `value` is device-timed throughput of K
steps with the state resident in HBM (CUDA events on the engine's stream);
`e2e` is the same steps through the C ABI with the host-owned particle
arrays copied in (pinned) and the step's results copied out every step.
`--impl reference` times the CPU oracle (the reference's algorithm restated
in C++/OpenMP, the reference's own sources need Eigen which is absent) on
this machine's host cores.  Multi-GPU runs are independent replicas (the
method has no data-parallel split of one scene); value sums all ranks.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time

import numpy as np

REPO = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, REPO)

METRIC = "particle-steps/s at 1M particles: mixed-precision vs plain FP64, same GB300"
UNIT = "particle-steps/s"


def workload(name: str):
    from mps_gb300 import scenes

    if name == "dambreak_1m":   # mixed-precision 1M workload
        l0 = 0.5 / 707
        return scenes.dam_break(l0, tank=(2.0, 1.2), column=(0.5, 1.0), dt=5e-5)
    if name == "dambreak_2m":   # plain FP64 2M workload
        return scenes.dam_break(5e-4, tank=(2.0, 1.2), column=(0.5, 1.0), dt=5e-5)
    if name == "dambreak_small":  # the reference's CPU-sized case
        return scenes.dam_break(0.01, tank=(1.0, 0.6), column=(0.25, 0.5), dt=1e-3)
    if name.startswith("dambreak_cols"):  # dambreak_cols<k>: k x 2k column, same tank
        k = int(name[len("dambreak_cols"):])
        return scenes.dam_break(0.5 / k, tank=(2.0, 1.2), column=(0.5, 1.0), dt=5e-5)
    raise SystemExit(f"unknown workload {name}")


def workload_config(name: str, prm: dict, nf: int, n: int) -> dict:
    """The `config` of both arms' JSON lines (the same workload, whatever
    runs it)."""
    return {"workload": f"{name}: 2-D dam break, {nf} fluid / {n} particles, dt {prm['dt']} s, "
                        f"l0 {prm['particle_distance']:.6g} m",
            "particles": n, "fluid_particles": nf,
            "cache": "inputs larger than L2: the state, neighbour lists and PPE matrix of one "
                     "step are GBs, re-sorted and re-assembled every step"}


# ---------------------------------------------------------------- clocks
class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region:
    the sampler is started (and its first sample awaited) before the region,
    the region's host wall-clock bounds are marked, and the summary keeps the
    samples whose timestamps fall inside them (the one nearest to the middle
    if the region is shorter than the sampling interval)."""

    Q = ("timestamp,index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.path = os.path.join(tempfile.gettempdir(), f"mps_clocks_{os.getpid()}.csv")
        self.window = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.Q}",
                 "--format=csv,noheader,nounits", "-lms", "20"],
                stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
            t_end = time.time() + 3.0
            while time.time() < t_end and os.path.getsize(self.path) == 0:
                time.sleep(0.01)
        except (FileNotFoundError, OSError):
            self.proc = None
        return self

    def mark(self, t0: float, t1: float):
        self.window = (t0, t1)

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        import datetime

        if not os.path.exists(self.path):
            return None
        rows = []
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            f = [x.strip() for x in line.split(",")]
            if len(f) < 10:
                continue
            try:
                ts = datetime.datetime.strptime(f[0], "%Y/%m/%d %H:%M:%S.%f").timestamp()
                rows.append((ts, float(f[2]), float(f[3]),
                             {nm for nm, v in zip(names, f[6:10]) if v.lower() == "active"}))
            except ValueError:
                continue
        if not rows:
            return None
        inside = rows
        if self.window:
            t0, t1 = self.window
            inside = [r for r in rows if t0 <= r[0] <= t1]
            if not inside:  # shorter than the interval: the sample nearest the middle
                mid = 0.5 * (t0 + t1)
                inside = [min(rows, key=lambda r: abs(r[0] - mid))]
        reasons = set().union(*(r[3] for r in inside))
        return {"sm_mhz": statistics.median(r[1] for r in inside), "sm_max_mhz": max(r[2] for r in inside),
                "reasons": sorted(reasons), "samples": len(inside),
                "window_s": round(self.window[1] - self.window[0], 4) if self.window else None}


# ---------------------------------------------------------------- roofline
def measured_peaks():
    p = os.path.join(REPO, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def traffic_per_row_iter(kernel: str):
    """DRAM bytes per (row x iteration) of the solver kernel from the committed
    ncu summary, if one exists (profiles/<kernel>_*.txt, line 'dram_bytes_per_row_iter: X')."""
    d = os.path.join(REPO, "profiles")
    if not os.path.isdir(d):
        return None
    for fn in sorted(os.listdir(d)):
        if fn.startswith(kernel) and fn.endswith(".txt"):
            for line in open(os.path.join(d, fn)):
                if line.startswith("dram_bytes_per_row_iter:"):
                    return float(line.split(":")[1])
    return None


# ---------------------------------------------------------------- CPU baseline
CPU_SAMPLE = "dambreak_cols200"  # 200 x 400 = 80,000 fluid particles, same tank and physics

# The CPU oracle on the benchmark's own scene (a child process, so that it
# runs on the host cores while the GPU legs run): `warmup` steps with the CG
# capped at CPU_WARMUP_CG iterations (they only bring the state to the
# physical time of the timed steps, as the GPU legs' warm-up steps do), then
# one full step as the reference runs it (CG to machine epsilon, solved
# twice, src/mps.cpp:452-460) and one step with one CG solve to the GPU
# solver's tolerance 1e-10.  Each full step of the 1M scene takes minutes
# (the reference's CG is serial), so one of each is the bounded sample.
CPU_WARMUP_CG = 50
_CPU_1M_CODE = """
import sys, time, json
sys.path.insert(0, %(repo)r); sys.path.insert(0, %(oracle)r)
import bench
from oracle import Oracle, build
build()
prm, pos, vel, t = bench.workload(%(wl)r)
nf = int((t == 0).sum())
o = Oracle(prm, pos, vel, t)
o.set_cg(max_iter=%(wcap)d, solves=1)
t0 = time.perf_counter()
for _ in range(%(warmup)d):
    o.step()
tw = time.perf_counter() - t0
out = {"wl": %(wl)r, "nf": nf, "n": int(len(t)), "warmup": %(warmup)d, "warmup_s": tw, "legs": []}
for tol, solves, name in %(legs)r:
    if tol is None:
        o.set_cg(solves=solves)
    else:
        o.set_cg(tol=tol, solves=solves)
    t0 = time.perf_counter()
    st = o.step()
    out["legs"].append({"name": name, "seconds": time.perf_counter() - t0,
                        "cg_iterations": int(st["cg_iterations"]), "cg_error": st["cg_error"],
                        "solves": solves})
    print(json.dumps(out), flush=True)
"""


def start_cpu_1m(warmup: int, legs, workload_name: str = "dambreak_1m", threads: int = 0):
    """Starts the CPU oracle on the full workload in a child process; returns
    (process, threads).  `legs`: list of (tol or None for eps, solves, name)."""
    cores = os.cpu_count() or 1
    threads = threads or max(1, cores - 2)  # leave the GPU legs' host thread and the sampler a core
    code = _CPU_1M_CODE % {"repo": REPO, "oracle": os.path.join(REPO, "oracle"), "wl": workload_name,
                           "wcap": CPU_WARMUP_CG, "warmup": warmup, "legs": list(legs)}
    env = dict(os.environ, OMP_NUM_THREADS=str(threads))
    proc = subprocess.Popen([sys.executable, "-c", code], stdout=subprocess.PIPE,
                            stderr=subprocess.PIPE, text=True, env=env)
    return proc, threads


def finish_cpu_1m(proc, threads: int, timeout: float = 3600) -> dict:
    out, err = proc.communicate(timeout=timeout)
    if proc.returncode != 0:
        raise RuntimeError(err[-2000:])
    d = json.loads(out.strip().splitlines()[-1])
    legs = {}
    for leg in d["legs"]:
        legs[leg["name"]] = {"value": d["nf"] / leg["seconds"], "unit": UNIT,
                             "seconds_per_step": leg["seconds"], "cg_iterations": leg["cg_iterations"],
                             "cg_solves": leg["solves"], "cg_relative_error": leg["cg_error"]}
    ref = d["legs"][0]
    return {"value": d["nf"] / ref["seconds"], "unit": UNIT, "cores": threads, "kind": "port",
            "sample": (f"{d['wl']} itself ({d['nf']} fluid / {d['n']} particles) on the CPU oracle: "
                       f"{d['warmup']} warm-up steps with the CG capped at {CPU_WARMUP_CG} iterations "
                       f"({d['warmup_s']:.1f} s, untimed), then one full step per leg: "
                       + "; ".join(f"{x['name']}: {x['seconds']:.1f} s, {x['cg_iterations']} CG iterations "
                                   f"x {x['solves']} solve(s)" for x in d["legs"])
                       + f"; {threads} OpenMP threads (the CG is serial, as the reference's)"),
            "legs": legs}


def cpu_sample(steps: int = 3, workload_name: str = CPU_SAMPLE) -> dict:
    """Times full oracle steps (all phases, CG to machine epsilon solved twice,
    as the reference) in a child process with OMP_NUM_THREADS = host cores."""
    cores = os.cpu_count() or 1
    code = (
        "import sys, time, json; sys.path.insert(0, %r); sys.path.insert(0, %r)\n"
        "import bench\nfrom oracle import Oracle, build\nbuild()\n"
        "prm, pos, vel, t = bench.workload(%r)\n"
        "o = Oracle(prm, pos, vel, t)\n"
        "nf = int((t == 0).sum()); times = []; its = []\n"
        "for s in range(%d):\n"
        "    t0 = time.perf_counter(); st = o.step(); times.append(time.perf_counter() - t0)"
        "; its.append(st['cg_iterations'])\n"
        "print(json.dumps({'nf': nf, 'times': times, 'its': its}))\n"
    ) % (REPO, os.path.join(REPO, "oracle"), workload_name, steps)
    env = dict(os.environ, OMP_NUM_THREADS=str(cores))
    out = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, env=env,
                         timeout=1800)
    if out.returncode != 0:
        raise RuntimeError(out.stderr[-2000:])
    d = json.loads(out.stdout.strip().splitlines()[-1])
    tot = sum(d["times"])
    return {"value": d["nf"] * len(d["times"]) / tot, "unit": UNIT, "cores": cores,
            "kind": "port",
            "sample": (f"{len(d['times'])} full steps of {workload_name} "
                       f"({d['nf']} fluid particles) on the CPU oracle, FP64 CG to machine "
                       f"epsilon solved twice per step as the reference (CG iterations "
                       f"{_its_summary(d['its'])}), {tot:.1f} s"
                       + ("; the 1M workload's CPU throughput would be lower since CG "
                          "iterations grow with resolution" if workload_name == CPU_SAMPLE else ""))}


def _its_summary(its):
    return str(its) if len(its) <= 5 else f"mean {np.mean(its):.1f}, max {max(its)}"



# ---------------------------------------------------------------- replicas
def max_over_ranks(seconds: float, dist, device=None) -> float:
    """The slowest rank's time (replicas: the job ends when the last one does)."""
    if dist is None:
        return seconds
    import torch

    if device is None:
        device = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([seconds], device=device, dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_throughput(fluid_particles: int, steps: int, seconds: float, world: int) -> float:
    """Whole-job particle-steps/s of `world` replicas that each advanced
    `fluid_particles` for `steps` steps, timed by the slowest rank."""
    return world * fluid_particles * steps / seconds


# ---------------------------------------------------------------- other workloads
def _event_timed(stream_ptr, fn):
    """Device seconds of fn() on the given stream (CUDA events, synchronised)."""
    import torch

    stream = torch.cuda.ExternalStream(stream_ptr)
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(stream)
    out = fn()
    e1.record(stream)
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / 1e3, out


def run_batched(steps: int, warmup: int) -> dict:
    """64 uneven scenes (seeded: 2k-60k fluid particles, aspect 0.5-2,
    l0 1e-3..5e-3 m, dam breaks and hydrostatic tanks) advanced together:
    one graph per step, one persistent launch for all 64 PPE solves."""
    from mps_gb300 import Batch, scenes

    sc = scenes.batch_scenes(seed=0)
    nf = sum(int((s[3] == 0).sum()) for s in sc)
    n = sum(len(s[3]) for s in sc)
    b = Batch(sc, tol=1e-8)
    b.step()  # autotuning step
    for _ in range(warmup):
        b.step()
    sec, (stats, _) = _event_timed(b.stream_ptr(), lambda: b.step(steps))
    info = b.launch_info()
    its = [s["cg_iterations"] for s in stats]
    out = {"workload": f"64 scenes (seed 0), {nf} fluid / {n} particles, mixed solver tol 1e-8",
           "value": nf * steps / sec, "unit": UNIT, "steps": steps,
           "ms_per_step": 1e3 * sec / steps,
           "launch": {k: info[k] for k in ("block", "alpha", "grid")},
           "autotune_ms": [round(x, 3) for x in info["tune_ms"]],
           "cg_iterations_min_max": [int(min(its)), int(max(its))],
           "max_rel_residual": float(max(s["cg_relative_residual"] for s in stats)),
           "cuda_graph_steps": steps if all(s["graph_replayed"] for s in stats) else 0}
    b.close()
    return out


def run_adjoint() -> dict:
    """Adjoint of a 200-step trajectory of the hydrostatic tank (0.4 x 0.4 m
    water, l0 2.5e-3 m: 25,600 fluid particles), FP64, checkpoints every 20
    steps; loss = mean-squared pressure at 16 wall taps over all steps + squared
    distance of the final fluid positions to a seeded target; checked against
    central finite differences (epsilon 1e-6) for gravity and one direction of
    the initial velocities.  dt = 0.1 s/m x l0 = 2.5e-4 s, the 1,250-particle
    case's dt / l0: at dt = 1e-3 s this resolution is unstable (the Courant
    number passes 6 within 10 steps), and so is any gradient of it."""
    from mps_gb300 import FP64, Engine, Trajectory, scenes

    l0, steps, every = 2.5e-3, 200, 20
    prm, pos, vel, t = scenes.hydrostatic(l0, size=(0.4, 0.4), dt=0.1 * l0)
    rng = np.random.default_rng(0)
    fl = t == scenes.FLUID
    vel[fl, :2] = rng.normal(0.0, 0.01, (fl.sum(), 2))
    target = pos[fl] + np.c_[rng.normal(0.0, 0.1 * l0, (fl.sum(), 2)), np.zeros(fl.sum())]
    taps = scenes.wall_taps(pos, t, l0, 16)
    eng = Engine(prm, pos, vel, t, precision=FP64)
    tr = Trajectory(eng, steps, every, taps)
    g = np.array(prm["gravity"], float)

    def loss(v0, gv):
        sp, pf, _ = tr.forward(v0, gv)
        return float(np.mean(sp ** 2) + np.sum((pf[fl] - target) ** 2)), sp, pf

    t0 = time.perf_counter()
    L, sp, pf = loss(vel, g)
    t_fwd = time.perf_counter() - t0
    d_pos = np.zeros_like(pf)
    d_pos[fl] = 2.0 * (pf[fl] - target)
    t0 = time.perf_counter()
    _, gv, gg = tr.backward(2.0 * sp / sp.size, d_pos, None)
    t_bwd = time.perf_counter() - t0
    eps = 1e-6
    gp, gm = g.copy(), g.copy()
    gp[1] += eps
    gm[1] -= eps
    fd_g = (loss(vel, gp)[0] - loss(vel, gm)[0]) / (2 * eps)
    u = np.zeros_like(vel)
    u[fl, :2] = rng.normal(size=(fl.sum(), 2))
    u /= np.linalg.norm(u)
    fd_v = (loss(vel + eps * u, g)[0] - loss(vel - eps * u, g)[0]) / (2 * eps)
    ad_v = float(np.sum(gv * u))
    tr.close()
    eng.close()
    return {"workload": f"hydrostatic tank 0.4 x 0.4 m, {int(fl.sum())} fluid / {len(t)} particles, "
                        f"dt {prm['dt']:.2e} s, {steps} steps, checkpoints every {every}, FP64",
            "forward_s": round(t_fwd, 3), "backward_s": round(t_bwd, 3), "loss": L,
            "dL_dgy": float(gg[1]), "fd_dL_dgy": fd_g,
            "rel_err_gravity": abs(gg[1] - fd_g) / max(abs(fd_g), 1e-300),
            "dL_dv0_dir": ad_v, "fd_dL_dv0_dir": fd_v,
            "rel_err_velocity_dir": abs(ad_v - fd_v) / max(abs(fd_v), 1e-300)}


def run_fp64_2m(steps: int) -> dict:
    """The plain FP64 step (the reference's Jacobi CG to machine epsilon) at
    2M fluid particles: dam break 0.5 x 1.0 m column, l0 5e-4 m, dt 5e-5 s."""
    from mps_gb300 import FP64, Engine

    prm, pos, vel, t = workload("dambreak_2m")
    nf = int((t == 0).sum())
    e = Engine(prm, pos, vel, t, precision=FP64)
    e.step()
    sec, stats = _event_timed(e.stream_ptr(), lambda: [e.step() for _ in range(steps)])
    out = {"workload": f"dambreak_2m: {nf} fluid / {len(t)} particles, FP64 solver", "steps": steps,
           "value": nf * steps / sec, "unit": UNIT, "ms_per_step": 1e3 * sec / steps,
           "cg_iterations_mean": float(np.mean([s["cg_iterations"] for s in stats])),
           "ms_solve_mean": float(np.mean([s["ms_solve"] for s in stats])),
           "solve_gbs": float(np.sum([s["solve_bytes"] for s in stats])
                              / (np.sum([s["ms_solve"] for s in stats]) / 1e3) / 1e9)}
    e.close()
    return out


def run_export(steps: int = 30, every: int = 10) -> dict:
    """The 1M step with the reference's export every `every` steps (CSV + VTU
    of every particle), three ways: no export; synchronous (the export step,
    then snapshot and write before the next step, as the reference does);
    asynchronous (snapshot, then the writer thread formats and writes while
    the next steps run).  Wall time on the stepping thread up to its last
    step; the wait for the last export's write after it is reported apart
    (no step is left to hide it behind)."""
    import shutil

    from mps_gb300 import MIXED, Engine

    prm, pos, vel, t = workload("dambreak_1m")
    nf = int((t == 0).sum())
    e = Engine(prm, pos, vel, t, precision=MIXED)
    for _ in range(2):
        e.step()
    shm = "/dev/shm" if os.path.isdir("/dev/shm") and os.access("/dev/shm", os.W_OK) else None
    d = tempfile.mkdtemp(dir=shm)
    try:
        def loop(mode):
            writer = None
            t0 = time.perf_counter()
            for s in range(steps):
                ex = mode != "none" and s % every == every - 1
                e.step(export=ex)
                if not ex:
                    continue
                csv, vtu = os.path.join(d, f"o{s}.csv"), os.path.join(d, f"o{s}.vtu")
                if writer is not None:
                    writer.join()
                e.export_begin()
                if mode == "sync":
                    e.export_write(csv, vtu, s * prm["dt"])
                else:
                    writer = threading.Thread(target=e.export_write, args=(csv, vtu, s * prm["dt"]))
                    writer.start()
            t1 = time.perf_counter()
            if writer is not None:
                writer.join()
            return t1 - t0, time.perf_counter() - t1

        (base, _), (sync, _), (asyn, tail) = loop("none"), loop("sync"), loop("async")
        t0 = time.perf_counter()
        e.export_begin()
        e.export_write(os.path.join(d, "w.csv"), os.path.join(d, "w.vtu"), 0.0)
        write_s = time.perf_counter() - t0
        size = os.path.getsize(os.path.join(d, "w.csv")) + os.path.getsize(os.path.join(d, "w.vtu"))
    finally:
        shutil.rmtree(d, ignore_errors=True)
    e.close()
    n_ex = steps // every
    return {"workload": f"dambreak_1m: {nf} fluid / {len(t)} particles, mixed solver, {steps} steps, "
                        f"export every {every} (CSV + VTU, {n_ex} exports)",
            "target": "tmpfs (/dev/shm)" if shm else "temporary directory",
            "ms_per_step": {"no_export": 1e3 * base / steps, "sync_export": 1e3 * sync / steps,
                            "async_export": 1e3 * asyn / steps},
            "export_cost_ms": {"sync": 1e3 * (sync - base) / n_ex, "async": 1e3 * (asyn - base) / n_ex},
            "last_write_wait_ms": 1e3 * tail,
            "one_export_write_ms": 1e3 * write_s, "bytes_per_export": int(size),
            "d2h_bytes_per_export": int(len(t) * 72)}


def run_accuracy_trajectory(prm, pos, vel, types, steps: int = 500, every: int = 50) -> dict:
    """The mixed step against the plain FP64 step over `steps` steps from the
    same initial state (config 2: "500 steps; report pressure and position
    error vs the FP64 run"): every `every` steps the pressure relative L2,
    the largest position and velocity differences and the count of surface
    flags that differ.  The mixed engine's device time over the whole window
    is reported too (its throughput over the configuration's 500 steps)."""
    import torch

    from mps_gb300 import FP64, MIXED, Engine

    nf = int((types == 0).sum())
    em = Engine(prm, pos, vel, types, precision=MIXED)
    ef = Engine(prm, pos, vel, types, precision=FP64)
    rows, sec_m, sec_f = [], 0.0, 0.0
    its_m, its_f = [], []
    first_flag_step = None  # the first step after which a surface flag differs
    bm, bf = np.zeros(len(types), np.int32), np.zeros(len(types), np.int32)
    for s0 in range(0, steps, every):
        dt_m = dt_f = 0.0
        for s in range(s0 + 1, s0 + every + 1):
            d, x = _event_timed(em.stream_ptr(), em.step)
            dt_m += d
            its_m.append(x["cg_iterations"])
            d, x = _event_timed(ef.stream_ptr(), ef.step)
            dt_f += d
            its_f.append(x["cg_iterations"])
            if first_flag_step is None:
                em.download_into(bc=bm)
                ef.download_into(bc=bf)
                if not np.array_equal(bm, bf):
                    first_flag_step = s
        sec_m += dt_m
        sec_f += dt_f
        a, b = em.state(), ef.state()
        pb = np.linalg.norm(b["pressure"]) or 1.0
        rows.append({"step": s0 + every,
                     "pressure_rel_l2": float(np.linalg.norm(a["pressure"] - b["pressure"]) / pb),
                     "position_max_abs_m": float(np.max(np.abs(a["pos"] - b["pos"]))),
                     "velocity_max_abs_mps": float(np.max(np.abs(a["vel"] - b["vel"]))),
                     "surface_flags_differing": int(np.sum(a["bc"] != b["bc"])),
                     "types_differing": int(np.sum(a["type"] != b["type"]))})
    em.close()
    ef.close()
    torch.cuda.synchronize()
    before = [r for r in rows if first_flag_step is None or r["step"] < first_flag_step]
    return {"steps": steps, "every": every, "rows": rows,
            "first_step_surface_flags_differ": first_flag_step,
            "before_that": {"max_pressure_rel_l2": max((r["pressure_rel_l2"] for r in before), default=None),
                            "max_position_abs_m": max((r["position_max_abs_m"] for r in before), default=None)},
            "note": ("surface detection is a threshold on the number density (src/mps.cpp:262-278): "
                     "once a particle within rounding of the threshold flips, the two trajectories "
                     "follow different PPE systems; the FP64 GPU step and the CPU oracle part the "
                     "same way (small_case.accuracy_vs_oracle)"),
            "max_pressure_rel_l2": max(r["pressure_rel_l2"] for r in rows),
            "max_position_abs_m": max(r["position_max_abs_m"] for r in rows),
            "mixed_value": nf * steps / sec_m, "fp64_value": nf * steps / sec_f, "unit": UNIT,
            "mixed_ms_per_step": 1e3 * sec_m / steps, "fp64_ms_per_step": 1e3 * sec_f / steps,
            "mixed_cg_iterations_mean": float(np.mean(its_m)),
            "fp64_cg_iterations_mean": float(np.mean(its_f))}


def run_precision_split(prm, state, steps: int = 4) -> dict:
    """How much of the mixed/FP64 ratio is precision, how much the
    preconditioner and how much the initial guess: from one developed state,
    `steps` steps each of the FP64 solver (the reference's Jacobi CG from
    zero), the mixed solver with the same Jacobi preconditioner from zero
    (multigrid mode 0), the mixed solver with its default multigrid from zero,
    and the same from the previous step's solution (the default); ms per
    solve and iterations of each."""
    from mps_gb300 import FP64, MIXED, Engine

    out = {}
    for name, prec, mode, warm in (("fp64_jacobi", FP64, None, False), ("mixed_jacobi", MIXED, 0, False),
                                   ("mixed_multigrid", MIXED, 1, False),
                                   ("mixed_multigrid_previous_guess", MIXED, 1, True)):
        e = Engine(prm, state["pos"], state["vel"], state["type"], precision=prec)
        if mode is not None:
            e.set_multigrid(mode)
        if prec == MIXED:
            e.set_initial_guess(warm)
        e.step()
        st = [e.step() for _ in range(steps)]
        out[name] = {"ms_solve_mean": float(np.mean([x["ms_solve"] for x in st])),
                     "cg_iterations_mean": float(np.mean([x["cg_iterations"] for x in st])),
                     "refinements_mean": float(np.mean([x["refinements"] for x in st]))}
        e.close()
    f, j, g = out["fp64_jacobi"], out["mixed_jacobi"], out["mixed_multigrid"]
    gw = out["mixed_multigrid_previous_guess"]
    out["solve_speedup_precision_only"] = f["ms_solve_mean"] / j["ms_solve_mean"]
    out["solve_speedup_preconditioner_on_top"] = j["ms_solve_mean"] / g["ms_solve_mean"]
    out["solve_speedup_initial_guess_on_top"] = g["ms_solve_mean"] / gw["ms_solve_mean"]
    out["solve_speedup_total"] = f["ms_solve_mean"] / gw["ms_solve_mean"]
    out["steps"] = steps
    return out


def run_collisions(steps: int = 3) -> dict:
    """The collision pass with ~10^5 candidate pairs per step: the 1M dam
    break shaken (fluid positions +-0.4 l0, velocities N(0, 0.1) m/s), the
    same steps with the pairs applied in parallel (default) and by one thread
    in the reference's order; the states agree bit for bit
    (tests/test_gpu_collisions.py checks the same on smaller scenes)."""
    from mps_gb300 import MIXED, Engine, scenes

    prm, pos, vel, t = scenes.shaken(workload("dambreak_1m"))
    out = {}
    for name, serial in (("parallel", False), ("serial", True)):
        e = Engine(prm, pos, vel, t, precision=MIXED)
        e.set_collisions(serial)
        st = [e.step() for _ in range(steps)]
        out[name] = {"ms_step": [round(x["ms_step"], 3) for x in st],
                     "candidates": [int(x["n_collision_candidates"]) for x in st]}
        out[name + "_state"] = e.state()
        e.close()
    same = all(np.array_equal(out["parallel_state"][k], out["serial_state"][k]) for k in out["serial_state"])
    del out["parallel_state"], out["serial_state"]
    out.update({"workload": f"dambreak_1m shaken: {int((t == 0).sum())} fluid particles, positions +-0.4 l0, "
                            f"velocities N(0, 0.1) m/s, {steps} steps, mixed solver",
                "states_bit_identical": bool(same),
                "ms_step_saved_by_parallel_pass": [round(a - b, 3) for a, b in
                                                   zip(out["serial"]["ms_step"], out["parallel"]["ms_step"])]})
    return out


def run_small_case() -> dict:
    """The reference's own CPU-sized case (1,250 fluid particles, dt 1e-3 s,
    1,000 steps), FP64 on the GPU (graph replays) and on the CPU oracle."""
    from mps_gb300 import FP64, Engine

    prm, pos, vel, t = workload("dambreak_small")
    nf = int((t == 0).sum())
    e = Engine(prm, pos, vel, t, precision=FP64)
    t0 = time.perf_counter()
    st = e.run(1000)
    gpu_s = time.perf_counter() - t0
    e.close()
    cpu = cpu_sample(steps=1000, workload_name="dambreak_small")
    return {"workload": f"dambreak_small: {nf} fluid / {len(t)} particles, 1000 steps, FP64",
            "gpu_wall_s": round(gpu_s, 3), "gpu_value": nf * 1000 / gpu_s,
            "courant_final": st["courant"], "unit": UNIT,
            "cpu_oracle": {k: cpu[k] for k in ("value", "cores", "kind", "sample")},
            "accuracy_vs_oracle": small_case_accuracy(prm, pos, vel, t)}


def small_case_accuracy(prm, pos, vel, t, steps: int = 1000, report=(100, 500, 1000)) -> dict:
    """The FP64 GPU step against the CPU oracle over the 1,000 steps: the
    first step (if any) at which types, surface or Dirichlet flags, or the
    collision candidate pairs differ, and the pressure / position /
    velocity differences at the reported steps."""
    sys.path.insert(0, os.path.join(REPO, "oracle"))
    from oracle import Oracle

    from mps_gb300 import FP64, Engine

    e = Engine(prm, pos, vel, t, precision=FP64)
    o = Oracle(prm, pos, vel, t)
    o.set_cg(solves=1)  # the second solve repeats the first exactly
    first_diff = {"flags": None, "collisions": None}
    at = {}
    n_coll = 0
    for s in range(1, steps + 1):
        e.step()
        o.step()
        ci, cj, _ = e.collisions()
        oi, oj, _ = o.collisions()
        n_coll += len(oi)
        if first_diff["collisions"] is None and not (np.array_equal(ci, oi) and np.array_equal(cj, oj)):
            first_diff["collisions"] = s
        a, b = e.state(), o.state()
        if first_diff["flags"] is None and not all(np.array_equal(a[k], b[k]) for k in ("type", "bc", "dirichlet")):
            first_diff["flags"] = s
        if s in report:
            pb = np.linalg.norm(b["pressure"]) or 1.0
            at[str(s)] = {"pressure_rel_l2": float(np.linalg.norm(a["pressure"] - b["pressure"]) / pb),
                          "position_max_abs_m": float(np.max(np.abs(a["pos"] - b["pos"]))),
                          "velocity_max_abs_mps": float(np.max(np.abs(a["vel"] - b["vel"]))),
                          "ghosts": int(np.sum(a["type"] == -1))}
    e.close()
    o.close()
    return {"steps": steps, "first_step_flags_differ": first_diff["flags"],
            "first_step_collisions_differ": first_diff["collisions"],
            "collision_candidates_total": n_coll, "at_step": at}

# ---------------------------------------------------------------- GPU arm
def run_ours(args, rank: int, world: int, dist):
    import torch

    from mps_gb300 import FP64, MIXED, Engine

    dev = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(dev)
    t_gen = time.perf_counter()
    prm, pos, vel, types = workload(args.workload)
    t_gen = time.perf_counter() - t_gen  # the scene on the host (numpy lattice, the reference's layout)
    n = len(types)
    nf = int((types == 0).sum())
    prec = MIXED if args.precision == "mixed" else FP64
    # the CPU baseline on this workload runs on the host cores meanwhile
    cpu_job = None
    if rank == 0 and not args.no_cpu:
        cpu_job = start_cpu_1m(args.warmup, [(None, 2, "reference_eps_two_solves"),
                                             (1e-10, 1, "gpu_tolerance_1e-10_one_solve")],
                               args.workload)

    def timed(eng, k):
        stream = torch.cuda.ExternalStream(eng.stream_ptr())
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        stats = []
        if dist:
            dist.barrier()
        torch.cuda.synchronize()
        e0.record(stream)
        for _ in range(k):
            stats.append(eng.step())
        e1.record(stream)
        torch.cuda.synchronize()
        if dist:
            dist.barrier()
        return e0.elapsed_time(e1) / 1e3, stats

    # main: mixed precision, state resident in HBM
    eng = Engine(prm, pos, vel, types, precision=prec)
    if prec == MIXED:
        eng.set_initial_guess(args.initial_guess == "previous")
    for _ in range(args.warmup):
        eng.step()
    with ClockSampler(dev) as clk:
        t_w0 = time.time()
        sec, stats = timed(eng, args.steps)
        clk.mark(t_w0, time.time())
    clocks = clk.summary()
    sec = max_over_ranks(sec, dist)
    value = replica_throughput(nf, args.steps, sec, world)
    warm_state = eng.state()

    # roofline of the dominant kernel (the pressure solve)
    hbm_peak, peak_kind = measured_peaks()
    solve_ms = [s["ms_solve"] for s in stats]
    sb = [s["solve_bytes"] for s in stats]  # the engine's algorithmic-bytes model
    achieved = sum(sb) / (sum(solve_ms) / 1e3) / 1e9
    row_iters = sum(s["cg_iterations"] for s in stats) * n / len(stats)
    solver_kernel = "k_cg_mixed_ov" if prec == MIXED else "k_cg64"  # mode 1: the overlapped kernel
    tpr = traffic_per_row_iter(solver_kernel)
    roofline = {"bound": "hbm", "achieved": round(achieved, 1), "peak": hbm_peak, "unit": "GB/s",
                "frac": round(achieved / hbm_peak, 4),
                "traffic": (tpr * row_iters) if tpr else None,
                "kernel": solver_kernel,
                "peak_source": peak_kind,
                "algorithmic_bytes_per_launch": sum(sb) / len(sb)}

    # plain FP64 on the same steps (skipped with --no-fp64)
    fp64 = None
    if not args.no_fp64 and prec == MIXED:
        e64 = Engine(prm, pos, vel, types, precision=FP64)
        for _ in range(args.warmup):
            e64.step()
        sec64, st64 = timed(e64, args.steps)
        sec64 = max_over_ranks(sec64, dist)
        fp64 = {"value": replica_throughput(nf, args.steps, sec64, world), "ms_per_step": 1e3 * sec64 / args.steps,
                "cg_iterations_mean": float(np.mean([s["cg_iterations"] for s in st64])),
                "ms_solve_mean": float(np.mean([s["ms_solve"] for s in st64]))}
        e64.close()

    # accuracy of the mixed step against FP64 from the same state
    acc = None
    if prec == MIXED and not args.no_fp64:
        ws = warm_state
        ea = Engine(prm, ws["pos"], ws["vel"], ws["type"], precision=FP64)
        eb = Engine(prm, ws["pos"], ws["vel"], ws["type"], precision=MIXED)
        ea.step()
        eb.step()
        ra, rb = ea.state(), eb.state()
        pa = np.linalg.norm(ra["pressure"]) or 1.0
        acc = {"pressure_rel_l2_vs_fp64": float(np.linalg.norm(rb["pressure"] - ra["pressure"]) / pa),
               "position_max_abs_diff_m": float(np.max(np.abs(rb["pos"] - ra["pos"]))),
               "surface_flags_equal": bool(np.array_equal(ra["bc"], rb["bc"]))}
        ea.close()
        eb.close()

    # config 2's own window: mixed against FP64 over 500 steps from rest
    traj = None
    if prec == MIXED and not args.no_fp64 and args.trajectory_steps > 0:
        traj = run_accuracy_trajectory(prm, pos, vel, types, steps=args.trajectory_steps)
    split = None
    if prec == MIXED and not args.no_fp64:
        split = run_precision_split(prm, warm_state)

    # end to end through the C ABI with host buffers, every step, over the
    # same physical steps as the device-resident window: a fresh engine from
    # the initial state, the same warm-up, then each step uploads its state
    # from pinned host memory and downloads the result
    e2e = None
    if not args.no_e2e:
        pin = lambda a: torch.from_numpy(np.ascontiguousarray(a)).pin_memory().numpy()  # noqa
        ee = Engine(prm, pos, vel, types, precision=prec)
        if prec == MIXED:
            ee.set_initial_guess(args.initial_guess == "previous")
        for _ in range(args.warmup):
            ee.step()
        st0 = ee.state()
        hpos, hvel, htype = pin(st0["pos"]), pin(st0["vel"]), pin(st0["type"])
        hp, hndr, hbc = pin(np.zeros(n)), pin(np.zeros(n)), pin(np.zeros(n, np.int32))
        k_e2e = args.e2e_steps if args.e2e_steps > 0 else args.steps
        if dist:
            dist.barrier()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(k_e2e):
            ee.upload(hpos, hvel, htype)
            ee.step()
            ee.download_into(pos=hpos, vel=hvel, pressure=hp, ndr=hndr, types=htype, bc=hbc)
        torch.cuda.synchronize()
        te = time.perf_counter() - t0
        te = max_over_ranks(te, dist)
        ee.close()
        e2e = {"value": replica_throughput(nf, k_e2e, te, world), "unit": UNIT,
               "h2d_bytes_per_step": int(hpos.nbytes + hvel.nbytes + htype.nbytes),
               "d2h_bytes_per_step": int(hpos.nbytes + hvel.nbytes + hp.nbytes + hndr.nbytes
                                         + htype.nbytes + hbc.nbytes),
               "steps": k_e2e,
               "window": "the same steps as the device-resident timing (same initial state and warm-up)",
               "initial_guess": "the previous step's solution (kept across mps_upload)"}
    eng.close()

    others = {}
    if not args.no_others and world == 1:  # single-GPU runs only: keeps scaling runs short
        others["batched"] = run_batched(steps=300, warmup=3)
        others["adjoint"] = run_adjoint()
        others["fp64_2m"] = run_fp64_2m(steps=3)
        others["small_case"] = run_small_case()
        others["export"] = run_export()
        others["collisions"] = run_collisions()

    if rank != 0:
        return None
    cpu = None
    if cpu_job is not None:
        try:
            cpu = finish_cpu_1m(*cpu_job)
        except Exception as ex:  # reported, not hidden
            cpu = {"value": None, "error": str(ex)[-300:]}
    mean = lambda k: float(np.mean([s[k] for s in stats]))  # noqa
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * sec / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "fp32-krylov/fp64" if prec == MIXED else "f64",
        "data": "synthetic (seeded lattice dam break, the reference generator's layout)",
        "config": workload_config(args.workload, prm, nf, n),
        "solver": f"{args.precision} PPE solver", "parallelism": f"replicas x{world}",
        "initial_guess": ("the previous step's solution" if args.initial_guess == "previous" else "zero")
        if prec == MIXED else "zero",
        "gpu_launches": int(sum(s["kernel_launches"] for s in stats)),
        "cuda_graph_steps": int(sum(s["graph_replayed"] for s in stats)),
        "cg_iterations_mean": mean("cg_iterations"), "refinements_mean": mean("refinements"),
        "ms_solve_mean": mean("ms_solve"),
        "roofline": roofline, "fp64": fp64,
        "mixed_over_fp64": (value / fp64["value"]) if fp64 else None,
        "accuracy": acc, "accuracy_trajectory": traj, "precision_split": split,
        "scene_generation_s": round(t_gen, 3),
        "e2e": e2e, "cpu_baseline": cpu, "clocks": clocks,
        "other_workloads": others or None,
    }
    return line


def run_reference(args, rank: int):
    """The reference's algorithm on the host cores (the CPU oracle: the
    reference's own sources need Eigen, absent here), on this arm's workload:
    W warm-up steps with the CG capped, then one full step as the reference
    runs it (CG to machine epsilon, solved twice).  One step of the 1M scene
    takes minutes, so one step is the timed sample whatever --steps says."""
    if rank != 0:
        return None
    prm, pos, vel, types = workload(args.workload)
    nf, n = int((types == 0).sum()), len(types)
    proc, threads = start_cpu_1m(args.warmup, [(None, 2, "reference_eps_two_solves")], args.workload,
                                 threads=os.cpu_count() or 1)
    cpu = finish_cpu_1m(proc, threads)
    cfg = workload_config(args.workload, prm, nf, n)
    leg = cpu["legs"]["reference_eps_two_solves"]
    return {"metric": METRIC, "value": cpu["value"], "unit": UNIT, "n_gpus": args.gpus,
            "steps": 1, "steps_requested": args.steps, "warmup": args.warmup,
            "ms_per_step": 1e3 * leg["seconds_per_step"], "higher_is_better": True, "impl": "reference",
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic", "config": cfg,
            "solver": "FP64 Jacobi CG to machine epsilon, solved twice (the reference's), on the CPU",
            "parallelism": f"{threads} host threads (OpenMP where the reference has it)",
            "cpu_baseline": {k: cpu[k] for k in ("value", "unit", "cores", "kind", "sample")},
            "e2e": {"value": cpu["value"], "unit": UNIT, "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="dambreak_1m")
    ap.add_argument("--precision", default="mixed", choices=["mixed", "fp64"])
    ap.add_argument("--initial-guess", default="previous", choices=["previous", "zero"],
                    help="the mixed solver's start: the previous step's solution, or zero as the reference's CG")
    ap.add_argument("--e2e-steps", type=int, default=0, help="0: the same K as the timed steps")
    ap.add_argument("--no-fp64", action="store_true")
    ap.add_argument("--trajectory-steps", type=int, default=500,
                    help="mixed vs FP64 accuracy window (0: skip)")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-others", action="store_true",
                    help="skip the batched, adjoint, 2M FP64 and small-case workloads")
    args = ap.parse_args()
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    dist = None
    if args.impl == "reference":
        line = run_reference(args, rank)
    else:
        if world > 1:
            import torch.distributed as dist_mod

            dist_mod.init_process_group("nccl")
            dist = dist_mod
        line = run_ours(args, rank, world, dist)
        if dist:
            dist.destroy_process_group()
    if line is not None:
        print(json.dumps(line), flush=True)


if __name__ == "__main__":
    main()
