#!/usr/bin/env python
"""Benchmark of the GB300 PM force chain: particle-steps/s at 100M particles, 256^3.

One *step* is one KDK step of the fused engine on the resident state: int64
fixed-point CIC deposit, multigrid to a 1e-6 relative residual (FP64-class
double-float finest level, FP64 faces and coarsest solve) started from the
linear extrapolation of the previous potentials (``--warmstart``), and the
fused gather(-grad phi) + kick + drift particle pass. A Poisson comparison
reports V-cycles and solve time from the plain, extrapolated and learned
initial guesses. Workload (default): the
two-disk collision with 40M + 60M particles on a 256^3 grid over [-32, 32]^3,
dt = 0.005, seed 2, mass quantum 2^-40 of the total.

Printed: one JSON line (rank 0) with the value, per-step time, the roofline of
the dominant kernel (CUDA-event time of its launches inside this run), the
CPU baseline (the reference algorithm restated in C, on this host's cores),
the end-to-end rate through the public API with host buffers, the SM clocks
sampled during the timed region and the number of kernel launches.

``--impl reference`` times the reference's algorithm instead: the C
restatement of its Taichi kernels (the Taichi package itself cannot be
installed here) with the reference's solver schedule, on all host threads.
Multi-GPU: one process per GPU (torchrun); the simulation does not shard, so
the ranks run independent replicas (weak scaling, no collective in the step).
"""

from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
for _p in (str(ROOT), str(ROOT / "galaxy-collision-with-cuda-fft_gb300")):
    if _p not in sys.path:
        sys.path.insert(0, _p)

import numpy as np  # noqa: E402

METRIC = "particle-steps/s at 100M, 256^3"
UNIT = "particle-steps/s"
REFERENCE_PUBLISHED = 6.95e8  # reference, RTX 3070, 100M at 256^3 (its tol 1e-3): 6.95 steps/s x 1e8
L2_BYTES = 126 * 1024**2

# Algorithmic bytes per unit (per particle, or per finest cell) for each kernel.
ALGO_BYTES = {
    "gather_kick_drift": ("particle", 48.0),  # read x,y,z,vx,vy,vz; write them back
    "grad": ("cell", 20.0),                   # read phi, write the float4 node field
    "deposit_runs": ("particle", 16.0),       # read x,y,z,m
    "deposit": ("particle", 16.0),
    "smooth0": ("cell", 6.0),                 # colour-split half-sweep: other colour's e, own r, own e (2 B each)
    "update0": ("cell", 20.0),                # last half-sweep + phi += e: red e, black r, read/write hi,lo
    "resid0": ("cell", 18.0),                 # read hi,lo,b0; write r and the first red half-sweep
    "resid0e": ("cell", 12.0),                # read e, r; write the correction residual
    "convert_q": ("cell", 20.0),              # read q, clear q, write b
    "prolong0": ("cell", 4.0),                # read/write the black correction
}
# Kernels of the Poisson solve (the multigrid, its faces and norms, and the b0 conversion).
MG_KERNELS = ("smooth0", "update0", "resid0", "resid0e", "restrict", "smooth", "resid", "prolong", "prolong0",
              "coarse", "tail", "faces", "moments", "rhs", "reduce", "convert_q")


def _parse(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=100,
                    help="timed steps (default: five cell-sort periods, so the sorts are inside the timed region)")
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=("ours", "reference"), default="ours")
    ap.add_argument("--config", default="two_disk_100M")
    ap.add_argument("--scale", type=float, default=1.0, help="particle-count scale of the configuration")
    ap.add_argument("--tol", type=float, default=1e-6)
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--cpu-budget-s", type=float, default=25.0)
    ap.add_argument("--profile-steps", type=int, default=3)
    ap.add_argument("--grad-grid", type=int, default=1,
                    help="1: gather from a float4 -grad(phi) grid; 0: form the gradient at the corners on the fly")
    ap.add_argument("--warmstart", choices=("plain", "extrapolate", "learned"), default="extrapolate",
                    help="initial guess of each solve: previous potential (the reference's), its linear "
                         "extrapolation, or the extrapolation + the trained network's correction")
    ap.add_argument("--pre-sweeps", type=int, default=2, help="red-black sweeps before restriction (reference: 2)")
    ap.add_argument("--post-sweeps", type=int, default=2, help="red-black sweeps after prolongation (reference: 2)")
    ap.add_argument("--coarse-level-sweeps", type=int, default=None,
                    help="sweeps each way below the finest level: 1, or (default) the same as --pre/--post-sweeps "
                         "as the reference")
    ap.add_argument("--sort-every", type=int, default=20, help="steps between cell sorts of the particles")
    ap.add_argument("--deposit-next", action="store_true",
                    help="the particle pass also deposits the drifted positions for the next step")
    ap.add_argument("--sort-ahead", type=float, default=None,
                    help="sort by the cells predicted this many steps ahead (x + v * steps * dt); "
                         "default half the sort period")
    ap.add_argument("--compare-steps", type=int, default=6,
                    help="steps per initial guess in the Poisson comparison (0 skips it)")
    ap.add_argument("--plain-steps", type=int, default=5,
                    help="steps of the stepwise (unfused) chain timed for comparison; 0 skips it")
    ap.add_argument("--no-accuracy", action="store_true",
                    help="skip the potential/force error against the FP64 FFT and the converged multigrid")
    ap.add_argument("--accuracy-steps", type=int, default=200,
                    help="length of the accuracy run (the precision configuration: 200 steps)")
    ap.add_argument("--accuracy-every", type=int, default=50,
                    help="steps between its FP64 checks (the precision configuration: every 50th step)")
    ap.add_argument("--precision", choices=("mixed", "plain_f32"), default="mixed",
                    help="mixed: double-float finest level (reaches --tol); plain_f32: the all-FP32 multigrid of "
                         "the plain method, capped at the reference's 20 V-cycles (it stalls near 5e-5)")
    ap.add_argument("--graph", type=int, default=1,
                    help="1: time whole-step CUDA graph replays (stopping rule decided on the device); "
                         "0: eager steps that read the residual on the host after every V-cycle")
    ap.add_argument("--verbose", action="store_true")
    return ap.parse_args(argv)


def _dist():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def _log(args, *msg):
    if args.verbose:
        print("[bench]", *msg, file=sys.stderr, flush=True)


# ---------------------------------------------------------------------------- clocks
class ClockSampler:
    """nvidia-smi samples (50 ms) of SM clock and throttle reasons during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.idx = gpu_index
        self.proc = None
        self.path = None

    def start(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.idx}", f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "50"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons, power = [], [], set(), []
        names = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")
        for line in Path(self.path).read_text().splitlines():
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
                power.append(float(f[3]))
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        os.unlink(self.path)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm),
                "power_w_max": max(power) if power else None}


# ---------------------------------------------------------------------------- CPU arm
def _reference_chain(pos_grid, vel, mass, G, dx, dt, steps, budget_s, threads=None, fp64_tol=None):
    """The reference's KDK step (bench.py:145-152 / sim.py:320-327) on the C restatement
    of its kernels: kick, drift, deposit (parallel f32 atomics), multigrid with its
    schedule (tol 1e-3, 20 cycles, warm start), grad, gather, kick. With
    ``fp64_tol`` the multigrid is the same algorithm in FP64 iterated (warm
    started, at most 100 cycles) to that relative residual instead.
    Returns (seconds per step list, last solver cycles, residual ratio reached)."""
    from oracle import pm

    if threads:
        pm.set_threads(threads)
    x = [np.ascontiguousarray(pos_grid[:, i], dtype=np.float32) for i in range(3)]
    v = [np.ascontiguousarray(vel[:, i], dtype=np.float32) for i in range(3)]
    m = np.ascontiguousarray(mass, dtype=np.float32)
    if fp64_tol is None:
        phi = np.zeros((G, G, G), np.float32)
        mg = pm.ReferenceMultigrid(G, dx=dx, grav_constant=1.0)
    else:
        phi = np.zeros((G, G, G), np.float64)
        mg = pm.ReferenceMultigrid64(G, dx=dx, grav_constant=1.0, tol=fp64_tol, n_cycles=100)
    warm = {"on": False}
    acc = [None]

    def accel():
        rho = np.zeros((G, G, G), np.float32)
        pm.lib().or_deposit_f32(x[0], x[1], x[2], m, m.shape[0], float(dx), int(G), rho, 1)
        mg.solve(rho, phi, warm_start=warm["on"])
        warm["on"] = True
        acc[0] = pm.gather(np.stack(x, 1), *pm.grad(phi.astype(np.float32), dx), dx)

    accel()
    times = []
    for _ in range(steps):
        t0 = time.perf_counter()
        pm.axpy3(*v, *acc[0], np.float32(0.5 * dt))
        pm.axpy3(*x, *v, np.float32(dt))
        accel()
        pm.axpy3(*v, *acc[0], np.float32(0.5 * dt))
        times.append(time.perf_counter() - t0)
        if sum(times) > budget_s:
            break
    ratio = mg.norms[1] / mg.norms[0] if mg.norms[0] > 0 else 0.0
    return times, mg.last_cycles, float(ratio)


def _cpu_baseline(args, icr, cfg, n, G, dx, dt):
    """The reference chain restated in C on this host's cores: the reference's
    schedule on the full workload (the headline CPU number), the same chain with
    the FP64 multigrid driven to the GPU's tolerance, and the Plummer
    configuration's full 200-step run."""
    from galaxy_collision_gb300 import ic

    pos_grid = (icr.pos.astype(np.float64) - np.asarray(cfg["origin"])).astype(np.float32)
    times, cyc, ratio = _reference_chain(pos_grid, icr.vel, icr.mass, G, dx, dt, 3, args.cpu_budget_s)
    out = {
        "value": n * len(times) / sum(times), "unit": UNIT, "cores": _cpu_cores(), "kind": "port",
        "sample": f"{len(times)} KDK step(s) of the full workload ({n:,} particles, {G}^3) after one priming "
                  f"force evaluation; reference schedule tol=1e-3, n_cycles=20, warm start (last solve "
                  f"{cyc} cycles, residual ratio {ratio:.2e})",
    }
    t64, c64, r64 = _reference_chain(pos_grid, icr.vel, icr.mass, G, dx, dt, 2, args.cpu_budget_s,
                                     fp64_tol=args.tol)
    out["fp64_to_tol"] = {
        "value": n * len(t64) / sum(t64), "unit": UNIT,
        "sample": f"{len(t64)} KDK step(s) of the full workload, the same chain with the reference multigrid in "
                  f"FP64 iterated to {args.tol:g} (last solve {c64} cycles, residual ratio {r64:.2e})"}
    p_icr, p_cfg = ic.build("plummer_131k")
    p_pos = (p_icr.pos.astype(np.float64) - np.asarray(p_cfg["origin"])).astype(np.float32)
    tp, cp, rp = _reference_chain(p_pos, p_icr.vel, p_icr.mass, p_cfg["grid"], p_cfg["dx"], p_cfg["dt"],
                                  p_cfg["steps"], 10.0 * args.cpu_budget_s)
    out["plummer_131k_full_run"] = {
        "value": p_icr.n * len(tp) / sum(tp), "unit": UNIT, "steps": len(tp),
        "sample": f"the Plummer configuration ({p_icr.n:,} particles, {p_cfg['grid']}^3, dt {p_cfg['dt']}): "
                  f"{len(tp)} of {p_cfg['steps']} steps, reference schedule (last solve {cp} cycles, residual "
                  f"ratio {rp:.2e})"}
    return out


def _cpu_cores():
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:  # pragma: no cover
        return os.cpu_count() or 1


# ---------------------------------------------------------------------------- GPU arm
def aggregate(ms_local: float, n_local: int, steps: int, world: int, device="cpu"):
    """Whole-job rate of `world` independent replicas: the slowest rank's time
    (MAX over ranks) and the particles of all ranks. Returns (ms_max, value)."""
    ms_max = float(ms_local)
    total_n = int(n_local) * world
    if world > 1:
        import torch
        import torch.distributed as dist

        t = torch.tensor([ms_local, float(n_local)], dtype=torch.float64, device=device)
        tmax = t.clone()
        dist.all_reduce(tmax, op=dist.ReduceOp.MAX)
        tsum = t.clone()
        dist.all_reduce(tsum, op=dist.ReduceOp.SUM)
        ms_max = float(tmax[0].item())
        total_n = int(round(float(tsum[1].item())))
    return ms_max, total_n * steps / (ms_max / 1e3)


def _roofline(stats: dict, n: int, G: int, hbm_gbs: float, traffic: dict):
    best = None
    for name, (launches, timed, ms) in stats.items():
        if timed == 0 or ms <= 0:
            continue
        if best is None or ms > best[3]:
            best = (name, launches, timed, ms)
    if best is None:
        return None
    name, _, timed, ms = best
    kind, b = ALGO_BYTES.get(name, (None, None))
    if kind is None:
        return {"kernel": name, "bound": "hbm", "achieved": None, "peak": hbm_gbs, "unit": "GB/s", "frac": None,
                "traffic": None}
    units = n if kind == "particle" else G**3
    per_launch_bytes = b * units
    avg_s = ms / timed / 1e3
    achieved = per_launch_bytes / avg_s / 1e9
    tr = traffic.get(name)
    return {"kernel": name, "bound": "hbm", "achieved": round(achieved, 1), "peak": hbm_gbs, "unit": "GB/s",
            "frac": round(achieved / hbm_gbs, 4), "traffic": (tr * units if tr is not None else None),
            "algorithmic_bytes_per_launch": per_launch_bytes, "avg_launch_ms": round(avg_s * 1e3, 4),
            "launches_timed": timed, "peak_source": "measured (MEASURED_PEAKS.json hbm_gbs)"}


def _load_traffic() -> dict:
    """Per-unit DRAM bytes of each kernel from the committed ncu summary (or {})."""
    p = ROOT / "profiles" / "dram_traffic_per_unit.txt"
    out = {}
    if p.exists():
        for line in p.read_text().splitlines():
            if line.startswith("#") or ":" not in line:
                continue
            k, v = line.split(":", 1)
            try:
                out[k.strip()] = float(v.split()[0])
            except (ValueError, IndexError):
                pass
    return out


def run_ours(args):
    import torch

    rank, world, local = _dist()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group(backend="nccl", device_id=torch.device("cuda", local))
    from galaxy_collision_gb300 import _build, ic
    from galaxy_collision_gb300.accuracy import force_chain_errors
    from galaxy_collision_gb300.engine import PMEngine

    _build.build()
    peaks = json.loads((ROOT / "MEASURED_PEAKS.json").read_text()) if (ROOT / "MEASURED_PEAKS.json").exists() else {}
    hbm = float(peaks.get("hbm_gbs", 6800.0))
    t0 = time.time()
    icr, cfg = ic.build(args.config, scale=args.scale)
    _log(args, f"IC {icr.n} particles in {time.time() - t0:.1f}s")
    G, dx, dt = cfg["grid"], cfg["dx"], cfg["dt"]
    bits = cfg.get("fixed_point_bits", 52)
    n = icr.n

    net = _load_net() if args.warmstart == "learned" else None

    def make_engine(mode=None, plain_f32=False):
        e = PMEngine(G, dx, grav=1.0, origin=cfg["origin"], tol=args.tol, max_cycles=20 if plain_f32 else 60,
                     fixed_point_bits=bits, sort_every=args.sort_every, sort_ahead=args.sort_ahead,
                     grad_grid=bool(args.grad_grid), deposit_next=args.deposit_next,
                     pre_sweeps=args.pre_sweeps, post_sweeps=args.post_sweeps, plain_f32=plain_f32,
                     # the plain FP32 chain is the reference's method: the same sweeps on every level
                     coarse_level_sweeps=None if plain_f32 else args.coarse_level_sweeps)
        m = mode or args.warmstart
        e.set_warmstart(m, net=(net if net is not None else _load_net()) if m == "learned" else None)
        return e

    eng = make_engine(plain_f32=args.precision == "plain_f32")
    eng.load(icr.pos, icr.vel, icr.mass, icr.gid, sort=True)
    eng.prime(dt)
    # the sampler starts before the warm-up steps so that it samples the loaded GPU
    # from the first timed step on
    sampler = ClockSampler(local)
    sampler.start()
    # eager warm-up steps fill the warm-start history; with --graph the step
    # graphs of both particle-buffer sets are captured here, outside the timing
    for _ in range(max(args.warmup, 3 if args.graph else 0)):
        eng.advance(dt)
    if args.graph:
        eng.prepare_graphs(dt)
        eng.advance_graph(dt)
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()

    counts0 = {k: v[0] for k, v in eng.ctx.kernel_stats().items()}
    if args.graph:
        eng.solve_counters(reset=True)
    stream = torch.cuda.current_stream()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    ev0.record(stream)
    results = []
    for _ in range(args.steps):
        if args.graph:
            eng.advance_graph(dt)
        else:
            results.append(eng.advance(dt))
    ev1.record(stream)
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    clocks = sampler.stop()
    ms = ev0.elapsed_time(ev1)
    ms_max, value = aggregate(ms, n, args.steps, world, device="cuda")
    counts1 = {k: v[0] for k, v in eng.ctx.kernel_stats().items()}
    launches = int(sum(counts1.values()) - sum(counts0.get(k, 0) for k in counts1))  # eager calls (sorts)
    if args.graph:
        sc = eng.solve_counters(reset=True)
        g = eng.last_graph
        launches += args.steps * g.fixed_launches + sc["cycles"] * g.body_launches
        cycles = [sc["cycles"] / max(sc["solves"], 1)]
        rel = [sc["max_rel_residual"]]
        all_conv = sc["solves"] == args.steps and sc["max_rel_residual"] < args.tol
    else:
        cycles = [r.cycles for r in results]
        rel = [r.rel_residual for r in results]
        all_conv = all(r.converged for r in results)

    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_max / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": value / REFERENCE_PUBLISHED, "dtype": "f32", "data": "synthetic",
        "config": {
            "workload": f"{args.config}: {n:,} particles (two-disk collision), {G}^3 grid, box "
                        f"[{cfg['origin'][0]:g},{-cfg['origin'][0]:g}]^3, dt={dt}, seed {cfg['seed']}, "
                        f"multigrid to {args.tol:g} relative residual, int64 deposit quantum 2^-{bits} of the total",
            "warm_start": args.warmstart, "precision": args.precision, "sweeps": [args.pre_sweeps, args.post_sweeps],
            "coarse_level_sweeps": None if args.precision == "plain_f32" else args.coarse_level_sweeps,
            "sort_every": args.sort_every,
            "sort_ahead": args.sort_every / 2.0 if args.sort_ahead is None else args.sort_ahead, "particles_per_gpu": n, "grid": G, "parallelism": f"replicas x{world}",
            "l2": "inputs larger than L2: 32 B/particle state = %.1f GB per GPU" % (n * 32 / 1e9),
            "vs_baseline_ref": "reference RTX 3070 published 6.95 steps/s at 100M, 256^3 (its tol 1e-3)",
        },
        "clocks": clocks,
        "gpu_launches": launches,
        "poisson": {"mean_vcycles": float(np.mean(cycles)), "max_rel_residual": float(max(rel)),
                    "all_converged": bool(all_conv) if args.precision == "mixed" else False,
                    "step": ("one CUDA graph replay per step, V-cycle count decided on the device" if args.graph
                             else "eager launches, residual read on the host after every V-cycle")},
    }

    if rank == 0:
        # roofline: CUDA-event time of each kernel's launches over a few more steps
        eng.ctx.profile_reset()
        eng.ctx.profile(True)
        for _ in range(args.profile_steps):
            eng.advance(dt)
        stats = eng.ctx.kernel_stats()
        eng.ctx.profile(False)
        tot = sum(v[2] for v in stats.values()) or 1.0
        line["per_kernel_ms_per_step"] = {k: round(v[2] / args.profile_steps, 4) for k, v in
                                          sorted(stats.items(), key=lambda kv: -kv[1][2])}
        line["kernel_share"] = {k: round(v[2] / tot, 4) for k, v in sorted(stats.items(), key=lambda kv: -kv[1][2])}
        line["roofline"] = _roofline(stats, n, G, hbm, _load_traffic())
        # one re-sort of the current state (the sort period's), CUDA-event ms per kernel group
        eng.ctx.profile_reset()
        eng.ctx.profile(True)
        eng.sort(dt)
        sort_stats = eng.ctx.kernel_stats()
        eng.ctx.profile(False)
        line["cell_sort_ms"] = {k: round(v[2], 4) for k, v in sorted(sort_stats.items(), key=lambda kv: -kv[1][2])}
        poisson_ms = sum(v[2] for k, v in stats.items() if k in MG_KERNELS) / args.profile_steps
        line["poisson"]["ms_per_solve"] = round(poisson_ms, 4)
        line["poisson"]["warm_start"] = args.warmstart

        del eng  # its blocks stay in torch's cache for the e2e engine (no cudaMalloc in that timed region)
        if not args.no_accuracy:
            line["accuracy_schedule"] = _accuracy_schedule(args, icr, make_engine, dt)
            line["accuracy"] = dict(line["accuracy_schedule"][-1])
            line["accuracy"]["note"] = (
                "relative L2 over the grid (phi) and over all particles and components (CIC-gathered -grad phi) "
                "of the engine's synchronised state against three FP64 references of the same density: the "
                "zero-padded FFT with the reference's continuum kernel (fft: discretisation + boundary + "
                "solver), the same FFT with the lattice Green's function of the 7-point Laplacian (lattice: "
                "boundary + solver) and the multigrid converged to 1e-10 (converged: solver); last sample of "
                "accuracy_schedule")
            torch.cuda.empty_cache()
        if not args.no_e2e:
            line["e2e"] = _e2e(args, icr, make_engine, dt)
        torch.cuda.empty_cache()
        if args.compare_steps > 0:
            line["poisson_comparison"] = _compare_warm_starts(icr, make_engine, dt, args.compare_steps)
        if args.plain_steps > 0:
            line["plain_chain"] = _plain_chain(icr, cfg, args.tol, args.plain_steps, min(args.warmup, 3))
            line["plain_chain"]["fused_speedup"] = round(line["plain_chain"]["ms_per_step"] /
                                                         line["ms_per_step"], 3)
        if not args.no_cpu_baseline and world == 1:
            line["cpu_baseline"] = _cpu_baseline(args, icr, cfg, n, G, dx, dt)
    if world > 1:
        torch.distributed.destroy_process_group()
    if rank == 0:
        print(json.dumps(line), flush=True)


def _accuracy_schedule(args, icr, make_engine, dt):
    """The precision configuration's check: a fresh run of ``accuracy_steps``
    steps from the same initial conditions, the potential and force errors of
    its synchronised state against the FP64 references (see force_chain_errors)
    at step 0 and every ``accuracy_every`` steps."""
    import torch
    from galaxy_collision_gb300.accuracy import force_chain_errors

    eng = make_engine()
    eng.load(icr.pos, icr.vel, icr.mass, icr.gid, sort=True)
    solvers = {}  # the two 512^3 FP64 kernels are transformed once

    def sample(step):
        acc = force_chain_errors(eng, solvers=solvers)
        row = {"step": step}
        row.update({k: (float(f"{v:.4e}") if isinstance(v, float) else v) for k, v in acc.items()})
        return row

    eng.evaluate(diagnostics=False)  # the potential of the initial state
    rows = [sample(0)]
    done = 0
    while done < args.accuracy_steps:
        k = min(args.accuracy_every, args.accuracy_steps - done)
        eng.prime(dt)
        for _ in range(k - 1):
            eng.advance(dt)
        eng.synchronize(dt)
        done += k
        rows.append(sample(done))
    del eng, solvers
    torch.cuda.empty_cache()
    return rows


def _load_net():
    """The trained warm-start network shipped with the package (None if absent)."""
    from galaxy_collision_gb300.warmstart import WEIGHTS_PATH, WarmStartNet

    return WarmStartNet.load(WEIGHTS_PATH) if WEIGHTS_PATH.exists() else None


def _compare_warm_starts(icr, make_engine, dt, steps, warm=4):
    """V-cycles and solve time to the same relative residual from each initial
    guess: plain (previous potential, the reference's warm start), linear
    extrapolation, and extrapolation + the trained network (when its weights are
    present). Same initial conditions; CUDA-event time of each kernel."""
    import torch

    out = {}
    modes = ["plain_f32", "plain", "extrapolate"] + (["learned"] if _load_net() is not None else [])
    for mode in modes:
        # plain_f32: the plain FP32 chain (previous-step warm start, all-FP32 multigrid, the reference's cap
        # of 20 V-cycles since it cannot reach the tolerance)
        eng = make_engine("plain", plain_f32=True) if mode == "plain_f32" else make_engine(mode)
        eng.load(icr.pos, icr.vel, icr.mass, icr.gid, sort=True)
        eng.prime(dt)
        for _ in range(warm):
            eng.advance(dt)
        eng.ctx.profile_reset()
        eng.ctx.profile(True)
        ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        ev0.record()
        res = [eng.advance(dt) for _ in range(steps)]
        ev1.record()
        torch.cuda.synchronize()
        stats = eng.ctx.kernel_stats()
        eng.ctx.profile(False)
        solve = sum(v[2] for k, v in stats.items() if k in MG_KERNELS + ("warmstart",)) / steps
        out[mode] = {"mean_vcycles": float(np.mean([r.cycles for r in res])),
                     "max_rel_residual": float(max(r.rel_residual for r in res)),
                     "ms_per_solve": round(solve, 4),
                     "initial_guess_ms": round(stats.get("warmstart", (0, 0, 0.0))[2] / steps, 4),
                     "ms_per_step": round(ev0.elapsed_time(ev1) / steps, 4)}
        del eng
        torch.cuda.empty_cache()
    out["note"] = ("same initial conditions, steps after a short warm-up; solve = multigrid kernels + faces + "
                   "initial-guess kernels, the network's convolutions included; plain, extrapolate and learned "
                   "reach the same relative residual; plain_f32 is the plain FP32 chain (previous-step warm start, "
                   "all-FP32 multigrid) stopped at the reference's 20 V-cycles with the residual it reached")
    return out


def _plain_chain(icr, cfg, tol, steps, warmup):
    """The reference's stepwise chain on this GPU through the package's drop-in API:
    per force evaluation deposit_density, MultigridPoissonSolver.solve (warm start
    from the previous potential), potential_to_accel into three node grids and
    gather_acceleration into per-particle arrays; kdk_step's kick/drift/kick as
    separate launches (sim.py:320-327, integrator.py:100-131). Same kernels,
    fixed-point quantum and solver tolerance as the fused engine; what differs is
    the fusion, so the ratio is what the fused step buys."""
    import torch
    from galaxy_collision_gb300.data import Field, GridState, ParticleState
    from galaxy_collision_gb300.deposit import deposit_density, gather_acceleration, potential_to_accel
    from galaxy_collision_gb300.integrator import kdk_step
    from galaxy_collision_gb300.solver import make_solver

    G, dx, dt = cfg["grid"], cfg["dx"], cfg["dt"]
    bits = cfg.get("fixed_point_bits", 52)
    n = icr.n
    parts = ParticleState(n)
    pos = torch.from_numpy(icr.pos).cuda().to(torch.float64) - torch.tensor(cfg["origin"], dtype=torch.float64,
                                                                              device="cuda")
    vel = torch.from_numpy(icr.vel).cuda()
    for i, f in enumerate((parts.pos_x, parts.pos_y, parts.pos_z)):
        f.tensor.copy_(pos[:, i].to(torch.float32))
    for i, f in enumerate((parts.vel_x, parts.vel_y, parts.vel_z)):
        f.tensor.copy_(vel[:, i])
    parts.mass.tensor.copy_(torch.from_numpy(icr.mass).cuda())
    del pos, vel
    grid = GridState(G)
    acc = [Field(n) for _ in range(3)]
    solver = make_solver("multigrid", G, dx=dx, grav_constant=1.0, tol=tol, n_cycles=60)
    warm = {"on": False}
    cycles = []

    def accel_fn():
        deposit_density(parts, grid.rho, dx, fixed_point_bits=bits)
        solver.solve(grid.rho, grid.phi, warm_start=warm["on"])
        warm["on"] = True
        cycles.append(solver.last_cycles)
        potential_to_accel(grid.phi, grid.ax, grid.ay, grid.az, dx)
        gather_acceleration(parts, grid.ax, grid.ay, grid.az, *acc, dx)

    accel_fn()
    for _ in range(warmup):
        kdk_step(parts, *acc, accel_fn, dt)
    stream = torch.cuda.current_stream()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    cycles.clear()
    ev0.record(stream)
    for _ in range(steps):
        kdk_step(parts, *acc, accel_fn, dt)
    ev1.record(stream)
    torch.cuda.synchronize()
    ms = ev0.elapsed_time(ev1) / steps
    out = {"value": n / (ms / 1e3), "unit": UNIT, "ms_per_step": round(ms, 4), "steps": steps,
           "mean_vcycles": float(np.mean(cycles)),
           "note": "stepwise chain through deposit_density / MultigridPoissonSolver.solve(warm_start) / "
                   "potential_to_accel / gather_acceleration / kdk_step on this GPU, same solver tolerance"}
    del parts, grid, acc, solver
    torch.cuda.empty_cache()
    return out


def _e2e(args, icr, make_engine, dt):
    """Same metric through the public API with host buffers: pinned host state ->
    device (load + cell sort), prime, K-1 steps, close, state back to the host."""
    import torch

    pos = torch.from_numpy(icr.pos).pin_memory()
    vel = torch.from_numpy(icr.vel).pin_memory()
    mass = torch.from_numpy(icr.mass).pin_memory()
    gid = torch.from_numpy(icr.gid).pin_memory()
    out_pos = torch.empty((icr.n, 3), dtype=torch.float32).pin_memory()
    out_vel = torch.empty((icr.n, 3), dtype=torch.float32).pin_memory()
    eng = make_engine()
    eng.reserve(icr.n)  # construction: particle sets and sort scratch allocated before the timed region
    # the first DMA from freshly pinned pages costs the driver's one-time mapping
    # (up to ~75 ms for these buffers); pinning is set-up, so it happens here
    stage = eng.alt["_block"]
    for t in (pos, vel, mass, gid):
        stage[:t.numel()].view(t.dtype).view(t.shape).copy_(t, non_blocking=True)
    for t in (out_pos, out_vel):
        t.copy_(stage[:t.numel()].view(t.shape), non_blocking=True)
    torch.cuda.synchronize()
    marks = []

    def mark(name):
        if args.verbose:  # phase breakdown (synchronising) only when asked for
            torch.cuda.synchronize()
            marks.append((name, time.perf_counter()))

    if args.verbose:
        eng.ctx.profile_reset()
        eng.ctx.profile(True)
    t0 = time.perf_counter()
    eng.load(pos, vel, mass, gid, sort=True)  # pinned host arrays: staged H2D + gc_pm_import_sorted
    mark("load+sort")
    if args.verbose:
        _log(args, "e2e load kernels (ms): " + ", ".join(f"{k} {v[2]:.2f}" for k, v in eng.ctx.kernel_stats().items()
                                                       if v[2] > 0))
        eng.ctx.profile(False)
    eng.prime(dt)
    mark("prime")
    for _ in range(args.steps - 1):
        eng.advance(dt)
    mark("advance")
    eng.synchronize(dt, diagnostics=True)
    mark("close")
    eng.export(out_pos, out_vel)  # gc_pm_export (original order, physical) + pinned D2H
    torch.cuda.synchronize()
    t = time.perf_counter() - t0
    if args.verbose:
        prev = t0
        for name, tm in marks:
            _log(args, f"e2e {name}: {1e3 * (tm - prev):.1f} ms")
            prev = tm
        _log(args, f"e2e state back: {1e3 * (t0 + t - prev):.1f} ms")
    n = icr.n
    return {"value": n * args.steps / t, "unit": UNIT, "h2d_bytes_per_step": int(n * 32 / args.steps),
            "d2h_bytes_per_step": int((n * 24 + 12 * 8) / args.steps),
            "note": "wall clock around load (pinned H2D of the reference layout, cell sort and gather into cell order), "
                    "prime, steps-1 advances, close with diagnostics, export in the original order + "
                    "pinned D2H of positions and velocities (the pinned buffers are mapped by one untimed transfer "
                    "before, as part of pinning)"}


def run_reference(args):
    rank, world, _ = _dist()
    if rank != 0:
        return
    from galaxy_collision_gb300 import ic

    icr, cfg = ic.build(args.config, scale=args.scale)
    G, dx, dt = cfg["grid"], cfg["dx"], cfg["dt"]
    pos_grid = (icr.pos.astype(np.float64) - np.asarray(cfg["origin"])).astype(np.float32)
    budget = max(30.0, min(150.0, 12.0 * (args.steps + args.warmup)))
    from oracle import pm

    w_times, _, _ = _reference_chain(pos_grid, icr.vel, icr.mass, G, dx, dt, min(args.warmup, 1), budget / 4)
    times, cyc, ratio = _reference_chain(pos_grid, icr.vel, icr.mass, G, dx, dt, args.steps, budget)
    n = icr.n
    value = n * len(times) / sum(times)
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": len(times),
        "warmup": len(w_times), "ms_per_step": 1e3 * sum(times) / len(times), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": value / REFERENCE_PUBLISHED, "dtype": "f32", "data": "synthetic",
        "impl": "reference",
        "config": {"workload": f"{args.config}: {n:,} particles, {G}^3 grid (the same workload as the GPU arm)",
                   "implementation": "reference PM chain (deposit f32 atomics, multigrid tol=1e-3 n_cycles=20, "
                                     "grad, gather, KDK) restated in C from its Taichi kernels; OpenMP on all "
                                     "host threads",
                   "requested_steps": args.steps},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": pm.num_threads(), "kind": "port",
                         "sample": f"{len(times)} of {args.steps} requested KDK steps of the full workload "
                                   f"(bounded to ~{budget:.0f} s); last solve {cyc} cycles, residual ratio "
                                   f"{ratio:.2e}"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def main(argv=None):
    args = _parse(argv)
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
