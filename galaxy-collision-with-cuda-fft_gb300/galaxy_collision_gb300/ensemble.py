"""Batched ensemble of independent collisions on one GPU.

Many small runs cannot fill a GB300 one at a time: a 64^3 or 128^3 grid step is
a few hundred microseconds of mostly latency-bound kernels, and each solve of
the adaptive multigrid reads its residual on the host. The ensemble advances
all runs together. Every engine solves with one V-cycle (enough for 1e-6 from
the extrapolated warm start at almost every step) and writes its residual to
pinned host memory; the solves of all runs are captured into ONE CUDA graph
with one stream branch per run, the particle passes into a second one. Between
the two replays the host reads every run's residual after one synchronisation
and runs extra V-cycles for the few runs above the tolerance, so every solve
still meets it. Replaying a graph launches every kernel of every run with no
host gaps and lets independent runs overlap on the SMs. Runs are sorted at the
same steps, so one pair of graphs per particle-buffer parity covers the run.

Workload (the batched-ensemble configuration): 64 two-disk collisions with
particle counts log-uniform in [0.25M, 4M], 64^3 grids below 1M particles and
128^3 otherwise, geometry randomised as in the training set. The comparison is
the same runs advanced one after the other with the adaptive solve.

Command line::

    python -m galaxy_collision_gb300.ensemble --runs 64 --steps 300
"""

from __future__ import annotations

import argparse
import json
import time

import numpy as np
import torch

from galaxy_collision_gb300 import _native
from galaxy_collision_gb300.engine import PMEngine
from galaxy_collision_gb300.warmstart_train import random_collision

BOX, DT = 64.0, 0.005


def ensemble_members(n_runs: int, seed: int = 5, n_min: float = 2.5e5, n_max: float = 4e6):
    """(particle count, grid) per run: counts log-uniform in [n_min, n_max]."""
    rng = np.random.default_rng(seed)
    counts = np.exp(rng.uniform(np.log(n_min), np.log(n_max), size=n_runs)).astype(np.int64)
    return [(int(n), 64 if n < 1_000_000 else 128) for n in counts], rng


class Ensemble:
    """Independent PM engines advanced together through one multi-stream CUDA graph."""

    def __init__(self, n_runs: int = 64, seed: int = 5, tol: float = 1e-6, warmstart: str = "extrapolate",
                 fixed_cycles: int = 1, sort_every: int = 20, dt: float = DT, box: float = BOX, net=None):
        members, rng = ensemble_members(n_runs, seed)
        self.dt = dt
        self.fixed_cycles = int(fixed_cycles)
        self.engines: list[PMEngine] = []
        self.counts = []
        for n, grid in members:
            icr = random_collision(rng, n, box / grid)
            e = PMEngine(grid, box / grid, grav=1.0, origin=(-box / 2.0,) * 3, tol=tol, sort_every=sort_every,
                         fixed_point_bits=40, fixed_cycles=fixed_cycles)
            e.set_warmstart(warmstart, net=net if warmstart == "learned" else None)
            e.load(icr.pos, icr.vel, icr.mass, icr.gid)
            self.engines.append(e)
            self.counts.append(n)
        self.streams = [torch.cuda.Stream() for _ in self.engines]
        self._graphs = {}
        self.steps_since_sort = 0
        self.sort_every = sort_every
        self.extra_cycles = 0

    @property
    def particles(self) -> int:
        return int(sum(self.counts))

    def prime(self, warm_steps: int = 10) -> None:
        """Prime every run and take its first steps with the adaptive solve (until
        the extrapolated start is accurate enough for one V-cycle); the graph
        takes over from there."""
        for e in self.engines:
            fixed = e.fixed_cycles
            self._adaptive(e)
            e.prime(self.dt)
            for _ in range(warm_steps):
                e.advance(self.dt)
            self._fixed(e, fixed)
        torch.cuda.synchronize()
        self.steps_since_sort = max(e.steps_since_sort for e in self.engines)

    @staticmethod
    def _adaptive(e: PMEngine) -> None:
        e.mg.flags &= ~_native.GC_MG_FIXED_CYCLES
        e.mg.max_cycles, e.mg.min_cycles = 60, 1
        e.fixed_cycles = 0

    @staticmethod
    def _fixed(e: PMEngine, cycles: int) -> None:
        e.mg.flags |= _native.GC_MG_FIXED_CYCLES
        e.mg.max_cycles = e.mg.min_cycles = cycles
        e.fixed_cycles = cycles

    def _capture(self, what: str):
        g = torch.cuda.CUDAGraph()
        torch.cuda.synchronize()
        with torch.cuda.graph(g):
            cap = torch.cuda.current_stream()
            for e, s in zip(self.engines, self.streams):
                s.wait_stream(cap)
                with torch.cuda.stream(s):
                    if what == "solve":
                        e.solve_kernels(self.dt)
                    else:
                        e.push_kernels(self.dt)
            for s in self.streams:
                cap.wait_stream(s)
        return g

    def step(self) -> int:
        """One KDK step of every run: the solves of all runs as one graph (fixed
        V-cycles), the residual of each run read from its pinned host copy after one
        synchronisation, extra V-cycles for the runs above the tolerance, then the
        particle passes of all runs as a second graph. Runs are sorted together every
        sort_every steps, outside the graphs. Returns the extra V-cycles run."""
        if self.sort_every > 0 and self.steps_since_sort >= self.sort_every:
            for e in self.engines:
                e.sort()
            self.steps_since_sort = 0
        key = tuple(e.cur["x"].data_ptr() for e in self.engines)
        gs = self._graphs.get(key)
        if gs is None:
            gs = self._graphs[key] = (self._capture("solve"), self._capture("push"))
        gs[0].replay()
        torch.cuda.current_stream().synchronize()
        extra = 0
        for e in self.engines:
            if e.residual_host() >= e.mg.tol:
                extra += e.refine()
        gs[1].replay()
        self.steps_since_sort += 1
        for e in self.engines:
            e.steps_since_sort = self.steps_since_sort
        self.extra_cycles += extra
        return extra

    def max_residual(self) -> float:
        return max(e.last_residual() for e in self.engines)


def run_comparison(n_runs: int = 64, steps: int = 300, seed: int = 5, one_by_one_steps: int | None = None,
                   log=None) -> dict:
    """Aggregate particle-steps/s of the batched graph and of the same runs advanced
    one by one (adaptive solve, one run after the other)."""
    t0 = time.time()
    ens = Ensemble(n_runs, seed=seed)
    if log:
        log(f"{n_runs} runs, {ens.particles:,} particles, IC {time.time() - t0:.0f}s")
    ens.prime()
    # batched: graph replays; the residual of every run is read every 25 steps
    # (outside the timed windows)
    ens.step()  # capture + first replay
    torch.cuda.synchronize()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ms_batched, resid, done = 0.0, 0.0, 0
    while done < steps:
        chunk = min(25, steps - done)
        ev0.record()
        for _ in range(chunk):
            ens.step()
        ev1.record()
        torch.cuda.synchronize()
        ms_batched += ev0.elapsed_time(ev1)
        resid = max(resid, ens.max_residual())
        done += chunk
    # one by one: each run alone with the adaptive solve (host check each V-cycle)
    k = one_by_one_steps or steps
    ms_single = 0.0
    cycles = []
    for e in ens.engines:
        ens._adaptive(e)
        torch.cuda.synchronize()
        ev0.record()
        for _ in range(k):
            cycles.append(e.advance(ens.dt).cycles)
        ev1.record()
        torch.cuda.synchronize()
        ms_single += ev0.elapsed_time(ev1)
    n = ens.particles
    out = {
        "runs": n_runs, "particles": n, "grids": sorted({e.grid_size for e in ens.engines}),
        "batched": {"particle_steps_per_s": n * steps / (ms_batched / 1e3), "ms_per_step": ms_batched / steps,
                    "v_cycles_per_solve": ens.fixed_cycles + ens.extra_cycles / (n_runs * (steps + 1)),
                    "extra_v_cycles": ens.extra_cycles, "max_rel_residual_checked": resid,
                    "residual_check": "every run after every step's fixed cycle (extra cycles below tol); the "
                                      "final residual of every run every 25 steps"},
        "one_by_one": {"particle_steps_per_s": n * k / (ms_single / 1e3), "ms_per_step": ms_single / k,
                       "mean_v_cycles": float(np.mean(cycles))},
        "steps": steps, "one_by_one_steps": k,
    }
    out["speedup"] = out["batched"]["particle_steps_per_s"] / out["one_by_one"]["particle_steps_per_s"]
    return out


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    ap.add_argument("--runs", type=int, default=64)
    ap.add_argument("--steps", type=int, default=300)
    ap.add_argument("--one-by-one-steps", type=int, default=None)
    ap.add_argument("--seed", type=int, default=5)
    args = ap.parse_args(argv)
    from galaxy_collision_gb300 import _build

    _build.build()
    res = run_comparison(args.runs, args.steps, args.seed, args.one_by_one_steps,
                         log=lambda m: print(f"[ensemble] {m}", flush=True))
    print(json.dumps(res), flush=True)


if __name__ == "__main__":
    main()
