"""Batched ensemble of independent collisions on one GPU.

Many small runs cannot fill a GB300 one at a time: a 64^3 or 128^3 grid step is
a few hundred microseconds of mostly latency-bound kernels. The ensemble
advances all runs together: every run's whole KDK step is one CUDA graph
(``gc_pm_graph_create``: deposit, conversion, initial guess, faces, the
adaptive multigrid with its stopping rule decided on the device by a
conditional while node, the particle pass), and each step replays all runs'
graphs at once, each on its own stream, ordered only after the work that
precedes the step (the periodic cell sort). No host synchronisation happens
inside a step and every solve meets the tolerance on its own; independent runs
overlap on the SMs. The solve counters of each run (solves, V-cycles, largest
residual) are read on the device after the timed steps.

Workload (the batched-ensemble configuration): 64 two-disk collisions with
particle counts log-uniform in [0.25M, 4M], 64^3 grids below 1M particles and
128^3 otherwise, geometry randomised as in the training set. The comparison is
the same runs advanced one after the other, each through its own step graph.
The runs' coarse multigrid levels are launched phase by phase
(GC_MG_PHASE_LAUNCHES): at 64^3 and 128^3 that is faster than the persistent
cooperative kernels, alone and side by side.

Command line::

    python -m galaxy_collision_gb300.ensemble --runs 64 --steps 300
"""

from __future__ import annotations

import argparse
import json
import time

import numpy as np
import torch

from galaxy_collision_gb300.engine import PMEngine
from galaxy_collision_gb300.warmstart_train import random_collision

BOX, DT = 64.0, 0.005


def ensemble_members(n_runs: int, seed: int = 5, n_min: float = 2.5e5, n_max: float = 4e6):
    """(particle count, grid) per run: counts log-uniform in [n_min, n_max]."""
    rng = np.random.default_rng(seed)
    counts = np.exp(rng.uniform(np.log(n_min), np.log(n_max), size=n_runs)).astype(np.int64)
    return [(int(n), 64 if n < 1_000_000 else 128) for n in counts], rng


class Ensemble:
    """Independent PM engines advanced together, one whole-step graph per run per step."""

    def __init__(self, n_runs: int = 64, seed: int = 5, tol: float = 1e-6, warmstart: str = "extrapolate",
                 sort_every: int = 20, dt: float = DT, box: float = BOX, net=None, phase_launches: bool = True,
                 tuned: bool = False):
        members, rng = ensemble_members(n_runs, seed)
        self.dt = dt
        self.engines: list[PMEngine] = []
        self.counts = []
        ics = [random_collision(rng, n, box / grid) for n, grid in members]

        def make(grid, **settings):
            e = PMEngine(grid, box / grid, grav=1.0, origin=(-box / 2.0,) * 3, tol=tol, fixed_point_bits=40,
                         **settings)
            e.set_warmstart(warmstart, net=net if warmstart == "learned" else None)
            return e

        # per (grid, particle-count bucket): the tuned settings (autotune.py), timed on
        # the group's first run when the cache has none; otherwise the given ones
        settings = {}
        if tuned:
            import torch

            from galaxy_collision_gb300 import autotune

            device = torch.cuda.get_device_name()
            for (n, grid), icr in zip(members, ics):
                k = (grid, autotune.bucket(n))
                if k not in settings:
                    settings[k] = autotune.settings_for(
                        grid, n, lambda g=grid, **st: make(g, **st), (icr.pos, icr.vel, icr.mass, icr.gid), dt,
                        device=device)
        self.settings = []
        for (n, grid), icr in zip(members, ics):
            st = settings.get((grid, int(n).bit_length() - 1)) if tuned else None
            st = st or {"phase_launches": phase_launches, "sort_every": sort_every}
            e = make(grid, **st)
            e.load(icr.pos, icr.vel, icr.mass, icr.gid)
            self.engines.append(e)
            self.counts.append(n)
            self.settings.append(st)

    @property
    def particles(self) -> int:
        return int(sum(self.counts))

    def prime(self, warm_steps: int = 3) -> None:
        """Prime every run, take the eager steps that fill its warm-start
        history, and capture its step graphs (both particle-buffer sets)."""
        for e in self.engines:
            e.prime(self.dt)
            for _ in range(warm_steps):
                e.advance(self.dt)
            e.steps_since_sort = 0
            e.prepare_graphs(self.dt)
        torch.cuda.synchronize()
        for e in self.engines:
            e.solve_counters(reset=True)

    def step(self) -> None:
        """One KDK step of every run: the runs due for their cell sort are
        sorted (on the current stream), then every run's step graph is replayed
        on its own stream after that, and the current stream waits for all of
        them."""
        main = torch.cuda.current_stream()
        for e in self.engines:
            if e.sort_every > 0 and e.steps_since_sort >= e.sort_every:
                e.sort(self.dt)
        ready = torch.cuda.Event()
        ready.record(main)
        streams = []
        for e in self.engines:
            e._graph_stream().wait_event(ready)
            streams.append(e.launch_graph(self.dt))
        for s in streams:
            main.wait_stream(s)

    def counters(self, reset: bool = True) -> dict:
        """Solves, V-cycles and the largest relative residual over all runs since
        the last reset (synchronises)."""
        c = [e.solve_counters(reset=reset) for e in self.engines]
        return {"solves": sum(x["solves"] for x in c), "cycles": sum(x["cycles"] for x in c),
                "max_rel_residual": max(x["max_rel_residual"] for x in c)}


def run_comparison(n_runs: int = 64, steps: int = 300, seed: int = 5, one_by_one_steps: int | None = None,
                   log=None, phase_launches: bool = True, tuned: bool = False) -> dict:
    """Aggregate particle-steps/s of the ensemble step and of the same runs
    advanced one after the other (each through its own step graph)."""
    t0 = time.time()
    ens = Ensemble(n_runs, seed=seed, phase_launches=phase_launches, tuned=tuned)
    if log:
        log(f"{n_runs} runs, {ens.particles:,} particles, IC {time.time() - t0:.0f}s")
    ens.prime()
    ens.step()
    torch.cuda.synchronize()
    ens.counters(reset=True)
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ev0.record()
    for _ in range(steps):
        ens.step()
    ev1.record()
    torch.cuda.synchronize()
    ms_batched = ev0.elapsed_time(ev1)
    cb = ens.counters(reset=True)
    # one by one: each run alone, one step graph after the other
    k = one_by_one_steps or steps
    ms_single = 0.0
    for e in ens.engines:
        torch.cuda.synchronize()
        ev0.record()
        for _ in range(k):
            e.advance_graph(ens.dt)
        ev1.record()
        torch.cuda.synchronize()
        ms_single += ev0.elapsed_time(ev1)
    cs = ens.counters(reset=True)
    n = ens.particles
    out = {
        "runs": n_runs, "particles": n, "grids": sorted({e.grid_size for e in ens.engines}),
        "batched": {"particle_steps_per_s": n * steps / (ms_batched / 1e3), "ms_per_step": ms_batched / steps,
                    "v_cycles_per_solve": cb["cycles"] / max(cb["solves"], 1),
                    "max_rel_residual": cb["max_rel_residual"], "solves": cb["solves"]},
        "one_by_one": {"particle_steps_per_s": n * k / (ms_single / 1e3), "ms_per_step": ms_single / k,
                       "v_cycles_per_solve": cs["cycles"] / max(cs["solves"], 1),
                       "max_rel_residual": cs["max_rel_residual"]},
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
    ap.add_argument("--persistent-coarse", action="store_true",
                    help="coarse multigrid levels by the persistent kernels instead of one launch per phase")
    ap.add_argument("--autotune", action="store_true",
                    help="per (grid, particle-count bucket) settings from the autotuner's JSON cache (tuned on "
                         "first use)")
    args = ap.parse_args(argv)
    from galaxy_collision_gb300 import _build

    _build.build()
    res = run_comparison(args.runs, args.steps, args.seed, args.one_by_one_steps,
                         log=lambda m: print(f"[ensemble] {m}", flush=True),
                         phase_launches=not args.persistent_coarse, tuned=args.autotune)
    print(json.dumps(res), flush=True)


if __name__ == "__main__":
    main()
