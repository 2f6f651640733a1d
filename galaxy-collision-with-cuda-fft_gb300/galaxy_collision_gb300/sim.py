"""Simulation driver over the fused GPU engine (the reference's ``run_simulation``).

Same loop contract as src/galaxy_collision/sim.py:194-450: build the initial
conditions, refuse a box that loses more than 10% of the mass
(sim.py:173-191), prime the force once, advance ``config.steps`` KDK steps,
record conservation diagnostics every ``history_cadence`` steps and write
snapshots every ``config.output_cadence`` steps (plus the last). Each step is
one :meth:`PMEngine.advance` (deposit -> multigrid -> fused gather/kicks/drift);
diagnostics at step n are reduced in FP64 inside that step's particle pass at
the synchronised time. History and snapshot steps close the staggered step
(one extra force evaluation) so the sampled state is synchronised, then re-prime.
"""

from __future__ import annotations

from pathlib import Path
from typing import Any

import numpy as np

from galaxy_collision_gb300 import ic as ic_mod
from galaxy_collision_gb300 import units
from galaxy_collision_gb300.config import SimConfig


def check_box_fit(pos_grid: np.ndarray, mass: np.ndarray, grid_size: int, dx: float, tol: float = 0.10) -> None:
    """Fail loudly if more than ``tol`` of the mass lies outside the node box (sim.py:173-191)."""
    hi = (grid_size - 1) * dx
    outside = np.any((pos_grid < 0.0) | (pos_grid > hi), axis=1)
    frac = float(mass[outside].astype(np.float64).sum() / mass.astype(np.float64).sum())
    if frac > tol:
        raise ValueError(f"{frac:.1%} of the IC mass lies outside the {grid_size}^3 box — the initial "
                         f"conditions do not fit (check grid_size vs galaxy placement/separation).")


def build_ic(config: SimConfig) -> ic_mod.ICResult:
    if config.ic_preset == "plummer_131k":
        return ic_mod.plummer(config.n_particles or 131072, seed=config.seed)
    if config.ic_preset == "two_disk":
        n = config.n_particles or 10_000_000
        return ic_mod.two_disk(int(0.4 * n), n - int(0.4 * n), seed=config.seed, dx=config.dx)
    if config.ic_preset == "plummer":
        # the reference's default sphere: M = 1e10 M_sun, a = 5 kpc, at the box centre
        g = units.G if config.grav_constant is None else config.grav_constant
        m_tot, a = 1.0e10, 5.0
        p = ic_mod.plummer(config.n_particles or 10_000, seed=config.seed, rmax=20.0)
        c = config.box_lo + config.grid_size * config.dx / 2.0
        vscale = np.sqrt(g * m_tot / a)
        return ic_mod.ICResult((p.pos * a + c).astype(np.float32), (p.vel * vscale).astype(np.float32),
                               (p.mass * m_tot).astype(np.float32), p.gid)
    raise NotImplementedError(f"ic_preset {config.ic_preset!r} has no GPU-engine builder "
                              f"(available: plummer, plummer_131k, two_disk)")


def run_simulation(config: SimConfig, *, history_cadence: int | None = None, write_snapshots: bool = True,
                   icr: ic_mod.ICResult | None = None, tracer_indices=None, direct_pe_softening: float | None = None,
                   half_mass: bool = True) -> dict[str, Any]:
    """Run ``config.steps`` KDK steps; return the reference's summary keys and history.

    History and snapshot steps are taken at synchronised states: the engine closes
    the step (FP64 diagnostics reduced in the same particle pass), the sample is
    recorded, and the engine re-primes (one extra force evaluation per sample).
    """
    from galaxy_collision_gb300 import diagnostics as host_diag
    from galaxy_collision_gb300 import diagnostics_device as dd
    from galaxy_collision_gb300.engine import PMEngine
    from galaxy_collision_gb300.io import snapshot_from_engine, write_snapshot

    icr = icr if icr is not None else build_ic(config)
    grav = units.G if config.grav_constant is None else config.grav_constant
    check_box_fit(icr.pos.astype(np.float64) - config.box_lo, icr.mass, config.grid_size, config.dx)
    eng = PMEngine(config.grid_size, config.dx, grav=grav, origin=(config.box_lo,) * 3, tol=config.solver_tol,
                   max_cycles=config.solver_max_cycles, fixed_point_bits=config.fixed_point_bits,
                   sort_every=config.sort_every)
    eng.load(icr.pos, icr.vel, icr.mass, icr.gid, sort=True)
    tracers = None if tracer_indices is None else [int(i) for i in np.atleast_1d(tracer_indices)]
    hist_cad = history_cadence or max(1, config.steps // 20)
    diag = dd.DeviceDiagnostics(config.grid_size, nbins=2048, r_max=config.grid_size * config.dx * np.sqrt(3.0))
    mass_np = icr.mass.astype(np.float64)
    history: list[dict[str, Any]] = []
    snapshots: list[str] = []
    cycles: list[int] = []

    def record(step: int, res) -> dict[str, Any]:
        d = eng.diagnostics_physical(res.diag)
        pe = 0.5 * config.dx**3 * res.grid_pe_raw
        rec = {"step": step, "time": step * config.dt, "kinetic": d["kinetic"], "potential": pe,
               "energy": d["kinetic"] + pe, "momentum": d["momentum"], "ang_momentum": d["ang_momentum"],
               "center_of_mass": d["center_of_mass"], "virial": d["kinetic"] / abs(pe) if pe else float("nan"),
               "solver_cycles": res.cycles, "rel_residual": res.rel_residual}
        if half_mass:
            rec["half_mass_radius"] = _half_mass(diag, eng, d)
        if tracers is not None or direct_pe_softening is not None:
            pos_t, _, _, _ = eng.state_arrays(physical=True)
            pos_np = pos_t.cpu().numpy()
            if tracers is not None:
                rec["tracer_pos"] = pos_np[tracers]
            if direct_pe_softening is not None:
                pd = host_diag.potential_energy_direct(mass_np, pos_np, direct_pe_softening, grav)
                rec["potential_direct"] = pd
                rec["energy_direct"] = d["kinetic"] + pd
        return rec

    def snapshot(step: int, rec: dict) -> None:
        keys = ("energy", "kinetic", "potential", "momentum", "ang_momentum", "virial")
        snap = snapshot_from_engine(step, step * config.dt, eng, {k: np.asarray(rec[k]) for k in keys})
        snapshots.append(str(write_snapshot(snap, Path(config.output_dir) / f"snapshot_{step:05d}.npz")))

    def snap_due(s: int) -> bool:
        return write_snapshots and config.output_cadence > 0 and (s % config.output_cadence == 0
                                                                   or s == config.steps)

    # step 0: a force evaluation without moving the particles gives the initial diagnostics
    res = eng.evaluate(diagnostics=True)
    cycles.append(res.cycles)
    history.append(record(0, res))
    if snap_due(0):
        snapshot(0, history[0])
    eng.prime(config.dt)
    for step in range(1, config.steps + 1):
        sample = step % hist_cad == 0 or step == config.steps or snap_due(step)
        if sample:
            res = eng.synchronize(config.dt, diagnostics=True)
            cycles.append(res.cycles)
            rec = record(step, res)
            history.append(rec)
            if snap_due(step):
                snapshot(step, rec)
            if step < config.steps:
                eng.prime(config.dt)
        else:
            cycles.append(eng.advance(config.dt).cycles)
    e0, ef = history[0]["energy"], history[-1]["energy"]
    return {
        "name": config.name, "preset": config.ic_preset, "solver": config.solver, "n_particles": eng.n,
        "grid_size": config.grid_size, "steps": config.steps, "dt": config.dt,
        "energy_initial": e0, "energy_final": ef,
        "energy_drift": abs((ef - e0) / e0) if e0 else float("nan"),
        "energy_drift_max": max(abs((h["energy"] - e0) / e0) for h in history) if e0 else float("nan"),
        "virial_final": history[-1]["virial"], "mean_solver_cycles": float(np.mean(cycles)),
        "history": history, "snapshots": snapshots, "engine": eng, "status": "ok",
    }


def _half_mass(diag, eng, d) -> float:
    """Half-mass radius about the centre of mass from the device radial histogram."""

    class _View:
        pass

    v = _View()
    v.n = eng.n
    v.pos_x, v.pos_y, v.pos_z, v.mass = eng.cur["x"], eng.cur["y"], eng.cur["z"], eng.cur["m"]
    cm_grid = np.asarray(d["center_of_mass"]) - eng.origin
    return diag._half_mass_radius(v, float(cm_grid[0]), float(cm_grid[1]), float(cm_grid[2]), d["M"])


__all__ = ["run_simulation", "build_ic", "check_box_fit"]
