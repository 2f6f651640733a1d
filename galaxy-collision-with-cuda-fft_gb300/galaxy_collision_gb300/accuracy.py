"""Potential and force error of the engine's force chain against FP64 references.

For a synchronised engine (the potential in the context belongs to the current
positions) this measures, on the device:

* ``phi_vs_fft`` / ``force_vs_fft`` -- relative L2 error against the FP64
  zero-padded isolated FFT convolution (``FFTPoissonSolver``, pad factor 2, the
  reference's validation solver, solver/fft_oracle.py:54-109). This is the
  model error of the open-boundary 7-point discretisation plus the solver's.
* ``phi_vs_lattice`` / ``force_vs_lattice`` -- the same against the FP64 FFT
  convolution with the lattice Green's function of the 7-point Laplacian
  (``FFTPoissonSolver(green="lattice")``): the exact free-space solution of the
  discrete problem, so this is the multipole boundary's error plus the
  solver's, without the discretisation.
* ``phi_vs_converged`` / ``force_vs_converged`` -- the same against the
  multigrid driven to a 1e-10 relative residual on the same density: the error
  that stopping at the working tolerance leaves.
* ``phi_isolated_vs_lattice`` / ``force_isolated_vs_lattice`` -- the multigrid
  with the isolated boundary (``boundary="isolated"``: James's method, faces
  from the lattice Green's function) at the engine's working tolerance, against
  the lattice-Green solution: the solver's error alone, without the multipole
  boundary's.

Forces are -grad(phi) (deposit.py:132-174) CIC-gathered at every particle
(deposit.py:85-129); the error is ||a - a_ref||_2 / ||a_ref||_2 over all
particles and components. The density is re-deposited from the engine's
particles with the engine's fixed-point quantum, which reproduces the engine's
own density bit for bit.
"""

from __future__ import annotations

from types import SimpleNamespace

import torch

from galaxy_collision_gb300.deposit import deposit_density, gather_acceleration, potential_to_accel


def _rel_l2(a: torch.Tensor, ref: torch.Tensor) -> float:
    d = (a.to(torch.float64) - ref.to(torch.float64)).square().sum()
    r = ref.to(torch.float64).square().sum()
    return float((d / r).sqrt().item()) if float(r.item()) > 0 else float("nan")


def _forces(parts, phi: torch.Tensor, dx: float):
    grids = [torch.empty_like(phi) for _ in range(3)]
    potential_to_accel(phi, *grids, dx)
    acc = [torch.empty(parts.n, dtype=torch.float32, device=phi.device) for _ in range(3)]
    gather_acceleration(parts, *grids, *acc, dx)
    del grids
    return torch.stack(acc, 0)


def force_chain_errors(eng, *, pad_factor: int = 2, converged_tol: float = 1e-10, with_fft: bool = True,
                       with_lattice: bool = True, with_isolated: bool = True, solvers: dict | None = None) -> dict:
    """Relative-L2 errors of the engine's current potential and particle forces."""
    from galaxy_collision_gb300.solver import make_solver

    if eng.state != "synced":
        raise RuntimeError("force_chain_errors needs a synchronised engine (call synchronize first)")
    G, dx = eng.grid_size, eng.dx
    parts = SimpleNamespace(n=eng.n, pos_x=eng.cur["x"], pos_y=eng.cur["y"], pos_z=eng.cur["z"], mass=eng.cur["m"])
    rho = torch.empty((G, G, G), dtype=torch.float32, device=eng.cur["x"].device)
    deposit_density(parts, rho, dx, fixed_point_bits=eng.fixed_point_bits)
    phi = eng.potential()
    a = _forces(parts, phi, dx)
    out = {"grid": G, "particles": eng.n}

    mg = make_solver("multigrid", G, dx=dx, grav_constant=eng.grav, tol=converged_tol, n_cycles=80)
    phi_c = torch.empty_like(phi)
    mg.solve(rho, phi_c)
    out["converged_rel_residual"] = mg.last_stats["res_norm"] / max(mg.last_stats["rhs_norm"], 1e-300)
    out["phi_vs_converged"] = _rel_l2(phi, phi_c)
    a_c = _forces(parts, phi_c, dx)
    out["force_vs_converged"] = _rel_l2(a, a_c)
    del a_c, phi_c

    # the FP64 FFT references (their kernels' transforms are kept in `solvers`,
    # when given, for the next call)
    cache = solvers if solvers is not None else {}
    for key, green, on in (("fft", "continuum", with_fft), ("lattice", "lattice", with_lattice)):
        if not on:
            continue
        fft = cache.get(green)
        if fft is None:
            fft = make_solver("fft", G, dx=dx, grav_constant=eng.grav, pad_factor=pad_factor, green=green)
            if solvers is not None:
                cache[green] = fft
        phi64 = fft.potential64(rho)
        out[f"phi_vs_{key}"] = _rel_l2(phi, phi64)
        phi_f = phi64.to(torch.float32)
        del phi64, fft
        if solvers is None:
            torch.cuda.empty_cache()
        a_f = _forces(parts, phi_f, dx)
        out[f"force_vs_{key}"] = _rel_l2(a, a_f)
        if key == "lattice" and with_isolated and pad_factor == 2:
            iso = make_solver("multigrid", G, dx=dx, grav_constant=eng.grav, tol=float(eng.mg.tol), n_cycles=80,
                              boundary="isolated")
            iso._lattice = cache.get("lattice")  # the kernel transform, when kept
            phi_i = torch.zeros_like(phi)
            iso.solve(rho, phi_i)
            out["isolated_cycles"] = [int(iso.last_stats["cycles_zero_faces"]), int(iso.last_cycles)]
            out["phi_isolated_vs_lattice"] = _rel_l2(phi_i, phi_f)
            out["force_isolated_vs_lattice"] = _rel_l2(_forces(parts, phi_i, dx), a_f)
            del iso, phi_i
        del phi_f, a_f
        out["fft_grid"] = pad_factor * G
    return out


__all__ = ["force_chain_errors"]
