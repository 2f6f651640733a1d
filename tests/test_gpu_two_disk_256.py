"""Parity on the graded grid: a two-disk collision at 256^3 against the CPU oracle.

The input is the two-disk 10M configuration's sampler (masses 1 and 1.5,
exponential sech^2 disks, the second inclined 30 degrees, box [-32, 32]^3 at
256^3) scaled to 1M particles. Every stage of the chain is compared with the
oracle on the same input:

* cell keys and the stable sort permutation: bit-exact (oracle/pm_oracle.c
  or_cell_keys; the reference's cell index, deposit.py:62-67);
* the fixed-point density: bit-exact against or_deposit_fixed;
* the potential, solved to a 1e-10 relative residual: relative L2 <= 1e-6
  against the exact FP64 DST-I solution of the same discrete problem (7-point
  Laplacian, FP64 multipole faces, solver/multigrid.py:261-295, 455-487);
* the particle forces -grad(phi) gathered by CIC: relative L2 <= 1e-5 against
  the oracle's grad + gather of the DST potential (deposit.py:85-174);
* a 15-step KDK trajectory of the fused engine against the oracle chain
  (FP64 deposit, exact solve, the reference's grad / gather / kicks in f32):
  every particle within 1e-3 box units, the gate of the reference's
  cross-implementation test (tests/test_determinism.py:31-69) applied at the
  reference's 256^3 test size (tests/test_solver_multigrid.py:178-209).
"""

from __future__ import annotations

from types import SimpleNamespace

import numpy as np
import pytest
import torch

from oracle import dst, pm

pytestmark = pytest.mark.gpu

SCALE = 0.1  # 400k + 600k particles


@pytest.fixture(scope="module")
def two_disk(cuda):
    from galaxy_collision_gb300 import ic

    icr, cfg = ic.build("two_disk_10M", scale=SCALE)
    pos_grid = (icr.pos.astype(np.float64) - np.asarray(cfg["origin"])).astype(np.float32)
    return icr, cfg, pos_grid


def _parts(pos_grid, mass):
    cols = [torch.from_numpy(np.ascontiguousarray(pos_grid[:, i])).cuda() for i in range(3)]
    return SimpleNamespace(n=pos_grid.shape[0], pos_x=cols[0], pos_y=cols[1], pos_z=cols[2],
                           mass=torch.from_numpy(np.ascontiguousarray(mass)).cuda())


def test_keys_sort_density_potential_forces_at_256(two_disk):
    from galaxy_collision_gb300.deposit import (cell_keys, deposit_density, gather_acceleration,
                                                potential_to_accel, sort_keys)
    from galaxy_collision_gb300.solver import make_solver

    icr, cfg, pos = two_disk
    G, dx = cfg["grid"], cfg["dx"]
    assert G == 256 and pos.shape[0] == 1_000_000
    parts = _parts(pos, icr.mass)

    keys_gpu = cell_keys(parts, G, dx)
    keys_ref = pm.cell_keys(pos, dx, G)
    np.testing.assert_array_equal(keys_gpu.cpu().numpy().view(np.uint32), keys_ref)
    skeys, perm = sort_keys(keys_gpu, G, dx)
    perm_ref = pm.stable_sort_perm(keys_ref)
    np.testing.assert_array_equal(perm.cpu().numpy().view(np.uint32), perm_ref)
    np.testing.assert_array_equal(skeys.cpu().numpy().view(np.uint32), keys_ref[perm_ref])

    bits = 52
    rho = torch.empty((G, G, G), dtype=torch.float32, device="cuda")
    deposit_density(parts, rho, dx, fixed_point_bits=bits)
    rho_ref, _, _ = pm.deposit_fixed(pos, icr.mass, dx, G, bits)
    rho_np = rho.cpu().numpy()
    np.testing.assert_array_equal(rho_np, rho_ref)

    solver = make_solver("multigrid", G, dx=dx, grav_constant=1.0, tol=1e-10, n_cycles=80)
    phi = torch.zeros_like(rho)
    solver.solve(rho, phi)
    assert solver.last_stats["converged"] == 1
    phi_ref = dst.solve_reference_problem(rho_np, dx, 1.0)
    phi_np = phi.cpu().numpy().astype(np.float64)
    err_phi = np.linalg.norm(phi_np - phi_ref) / np.linalg.norm(phi_ref)
    assert err_phi <= 1e-6, err_phi

    grids = [torch.empty_like(phi) for _ in range(3)]
    potential_to_accel(phi, *grids, dx)
    acc = [torch.empty(parts.n, dtype=torch.float32, device="cuda") for _ in range(3)]
    gather_acceleration(parts, *grids, *acc, dx)
    a_gpu = np.stack([a.cpu().numpy() for a in acc]).astype(np.float64)
    a_ref = np.stack(pm.gather(pos, *pm.grad(phi_ref.astype(np.float32), dx), dx)).astype(np.float64)
    err_f = np.linalg.norm(a_gpu - a_ref) / np.linalg.norm(a_ref)
    assert err_f <= 1e-5, err_f


def test_two_disk_trajectory_matches_oracle_chain_at_256(two_disk):
    from galaxy_collision_gb300.engine import PMEngine

    icr, cfg, pos = two_disk
    G, dx, dt = cfg["grid"], cfg["dx"], cfg["dt"]
    origin = np.asarray(cfg["origin"])
    steps = 15
    eng = PMEngine(G, dx, grav=1.0, origin=tuple(origin), tol=1e-9, max_cycles=80, sort_every=5)
    eng.set_warmstart("extrapolate")
    eng.load(icr.pos, icr.vel, icr.mass, icr.gid)
    eng.prime(dt)
    for _ in range(steps - 1):
        eng.advance(dt)
    eng.synchronize(dt)
    pe, _, _, _ = eng.state_arrays(physical=True)
    pe = pe.cpu().numpy()

    x = [np.ascontiguousarray(c) for c in pos.T]
    v = [np.ascontiguousarray(c) for c in icr.vel.T]

    def force():
        p = np.stack(x, 1)
        rho = pm.deposit_f64(p, icr.mass, dx, G).astype(np.float32)
        phi = dst.solve_reference_problem(rho, dx, 1.0).astype(np.float32)
        return pm.gather(p, *pm.grad(phi, dx), dx)

    a = force()
    for _ in range(steps):
        pm.axpy3(*v, *a, np.float32(0.5 * dt))
        pm.axpy3(*x, *v, np.float32(dt))
        a = force()
        pm.axpy3(*v, *a, np.float32(0.5 * dt))
    po = np.stack(x, 1).astype(np.float64) + origin
    err = np.abs(pe - po).max()
    assert err < 1e-3, err
