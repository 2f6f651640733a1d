"""The fused engine against the reference-shaped chain and the CPU oracle.

The engine's step is the reference's kdk_step around accel_fn (deposit -> solve
-> grad -> gather, sim.py:320-325) with the force gathered from phi on the fly.
With the solver driven to the same residual the trajectories must agree with
the step-by-step chain, the oracle chain, and themselves run to run.
"""

from __future__ import annotations

import numpy as np
import pytest

from conftest import golden
from oracle import diagnostics as odiag
from oracle import dst, pm

pytestmark = pytest.mark.gpu


def _cluster(n, G, seed, spread=2.5, vscale=0.15):
    rng = np.random.default_rng(seed)
    pos = (rng.normal(size=(n, 3)) * spread + (G - 1) / 2.0).astype(np.float32)
    vel = (rng.normal(size=(n, 3)) * vscale).astype(np.float32)
    mass = rng.uniform(0.5, 1.5, size=n).astype(np.float32) / n
    return pos, vel, mass


def _engine_run(pos, vel, mass, G, dt, steps, sort_every=5, tol=1e-7, grad_grid=True):
    from galaxy_collision_gb300.engine import PMEngine

    eng = PMEngine(G, 1.0, grav=1.0, tol=tol, max_cycles=60, sort_every=sort_every, grad_grid=grad_grid)
    eng.load(pos, vel, mass, sort=sort_every > 0)
    eng.prime(dt)
    for _ in range(steps - 1):
        eng.advance(dt)
    eng.synchronize(dt)
    p, v, m, _ = eng.state_arrays()
    return p.cpu().numpy(), v.cpu().numpy(), eng


def test_engine_matches_stepwise_gpu_chain(cuda):
    from galaxy_collision_gb300.data import Field, GridState, ParticleState
    from galaxy_collision_gb300.deposit import deposit_density, gather_acceleration, potential_to_accel
    from galaxy_collision_gb300.integrator import kdk_step
    from galaxy_collision_gb300.solver import make_solver

    G, n, dt, steps = 32, 20000, 0.05, 6
    pos, vel, mass = _cluster(n, G, 1)
    pe, ve, _ = _engine_run(pos, vel, mass, G, dt, steps)

    parts = ParticleState(n)
    for f, a in zip((parts.pos_x, parts.pos_y, parts.pos_z), pos.T):
        f.from_numpy(np.ascontiguousarray(a))
    for f, a in zip((parts.vel_x, parts.vel_y, parts.vel_z), vel.T):
        f.from_numpy(np.ascontiguousarray(a))
    parts.mass.from_numpy(mass)
    grid = GridState(G)
    acc = [Field(n) for _ in range(3)]
    solver = make_solver("multigrid", G, grav_constant=1.0, tol=1e-7, n_cycles=60)

    def accel_fn():
        deposit_density(parts, grid.rho, 1.0)
        solver.solve(grid.rho, grid.phi, warm_start=False)
        potential_to_accel(grid.phi, grid.ax, grid.ay, grid.az, 1.0)
        gather_acceleration(parts, grid.ax, grid.ay, grid.az, *acc, 1.0)

    accel_fn()
    for _ in range(steps):
        kdk_step(parts, *acc, accel_fn, dt)
    pc = np.stack([f.to_numpy() for f in (parts.pos_x, parts.pos_y, parts.pos_z)], 1)
    vc = np.stack([f.to_numpy() for f in (parts.vel_x, parts.vel_y, parts.vel_z)], 1)
    assert np.abs(pe - pc).max() < 2e-5
    assert np.abs(ve - vc).max() < 2e-4 * np.abs(vc).max()


def test_engine_matches_oracle_chain(cuda):
    """Oracle chain: FP64 deposit, exact FP64 discrete solve, reference grad/gather/KDK."""
    G, n, dt, steps = 24, 4000, 0.05, 3
    pos, vel, mass = _cluster(n, G, 2, spread=2.0)
    pe, ve, _ = _engine_run(pos, vel, mass, G, dt, steps, sort_every=0, tol=1e-8)

    x = [np.ascontiguousarray(c) for c in pos.T]
    v = [np.ascontiguousarray(c) for c in vel.T]

    def force():
        rho = pm.deposit_f64(np.stack(x, 1), mass, 1.0, G).astype(np.float32)
        phi = dst.solve_reference_problem(rho, 1.0, 1.0).astype(np.float32)
        return pm.gather(np.stack(x, 1), *pm.grad(phi, 1.0), 1.0)

    a = force()
    for _ in range(steps):
        pm.axpy3(*v, *a, np.float32(0.5 * dt))
        pm.axpy3(*x, *v, np.float32(dt))
        a = force()
        pm.axpy3(*v, *a, np.float32(0.5 * dt))
    po, vo = np.stack(x, 1), np.stack(v, 1)
    assert np.abs(pe - po).max() < 1e-5
    assert np.abs(ve - vo).max() < 1e-4 * np.abs(vo).max()


def test_engine_bitwise_reproducible_and_sort_invariant(cuda):
    G, n, dt, steps = 32, 50000, 0.05, 8
    pos, vel, mass = _cluster(n, G, 3)
    p1, v1, _ = _engine_run(pos, vel, mass, G, dt, steps, sort_every=3)
    p2, v2, _ = _engine_run(pos, vel, mass, G, dt, steps, sort_every=3)
    p3, v3, _ = _engine_run(pos, vel, mass, G, dt, steps, sort_every=0)
    np.testing.assert_array_equal(p1, p2)
    np.testing.assert_array_equal(v1, v2)
    # the fixed-point deposit is order-independent and every particle's update is
    # independent, so sorting changes nothing but memory order
    np.testing.assert_array_equal(p1, p3)
    np.testing.assert_array_equal(v1, v3)


def test_engine_gradient_grid_gather_is_bitwise_identical(cuda):
    """Gathering from a precomputed float4 -grad(phi) grid is the same arithmetic
    as forming the gradient at the corners on the fly."""
    G, n, dt, steps = 40, 30000, 0.05, 5
    pos, vel, mass = _cluster(n, G, 5)
    pos[:50] = np.random.default_rng(9).uniform(-0.9, G - 0.1, size=(50, 3))  # include edge cells
    p1, v1, _ = _engine_run(pos, vel, mass, G, dt, steps, sort_every=2, grad_grid=False)
    p2, v2, _ = _engine_run(pos, vel, mass, G, dt, steps, sort_every=2, grad_grid=True)
    np.testing.assert_array_equal(p1, p2)
    np.testing.assert_array_equal(v1, v2)


def test_engine_diagnostics_match_host(cuda):
    from galaxy_collision_gb300.engine import PMEngine

    g = golden("plummer_diag.npz")
    pos, vel, mass = g["pos"], g["vel"], g["mass"]
    G = int(g["grid_size"])
    eng = PMEngine(G, 1.0, grav=float(g["grav"]), tol=1e-6, sort_every=0)
    eng.load(pos, vel, mass, sort=True)
    r = eng.prime(0.0, diagnostics=True)
    d = eng.diagnostics_physical(r.diag)
    m = mass.astype(np.float64)
    p64, v64 = pos.astype(np.float64), vel.astype(np.float64)
    assert d["M"] == pytest.approx(m.sum(), rel=1e-12)
    assert d["kinetic"] == pytest.approx(float(g["kinetic"]), rel=1e-9)
    np.testing.assert_allclose(d["momentum"], odiag.linear_momentum(m, v64), rtol=1e-6,
                               atol=1e-9 * float((m[:, None] * np.abs(v64)).sum()))
    np.testing.assert_allclose(d["ang_momentum"], g["ang_momentum"], rtol=1e-6)
    np.testing.assert_allclose(d["center_of_mass"], g["center_of_mass"], rtol=1e-9)


def test_device_diagnostics_match_reference_golden(cuda):  # tests/test_diagnostics.py:107-171
    from galaxy_collision_gb300.data import GridState, ParticleState
    from galaxy_collision_gb300.deposit import deposit_density
    from galaxy_collision_gb300.diagnostics_device import DeviceDiagnostics
    from galaxy_collision_gb300.solver import make_solver

    g = golden("plummer_diag.npz")
    pos, vel, mass = g["pos"], g["vel"], g["mass"]
    gs = int(g["grid_size"])
    n = pos.shape[0]
    parts = ParticleState(n)
    for f, a in zip((parts.pos_x, parts.pos_y, parts.pos_z, parts.vel_x, parts.vel_y, parts.vel_z),
                    list(pos.T) + list(vel.T)):
        f.from_numpy(np.ascontiguousarray(a))
    parts.mass.from_numpy(mass)
    grid = GridState(gs)
    deposit_density(parts, grid.rho, 1.0)
    make_solver("fft", gs, grav_constant=float(g["grav"])).solve(grid.rho, grid.phi)
    dev = DeviceDiagnostics(gs).sample(parts, grid, 1.0)
    m = mass.astype(np.float64)
    assert dev["kinetic"] == pytest.approx(float(g["kinetic"]), rel=1e-9)
    assert dev["potential"] == pytest.approx(
        odiag.potential_energy_grid(grid.rho.to_numpy(), grid.phi.to_numpy(), 1.0), rel=1e-9)
    np.testing.assert_allclose(dev["momentum"], g["momentum"], rtol=1e-6,
                               atol=1e-9 * float((m[:, None] * np.abs(vel)).sum()))
    np.testing.assert_allclose(dev["ang_momentum"], g["ang_momentum"], rtol=1e-6)
    assert dev["half_mass_radius"] == pytest.approx(float(g["half_mass_radius"]), rel=5e-3)


def test_engine_state_machine_errors(cuda):
    from galaxy_collision_gb300.engine import PMEngine

    G = 16
    pos, vel, mass = _cluster(100, G, 4, spread=1.0)
    eng = PMEngine(G, 1.0)
    with pytest.raises(RuntimeError):
        eng.advance(0.1)
    eng.load(pos, vel, mass)
    with pytest.raises(RuntimeError):
        eng.synchronize(0.1)
    eng.prime(0.1)
    with pytest.raises(RuntimeError):
        eng.prime(0.1)
