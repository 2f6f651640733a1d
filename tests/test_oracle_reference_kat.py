"""Pin the CPU oracle to the reference's own known-answer tests.

Each test restates one assertion of the reference test suite (file:line cited)
against ``oracle/pm_oracle.c``. Passing them is what makes the oracle a faithful
stand-in for the Taichi kernels, which cannot run here.
"""

from __future__ import annotations

import numpy as np
import pytest

from conftest import gaussian_rho, rel_l2
from oracle import pm

G_REF = 4.4984945474465516e-12  # units.G of the reference (units.py:44)


def _pos(*rows):
    return np.asarray(rows, dtype=np.float32)


# ---- deposit: tests/test_deposit.py ------------------------------------------
def test_mass_conservation():  # test_deposit.py:34-52
    rng = np.random.default_rng(0)
    n, G = 5000, 64
    pos = rng.uniform(2.0, G - 2.0, size=(n, 3)).astype(np.float32)
    mass = rng.uniform(0.5, 2.0, size=n).astype(np.float32)
    rho = pm.deposit_f32(pos, mass, 1.0, G)
    assert rho.sum() == pytest.approx(mass.sum(), rel=1e-4)


def test_mass_conservation_dx_not_one():  # test_deposit.py:55-73
    rng = np.random.default_rng(3)
    n, G, dx = 4000, 32, 2.5
    pos = rng.uniform(2.0 * dx, (G - 3) * dx, size=(n, 3)).astype(np.float32)
    mass = rng.uniform(0.5, 2.0, size=n).astype(np.float32)
    rho = pm.deposit_f32(pos, mass, dx, G)
    assert rho.sum() * dx**3 == pytest.approx(mass.sum(), rel=1e-4)


def test_on_node_normalisation_dx_not_one():  # test_deposit.py:76-92
    dx = 2.5
    rho = pm.deposit_f32(_pos([2 * dx, 3 * dx, 4 * dx]), np.array([5.0], np.float32), dx, 8)
    assert rho[2, 3, 4] == pytest.approx(5.0 / dx**3)
    assert rho.sum() == pytest.approx(5.0 / dx**3)


def test_single_particle_on_node():  # test_deposit.py:95-109
    rho = pm.deposit_f32(_pos([8.0, 8.0, 8.0]), np.array([3.0], np.float32), 1.0, 16)
    assert rho[8, 8, 8] == pytest.approx(3.0)
    assert rho.sum() == pytest.approx(3.0)


def test_midpoint_splits_eight_ways():  # test_deposit.py:112-129
    rho = pm.deposit_f32(_pos([8.5, 8.5, 8.5]), np.array([8.0], np.float32), 1.0, 16)
    assert np.allclose(rho[8:10, 8:10, 8:10], 1.0)
    assert rho.sum() == pytest.approx(8.0)


def test_open_boundary_no_wrap():  # test_deposit.py:132-162
    pos = _pos([-3.0, 8.0, 8.0], [40.0, 8.0, 8.0], [15.5, 8.0, 8.0])
    rho = pm.deposit_f32(pos, np.ones(3, np.float32), 1.0, 16)
    assert rho.sum() <= 3.0 + 1e-5
    assert rho[15, 8, 8] == pytest.approx(0.5)
    assert rho[0, :, :].sum() == pytest.approx(0.0)


def test_gather_constant_field():  # test_deposit.py:165-190
    rng = np.random.default_rng(1)
    n, G = 1000, 32
    pos = rng.uniform(1.0, G - 2.0, size=(n, 3)).astype(np.float32)
    shape = (G, G, G)
    ax, ay, az = pm.gather(pos, np.full(shape, 2.0, np.float32), np.full(shape, -3.0, np.float32),
                           np.full(shape, 0.5, np.float32), 1.0)
    assert np.allclose(ax, 2.0, atol=1e-5) and np.allclose(ay, -3.0, atol=1e-5) and np.allclose(az, 0.5, atol=1e-5)


def test_gather_linear_field_exact():  # test_deposit.py:193-222
    rng = np.random.default_rng(2)
    n, G = 500, 32
    pos = rng.uniform(1.0, G - 2.0, size=(n, 3)).astype(np.float32)
    ii, jj, kk = np.meshgrid(np.arange(G), np.arange(G), np.arange(G), indexing="ij")
    field = (0.3 * ii + 0.1 * jj - 0.2 * kk).astype(np.float32)
    z = np.zeros_like(field)
    ax, _, _ = pm.gather(pos, field, z, z, 1.0)
    expected = 0.3 * pos[:, 0] + 0.1 * pos[:, 1] - 0.2 * pos[:, 2]
    assert np.allclose(ax, expected, atol=1e-3)


# ---- grad / integrator: tests/test_integrator.py -----------------------------
def test_kick_drift_uniform_acceleration():  # test_integrator.py:23-47
    n, dt = 4, 0.2
    p = [np.zeros(n, np.float32) for _ in range(3)]
    v = [np.zeros(n, np.float32) for _ in range(3)]
    a = [np.full(n, 0.5, np.float32), np.zeros(n, np.float32), np.zeros(n, np.float32)]
    pm.axpy3(*v, *a, dt / 2)
    pm.axpy3(*p, *v, dt)
    pm.axpy3(*v, *a, dt / 2)
    assert v[0][0] == pytest.approx(0.5 * dt, rel=1e-5)
    assert p[0][0] == pytest.approx(0.5 * 0.5 * dt**2, rel=1e-5)


@pytest.mark.parametrize("dx", [1.0, 2.0])
def test_grad_linear_potential(dx):  # test_integrator.py:50-69, 287-306
    n = 16
    ii, jj, kk = np.meshgrid(np.arange(n), np.arange(n), np.arange(n), indexing="ij")
    phi = (2.0 * ii * dx + 3.0 * jj * dx - 1.0 * kk * dx).astype(np.float32)
    ax, ay, az = pm.grad(phi, dx)
    core = (slice(1, n - 1),) * 3
    assert np.allclose(ax[core], -2.0, atol=1e-4)
    assert np.allclose(ay[core], -3.0, atol=1e-4)
    assert np.allclose(az[core], 1.0, atol=1e-4)


def test_force_near_boundary_not_dropped():  # test_integrator.py:309-341
    n = 16
    ii = np.meshgrid(np.arange(n), np.arange(n), np.arange(n), indexing="ij")[0]
    ax, ay, az = pm.grad((2.0 * ii).astype(np.float32), 1.0)
    acc = pm.gather(_pos([14.5, 8.0, 8.0]), ax, ay, az, 1.0)
    assert acc[0][0] == pytest.approx(-2.0, abs=1e-4)


# ---- multigrid: tests/test_solver_multigrid.py --------------------------------
def test_reference_level_sizes():  # multigrid.py:330-336, 3.2 of the reference call stack
    assert pm.ReferenceMultigrid(256).sizes == [256, 128, 64, 32, 16, 8, 4]
    assert pm.ReferenceMultigrid(64).sizes == [64, 32, 16, 8, 4]
    assert pm.ReferenceMultigrid(48).sizes == [48, 24, 12, 6, 3]


def test_vcycle_reduces_residual():  # test_solver_multigrid.py:50-70
    n = 32
    rho = gaussian_rho(n, 1.0, 3.0, 1.0e10)
    mg = pm.ReferenceMultigrid(n, grav_constant=G_REF, n_cycles=1)
    phi = np.zeros((n, n, n), np.float32)
    mg.solve(rho, phi)
    r1 = mg.residual_norm()
    for _ in range(6):
        mg.vcycle()
    assert mg.residual_norm() < 0.1 * r1


def test_adaptive_warm_start():  # test_solver_multigrid.py:98-132
    n = 64
    rho = gaussian_rho(n, 1.0, 4.0, 1.0e10)
    a = pm.ReferenceMultigrid(n, grav_constant=G_REF, n_cycles=30, tol=1e-3)
    f = pm.ReferenceMultigrid(n, grav_constant=G_REF, n_cycles=30, tol=0.0)
    pa = np.zeros((n, n, n), np.float32)
    pf = np.zeros((n, n, n), np.float32)
    a.solve(rho, pa)
    f.solve(rho, pf)
    a.solve(rho, pa, warm_start=True)
    f.solve(rho, pf, warm_start=True)
    assert a.last_cycles <= 3
    assert f.last_cycles == 30
    assert rel_l2(pa, pf) < 1e-2


def test_point_mass_far_field():  # test_solver_multigrid.py:135-174
    n, mass = 96, 1.0e10
    c = n // 2
    rho = np.zeros((n, n, n), np.float32)
    rho[c, c, c] = mass
    mg = pm.ReferenceMultigrid(n, grav_constant=G_REF, n_cycles=80, tol=0.0)
    phi = np.zeros_like(rho)
    mg.solve(rho, phi)
    rhs_norm = 4.0 * np.pi * G_REF * float(np.sqrt((rho.astype(np.float64) ** 2).sum()))
    assert mg.residual_norm() / rhs_norm < 1e-4
    prev = np.inf
    for r in (4, 6, 8, 12, 16, 20):
        analytic = -G_REF * mass / r
        vals = [phi[c + r, c, c], phi[c - r, c, c], phi[c, c + r, c], phi[c, c - r, c], phi[c, c, c + r],
                phi[c, c, c - r]]
        rel = abs(float(np.mean(vals)) - analytic) / abs(analytic)
        assert rel < 0.4 / r**2
        assert rel < prev * (1.0 + 1e-4) + 1e-7
        prev = rel


def test_moments_match_numpy():  # test_solver_multigrid.py:285-314
    n = 64
    ax = np.arange(n, dtype=np.float64)
    xx, yy, zz = np.meshgrid(ax, ax, ax, indexing="ij")
    blob = np.exp(-((xx - 20) ** 2 + (yy - 34) ** 2 + (zz - 28) ** 2) / (2 * 6.0**2))
    blob += 0.5 * np.exp(-((xx - 44) ** 2 + (yy - 30) ** 2 + (zz - 36) ** 2) / (2 * 4.0**2))
    rho = (blob / blob.sum() * 3.2e11).astype(np.float32)
    s = pm.moments(rho, 1.0)
    m = rho.astype(np.float64)
    assert s[0] == pytest.approx(m.sum(), rel=1e-12)
    np.testing.assert_allclose(s[1:4], [(m * xx).sum(), (m * yy).sum(), (m * zz).sum()], rtol=1e-12)
    np.testing.assert_allclose(s[7], (m * xx * yy).sum(), rtol=1e-12)
