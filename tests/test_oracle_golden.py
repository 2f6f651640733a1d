"""Pin the oracle's FFT, DST and diagnostics restatements to golden fixtures
generated by the reference's own code (tests/golden/make_golden.py), and the
reference-multigrid restatement to the exact discrete solution."""

from __future__ import annotations

import numpy as np
import pytest

from conftest import gaussian_rho, golden, rel_l2
from oracle import diagnostics as odiag
from oracle import dst, pm
from oracle.fft import FFTOracle


def test_fft_oracle_point_mass_golden():
    g = golden("fft_point_mass.npz")
    phi = FFTOracle(g["rho"].shape[0], dx=float(g["dx"]), grav_constant=float(g["grav"])).potential(g["rho"])
    np.testing.assert_allclose(phi.astype(np.float32), g["phi"], rtol=1e-6, atol=0)


def test_fft_oracle_point_mass_analytic():  # reference tests/test_solver_fft.py:16-40
    g = golden("fft_point_mass.npz")
    phi = g["phi"]
    n = phi.shape[0]
    c = n // 2
    mass = float(g["rho"][c, c, c])
    for r in (2, 4, 8):
        assert phi[c + r, c, c] == pytest.approx(-float(g["grav"]) * mass / r, rel=2e-3)
    assert phi[c + 6, c, c] == pytest.approx(phi[c, c + 6, c], rel=1e-4)


def test_fft_oracle_offcentre_golden_and_pe():
    g = golden("fft_offcenter_dx2.npz")
    phi = FFTOracle(g["rho"].shape[0], dx=float(g["dx"]), grav_constant=float(g["grav"])).potential(g["rho"])
    np.testing.assert_allclose(phi.astype(np.float32), g["phi"], rtol=1e-6)
    assert odiag.potential_energy_grid(g["rho"], g["phi"], float(g["dx"])) == pytest.approx(float(g["pe_grid"]),
                                                                                           rel=1e-12)


def test_fft_oracle_rejects_pad_factor_one():  # reference tests/test_solver_fft.py:43-44
    with pytest.raises(ValueError, match="pad_factor"):
        FFTOracle(16, pad_factor=1)


def test_host_diagnostics_golden():
    g = golden("plummer_diag.npz")
    m = g["mass"].astype(np.float64)
    pos, vel = g["pos"].astype(np.float64), g["vel"].astype(np.float64)
    assert odiag.kinetic_energy(m, vel) == pytest.approx(float(g["kinetic"]), rel=1e-14)
    np.testing.assert_allclose(odiag.linear_momentum(m, vel), g["momentum"], rtol=1e-12, atol=1e-3)
    np.testing.assert_allclose(odiag.angular_momentum(m, pos, vel), g["ang_momentum"], rtol=1e-12)
    np.testing.assert_allclose(odiag.center_of_mass(m, pos), g["center_of_mass"], rtol=1e-14)
    assert odiag.lagrangian_radius(m, pos, 0.5) == pytest.approx(float(g["half_mass_radius"]), rel=1e-14)
    assert odiag.potential_energy_direct(m[:2000], pos[:2000], 1.0, float(g["grav"])) == pytest.approx(
        float(g["pe_direct_soft1"]), rel=1e-12)


def test_dst_solver_satisfies_discrete_equation():
    rng = np.random.default_rng(5)
    n, dx = 20, 0.7
    rhs = rng.normal(size=(n, n, n))
    faces = rng.normal(size=(n, n, n))
    phi = dst.solve_dirichlet(rhs, faces, dx)
    lap = (phi[2:, 1:-1, 1:-1] + phi[:-2, 1:-1, 1:-1] + phi[1:-1, 2:, 1:-1] + phi[1:-1, :-2, 1:-1]
           + phi[1:-1, 1:-1, 2:] + phi[1:-1, 1:-1, :-2] - 6 * phi[1:-1, 1:-1, 1:-1]) / dx**2
    np.testing.assert_allclose(lap, rhs[1:-1, 1:-1, 1:-1], atol=1e-10)
    face = np.ones((n, n, n), bool)
    face[1:-1, 1:-1, 1:-1] = False
    np.testing.assert_array_equal(phi[face], faces[face])


def test_reference_multigrid_converges_to_dst_solution():
    """The restated reference multigrid, driven to its f32 floor, reaches the FP64 exact
    discrete solution (same faces up to f32 rounding of the multipole parameters)."""
    n, G_ = 32, 1.0
    rho = gaussian_rho(n, 1.0, 3.0, 100.0, center=(14.0, 16.5, 17.0))
    mg = pm.ReferenceMultigrid(n, grav_constant=G_, n_cycles=200, tol=0.0)
    phi = np.zeros((n, n, n), np.float32)
    mg.solve(rho, phi)
    exact = dst.solve_reference_problem(rho, 1.0, G_)
    assert rel_l2(phi, exact) < 1e-5


def test_reference_multigrid_matches_fft_oracle():  # test_solver_multigrid.py:212-247
    n = 48
    G_ = 4.4984945474465516e-12
    rho = gaussian_rho(n, 1.0, 4.0, 2.0e11)
    mg = pm.ReferenceMultigrid(n, grav_constant=G_, n_cycles=40)
    phi = np.zeros((n, n, n), np.float32)
    mg.solve(rho, phi)
    rhs_norm = 4 * np.pi * G_ * np.sqrt((rho.astype(np.float64) ** 2).sum())
    assert mg.residual_norm() / rhs_norm < 1e-3
    b = FFTOracle(n, grav_constant=G_).potential(rho)
    core = (slice(6, n - 6),) * 3
    peak = np.abs(b).max()
    assert np.abs(phi[core] - b[core]).max() / peak < 0.03
    assert np.abs(phi[core] - b[core]).mean() / peak < 0.005


def test_reference_multigrid_256_residual_golden():
    """test_solver_multigrid.py:73-95 quotes the reference's measured residual ratio on
    this source: ~0.29 at n_cycles=10 and ~2.1e-2 at n_cycles=20 ("identical on CPU
    and CUDA to three digits"). The restatement reproduces both."""
    G_ = 4.4984945474465516e-12
    n = 256
    rho = gaussian_rho(n, 1.0, 8.0, 2.32e11)
    rhs_norm = 4 * np.pi * G_ * np.sqrt((rho.astype(np.float64) ** 2).sum())
    ratios = {}
    for nc in (10, 20):
        mg = pm.ReferenceMultigrid(n, grav_constant=G_, n_cycles=nc)
        phi = np.zeros((n, n, n), np.float32)
        mg.solve(rho, phi)
        ratios[nc] = mg.residual_norm() / rhs_norm
    assert ratios[10] == pytest.approx(0.29, abs=0.005)
    assert ratios[20] == pytest.approx(2.1e-2, abs=0.05e-2)
