"""The lattice Green's function oracle, pinned by its defining properties.

No reference test covers it (the reference validates against the continuum
kernel only, src/galaxy_collision/solver/fft_oracle.py:82-96), so it is pinned
by what defines it: g(0) is Watson's constant for the simple cubic lattice, the
7-point Laplacian of g is minus the unit impulse, g -> 1/(4 pi r) far away, and
the potential it gives solves the discrete Poisson problem the multigrid
solves (checked against the exact FP64 DST-I solver with the same faces). The
package's own table (solver/lattice_green.py) must equal it.
"""

from __future__ import annotations

import numpy as np
import pytest

from conftest import gaussian_rho
from oracle import dst
from oracle import lattice_green as olg


@pytest.fixture(scope="module")
def table():
    return olg.lgf_table(40)


def _g(t, a, b, c):
    return t[abs(a), abs(b), abs(c)]


def _lap(t, a, b, c):
    return (_g(t, a + 1, b, c) + _g(t, a - 1, b, c) + _g(t, a, b + 1, c) + _g(t, a, b - 1, c) + _g(t, a, b, c + 1)
            + _g(t, a, b, c - 1) - 6.0 * _g(t, a, b, c))


def test_watson_constant(table):
    assert table[0, 0, 0] == pytest.approx(olg.WATSON_G0, abs=1e-13)


def test_laplacian_is_minus_delta(table):
    assert _lap(table, 0, 0, 0) == pytest.approx(-1.0, abs=1e-12)
    rng = np.random.default_rng(0)
    for _ in range(300):
        a, b, c = rng.integers(0, 38, size=3)
        if a == b == c == 0:
            continue
        assert abs(_lap(table, int(a), int(b), int(c))) < 1e-12


def test_symmetry_and_far_field(table):
    np.testing.assert_allclose(table, table.transpose(1, 0, 2), rtol=0, atol=1e-16)
    np.testing.assert_allclose(table, table.transpose(0, 2, 1), rtol=0, atol=1e-16)
    for n in [(12, 0, 0), (9, 9, 0), (20, 11, 5), (39, 39, 39)]:
        r = float(np.sqrt(np.sum(np.square(n))))
        assert abs(4.0 * np.pi * r * table[n] - 1.0) < 1.0 / r**2


def test_potential_solves_the_discrete_problem():
    """The free-space potential satisfies L phi / dx^2 = 4 pi G rho at every
    interior node, and the DST Dirichlet solve with its own face values gives
    it back: the two FP64 oracles agree on the discrete problem."""
    n, dx, grav = 32, 0.5, 1.3
    rho = gaussian_rho(n, dx, 2.0 * dx, 5.0, center=(7.0, 8.5, 9.0))
    phi = olg.lgf_potential(rho, dx, grav)
    lap = (phi[2:, 1:-1, 1:-1] + phi[:-2, 1:-1, 1:-1] + phi[1:-1, 2:, 1:-1] + phi[1:-1, :-2, 1:-1]
           + phi[1:-1, 1:-1, 2:] + phi[1:-1, 1:-1, :-2] - 6.0 * phi[1:-1, 1:-1, 1:-1]) / dx**2
    rhs = 4.0 * np.pi * grav * rho.astype(np.float64)[1:-1, 1:-1, 1:-1]
    assert np.abs(lap - rhs).max() < 1e-10 * np.abs(rhs).max()
    again = dst.solve_dirichlet(4.0 * np.pi * grav * rho.astype(np.float64), phi, dx)
    assert np.abs(again - phi).max() < 1e-11 * np.abs(phi).max()


def test_point_mass_far_field():
    n, dx, grav, M = 32, 1.0, 1.0, 2.0
    rho = np.zeros((n, n, n))
    rho[3, 4, 5] = M / dx**3
    phi = olg.lgf_potential(rho, dx, grav)
    for p in [(30, 4, 5), (25, 28, 20), (31, 31, 31)]:
        r = dx * float(np.linalg.norm(np.subtract(p, (3, 4, 5))))
        assert phi[p] == pytest.approx(-grav * M / r, rel=1.0 / (r / dx) ** 2)


def test_package_table_equals_oracle(table):
    from galaxy_collision_gb300.solver.lattice_green import lattice_green_table

    np.testing.assert_allclose(lattice_green_table(40), table, rtol=0, atol=1e-15)
