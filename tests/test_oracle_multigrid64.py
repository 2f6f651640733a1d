"""The reference multigrid restated in FP64 (the CPU baseline driven to 1e-6).

Same algorithm as the reference (solver/multigrid.py:298-494) with double
arrays: it must reach tolerances below the FP32 floor and converge to the exact
discrete solution (FP64 DST-I with the same multipole faces), at the
reference's convergence rate (0.6-0.7 per V-cycle, docs and AGENT notes of the
reference; its 256^3 test quotes 2.1e-2 after 20 cycles).
"""

from __future__ import annotations

import numpy as np

from conftest import gaussian_rho, rel_l2
from oracle import dst, pm


def test_fp64_reference_multigrid_reaches_1e_9_and_the_exact_solution():
    n, dx = 32, 0.5
    rho = gaussian_rho(n, dx, 1.5, 2.0, center=(7.0, 8.0, 8.5))
    mg = pm.ReferenceMultigrid64(n, dx=dx, grav_constant=1.0, tol=1e-9, n_cycles=200)
    phi = np.zeros((n, n, n))
    mg.solve(rho, phi)
    assert mg.norms[1] < 1e-9 * mg.norms[0]
    assert 20 < mg.last_cycles < 120  # the reference hierarchy's slow contraction
    assert rel_l2(phi, dst.solve_reference_problem(rho, dx, 1.0)) < 1e-7
    # a warm start from the answer stops after one cycle
    mg.solve(rho, phi, warm_start=True)
    assert mg.last_cycles == 1
