"""End-to-end: the fused engine holds a Plummer sphere in equilibrium.

The reference's exit gate (tests/test_sim.py:36-43, 87-114): over more than 5
dynamical times the half-mass radius stays within [0.8, 1.2] of its initial
value, the virial ratio T/|W| within [0.45, 0.55], the momentum drift below
1e-3 of M sqrt(GM/a), and the energy measured with the direct softened
pair-sum potential (softening one cell) drifts by less than 2%. Same
resolution ratio as the reference's test sphere (a = 5 cells).
"""

from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_plummer_equilibrium_gate(cuda, tmp_path):
    from galaxy_collision_gb300.config import SimConfig
    from galaxy_collision_gb300.io import read_snapshot
    from galaxy_collision_gb300.sim import run_simulation

    cfg = SimConfig(name="plummer-gate", ic_preset="plummer_131k", n_particles=4000, grid_size=64, box_lo=-6.4,
                    dx=0.2, grav_constant=1.0, dt=0.05, steps=120, solver_tol=1e-6, output_cadence=60,
                    output_dir=str(tmp_path), seed=7)
    res = run_simulation(cfg, history_cadence=8, direct_pe_softening=0.2)
    h = res["history"]
    n_tdyn = cfg.steps * cfg.dt / 1.0  # t_dyn = sqrt(a^3 / GM) = 1
    assert n_tdyn >= 5.0
    rh = np.array([x["half_mass_radius"] for x in h]) / h[0]["half_mass_radius"]
    virial = np.array([x["virial"] for x in h])
    p0 = h[0]["momentum"]
    pdrift = np.array([np.linalg.norm(x["momentum"] - p0) for x in h])  # M sqrt(GM/a) = 1
    ed0 = h[0]["energy_direct"]
    edrift = np.array([abs((x["energy_direct"] - ed0) / ed0) for x in h])
    assert 0.8 < rh.min() and rh.max() < 1.2, rh
    assert 0.45 < virial.min() and virial.max() < 0.55, virial
    assert pdrift.max() < 1e-3, pdrift
    assert edrift.max() < 0.02, edrift
    assert all(x["rel_residual"] < 1e-6 for x in h)
    # snapshots at steps 0, 60, 120 in the reference's layout
    assert len(res["snapshots"]) == 3
    snap = read_snapshot(res["snapshots"][-1])
    assert snap.step == 120 and snap.pos.shape == (4000, 3) and snap.phi.shape == (64, 64, 64)
    assert float(snap.diagnostics["energy"]) == pytest.approx(h[-1]["energy"])
