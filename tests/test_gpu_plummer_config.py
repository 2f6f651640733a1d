"""The Plummer configuration (131072 particles, 64^3 over [-12, 12]^3, dt 0.01).

* Trajectory parity: as the reference's cross-implementation test
  (tests/test_determinism.py:31-69: a 4000-particle Plummer sphere, 64^3, seed 3,
  tracers within 1e-3 after 15 steps), the engine's particles against the CPU
  oracle chain (FP64 deposit, exact FP64 solve of the same discrete problem,
  the reference's grad / gather / KDK in f32).
* Conservation over the full 200-step run of the configuration, tracked in FP64
  at the synchronised steps.
"""

from __future__ import annotations

import numpy as np
import pytest

from oracle import dst, pm

pytestmark = pytest.mark.gpu

BOX_LO, G, DX, DT = -12.0, 64, 0.375, 0.01


def test_tracers_match_oracle_chain(cuda):
    from galaxy_collision_gb300 import ic
    from galaxy_collision_gb300.engine import PMEngine

    icr = ic.plummer(4000, seed=3)
    steps = 15
    eng = PMEngine(G, DX, grav=1.0, origin=(BOX_LO,) * 3, tol=1e-9, max_cycles=80, sort_every=5)
    eng.set_warmstart("extrapolate")
    eng.load(icr.pos, icr.vel, icr.mass)
    eng.prime(DT)
    for _ in range(steps - 1):
        eng.advance(DT)
    eng.synchronize(DT)
    pe, ve, _, _ = eng.state_arrays(physical=True)
    pe = pe.cpu().numpy()

    x = [np.ascontiguousarray(c) for c in (icr.pos.astype(np.float64) - BOX_LO).astype(np.float32).T]
    v = [np.ascontiguousarray(c) for c in icr.vel.T]

    def force():
        p = np.stack(x, 1)
        rho = pm.deposit_f64(p, icr.mass, DX, G).astype(np.float32)
        phi = dst.solve_reference_problem(rho, DX, 1.0).astype(np.float32)
        return pm.gather(p, *pm.grad(phi, DX), DX)

    a = force()
    for _ in range(steps):
        pm.axpy3(*v, *a, np.float32(0.5 * DT))
        pm.axpy3(*x, *v, np.float32(DT))
        a = force()
        pm.axpy3(*v, *a, np.float32(0.5 * DT))
    po = np.stack(x, 1).astype(np.float64) + BOX_LO
    assert np.abs(pe - po).max() < 1e-3


def test_plummer_configuration_conserves(cuda, tmp_path):
    from galaxy_collision_gb300.config import SimConfig
    from galaxy_collision_gb300.sim import run_simulation

    cfg = SimConfig(name="plummer-131k", ic_preset="plummer_131k", n_particles=131072, grid_size=G, box_lo=BOX_LO,
                    dx=DX, grav_constant=1.0, dt=DT, steps=200, solver_tol=1e-6, output_cadence=0,
                    output_dir=str(tmp_path), seed=0)
    res = run_simulation(cfg, history_cadence=20, write_snapshots=False)
    h = res["history"]
    assert len(h) == 11
    e0 = h[0]["energy"]
    drift = max(abs((x["energy"] - e0) / e0) for x in h)
    p = max(np.linalg.norm(x["momentum"] - h[0]["momentum"]) for x in h)
    rh = np.array([x["half_mass_radius"] for x in h]) / h[0]["half_mass_radius"]
    virial = np.array([x["virial"] for x in h])
    assert drift < 0.02, drift
    assert p < 1e-3, p  # M sqrt(GM/a) = 1
    assert 0.85 < rh.min() and rh.max() < 1.15, rh
    assert 0.4 < virial.min() and virial.max() < 0.6, virial
    assert all(x["rel_residual"] < 1e-6 for x in h)
