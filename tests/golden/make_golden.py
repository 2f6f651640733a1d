"""Generate the golden fixtures of tests/golden/ from the reference implementation.

Run in a container where the reference checkout is available:

    python tests/golden/make_golden.py /path/to/Galaxy-Collision-with-CUDA-FFT

It imports the reference's pure-NumPy modules (src/galaxy_collision/units.py,
solver/fft_oracle.py, diagnostics.py, ic.py) -- the Taichi kernels cannot run
without Taichi -- with a stub for ``yaml`` (only imported by config.py for
load/dump, unused here), and writes small .npz fixtures. The tests only read
the fixtures; nothing at test time touches the reference checkout.
"""

from __future__ import annotations

import sys
import types
from pathlib import Path

import numpy as np

OUT = Path(__file__).resolve().parent


class _Field:
    """Duck-typed Taichi field (to_numpy/from_numpy), what FFTPoissonSolver.solve uses."""

    def __init__(self, arr):
        self.a = np.array(arr, dtype=np.float32)

    @property
    def shape(self):
        return self.a.shape

    def to_numpy(self):
        return self.a.copy()

    def from_numpy(self, arr):
        self.a[...] = arr


def main(ref_root: str) -> None:
    sys.modules.setdefault("yaml", types.ModuleType("yaml"))
    sys.path.insert(0, str(Path(ref_root) / "src"))
    from galaxy_collision import diagnostics, units
    from galaxy_collision.config import SimConfig
    from galaxy_collision.ic import PlummerModel, build_plummer_ic
    from galaxy_collision.solver.fft_oracle import FFTPoissonSolver

    # 1. point mass on one node (tests/test_solver_fft.py:16-40 setup, smaller grid)
    n, dx, mass = 24, 1.0, 1.0e10
    c = n // 2
    rho = np.zeros((n, n, n), np.float32)
    rho[c, c, c] = mass / dx**3
    phi = _Field(np.zeros_like(rho))
    FFTPoissonSolver(n, dx=dx, grav_constant=units.G, use_gpu=False).solve(_Field(rho), phi)
    np.savez_compressed(OUT / "fft_point_mass.npz", rho=rho, phi=phi.a, dx=dx, grav=units.G)

    # 2. off-centre Gaussian, dx != 1 (test_solver_multigrid.py:250-282 style)
    n, dx = 32, 2.0
    ax = np.arange(n) * dx
    xx, yy, zz = np.meshgrid(ax, ax, ax, indexing="ij")
    g = np.exp(-((xx - 40.0) ** 2 + (yy - 28.0) ** 2 + (zz - 34.0) ** 2) / (2.0 * 8.0**2))
    rho = (g / (g.sum() * dx**3) * 2.0e11).astype(np.float32)
    phi = _Field(np.zeros_like(rho))
    FFTPoissonSolver(n, dx=dx, grav_constant=units.G, use_gpu=False).solve(_Field(rho), phi)
    pe_grid = diagnostics.potential_energy_grid(rho, phi.a, dx)
    np.savez_compressed(OUT / "fft_offcenter_dx2.npz", rho=rho, phi=phi.a, dx=dx, grav=units.G, pe_grid=pe_grid)

    # 3. Plummer IC and the host FP64 diagnostics on it (test_diagnostics.py:107-171 setup)
    gs = 64
    cfg = SimConfig(ic_preset="plummer", grid_size=gs, n_particles=8000, seed=11)
    icr = build_plummer_ic(cfg, model=PlummerModel(total_mass=2.0e10, scale_a=4.0, center=(gs / 2.0,) * 3))
    m = icr.mass.astype(np.float64)
    pos, vel = icr.pos.astype(np.float64), icr.vel.astype(np.float64)
    np.savez_compressed(
        OUT / "plummer_diag.npz",
        pos=icr.pos, vel=icr.vel, mass=icr.mass, grid_size=gs, grav=units.G,
        kinetic=diagnostics.kinetic_energy(m, vel),
        momentum=diagnostics.linear_momentum(m, vel),
        ang_momentum=diagnostics.angular_momentum(m, pos, vel),
        center_of_mass=diagnostics.center_of_mass(m, pos),
        half_mass_radius=diagnostics.lagrangian_radius(m, pos, 0.5),
        pe_direct_soft1=diagnostics.potential_energy_direct(m[:2000], pos[:2000], softening=1.0, grav=units.G),
    )
    print("wrote", sorted(p.name for p in OUT.glob("*.npz")))


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_golden.py <path to the reference checkout>")
    main(sys.argv[1])
