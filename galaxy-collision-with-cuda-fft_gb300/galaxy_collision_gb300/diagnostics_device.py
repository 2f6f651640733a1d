"""Device-resident conservation diagnostics (drop-in for src/galaxy_collision/diagnostics_device.py).

FP64 reductions on the GPU: particle scalars [M, KE, P, L about the origin,
Sum m r] (diagnostics_device.py:42-74), Sum rho*phi (:78-88) and the
mass-weighted radial histogram for the half-mass radius (:153-185, 255-271).
Only a few scalars and the histogram cross to the host.
"""

from __future__ import annotations

import ctypes as C

import numpy as np
import torch

from galaxy_collision_gb300._ops import op_context
from galaxy_collision_gb300.data import as_tensor


def particle_scalars(parts, grid_size: int = 2, dx: float = 1.0) -> np.ndarray:
    n = int(parts.n)
    arrs = [as_tensor(getattr(parts, a), shape=(n,), name=a)
            for a in ("pos_x", "pos_y", "pos_z", "vel_x", "vel_y", "vel_z", "mass")]
    out = (C.c_double * 11)()
    op_context(grid_size, dx).call("gc_diag_particles", *(a.data_ptr() for a in arrs), n, out,
                                   what="diag particles")
    return np.array(out[:], dtype=np.float64)


def grid_pe_raw(rho, phi) -> float:
    r = rho.tensor if hasattr(rho, "tensor") else rho
    G = r.shape[0]
    rr = as_tensor(rho, shape=(G, G, G), name="rho")
    pp = as_tensor(phi, shape=(G, G, G), name="phi")
    out = C.c_double()
    op_context(G, 1.0).call("gc_diag_grid_pe", rr.data_ptr(), pp.data_ptr(), C.byref(out), what="grid pe")
    return float(out.value)


class DeviceDiagnostics:
    """Reusable device buffers + reductions; :meth:`sample` returns the reference's keys."""

    def __init__(self, grid_size: int, *, nbins: int = 2048, r_max: float | None = None):
        self.grid_size = int(grid_size)
        self.nbins = int(nbins)
        self.r_max = float(r_max) if r_max is not None else float(grid_size) * float(np.sqrt(3.0))
        self.binw = self.r_max / self.nbins
        self._hist = torch.zeros(self.nbins, dtype=torch.float64, device="cuda")

    def _half_mass_radius(self, parts, cx: float, cy: float, cz: float, total: float) -> float:
        n = int(parts.n)
        arrs = [as_tensor(getattr(parts, a), shape=(n,), name=a) for a in ("pos_x", "pos_y", "pos_z", "mass")]
        # the reference passes the centre and 1/binw as f32 kernel arguments
        f32 = lambda v: float(np.float32(v))  # noqa: E731
        op_context(self.grid_size, 1.0).call(
            "gc_radial_histogram", *(a.data_ptr() for a in arrs), n, f32(cx), f32(cy), f32(cz),
            f32(1.0 / self.binw), self.nbins, self._hist.data_ptr(), what="radial histogram")
        hist = self._hist.cpu().numpy()
        cum = np.cumsum(hist)
        target = 0.5 * total
        b = int(np.searchsorted(cum, target))
        if b >= self.nbins:
            return self.r_max
        cum_lo = cum[b - 1] if b > 0 else 0.0
        frac = (target - cum_lo) / hist[b] if hist[b] > 0.0 else 0.0
        return float((b + frac) * self.binw)

    def sample(self, parts, grid, dx: float, *, half_mass: bool = True) -> dict:
        s = particle_scalars(parts, self.grid_size, dx)
        pe = 0.5 * float(dx) ** 3 * grid_pe_raw(grid.rho, grid.phi)
        total = float(s[0])
        ke = float(s[1])
        com = (s[8:11] / total) if total > 0.0 else np.zeros(3)
        out = {
            "M": total,
            "kinetic": ke,
            "potential": pe,
            "energy": ke + pe,
            "momentum": s[2:5].copy(),
            "ang_momentum": s[5:8].copy(),
            "center_of_mass": com,
        }
        if half_mass:
            out["half_mass_radius"] = self._half_mass_radius(parts, float(com[0]), float(com[1]), float(com[2]),
                                                             total)
        return out


__all__ = ["DeviceDiagnostics", "particle_scalars", "grid_pe_raw"]
