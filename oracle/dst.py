"""Exact FP64 solution of the discrete Dirichlet problem (test infrastructure only).

Solves L phi = rhs on the interior of a G^3 node grid, L the 7-point Laplacian
with spacing dx, phi given on the six faces -- the discrete problem whose
solution the reference multigrid (and the GPU multigrid) converge to
(src/galaxy_collision/solver/multigrid.py:8-15). The face values move to the
right-hand side; the homogeneous interior problem is diagonal in the type-I
sine basis (scipy.fft.dstn, type=1).
"""

from __future__ import annotations

import numpy as np
from scipy.fft import dstn, idstn


def multipole_faces64(rho, dx, grav):
    """Monopole + quadrupole faces of rho about its centre of mass, in FP64
    (the formula of multigrid.py:261-295 and the moments of :364-389)."""
    rho = np.asarray(rho, dtype=np.float64)
    G = rho.shape[0]
    m = rho * dx**3
    ax = np.arange(G) * dx
    M = m.sum()
    phi = np.zeros((G, G, G))
    if M <= 0:
        return phi
    X, Y, Z = np.meshgrid(ax, ax, ax, indexing="ij")
    c = np.array([(m * X).sum(), (m * Y).sum(), (m * Z).sum()]) / M
    S = np.empty((3, 3))
    R = (X - c[0], Y - c[1], Z - c[2])
    for a in range(3):
        for b in range(3):
            S[a, b] = (m * R[a] * R[b]).sum()
    tr = np.trace(S)
    mask = np.zeros((G, G, G), bool)
    mask[0], mask[-1], mask[:, 0], mask[:, -1], mask[:, :, 0], mask[:, :, -1] = (True,) * 6
    rx, ry, rz = R[0][mask], R[1][mask], R[2][mask]
    d2 = rx * rx + ry * ry + rz * rz + 1e-12
    d = np.sqrt(d2)
    nv = np.stack([rx / d, ry / d, rz / d])
    nsn = np.einsum("ip,ij,jp->p", nv, S, nv)
    phi[mask] = -grav * (M / d + (3.0 * nsn - tr) / (2.0 * d2 * d))
    return phi


def solve_dirichlet(rhs, faces, dx):
    """phi with phi = faces on the boundary and L phi = rhs (f64) on the interior."""
    rhs = np.asarray(rhs, dtype=np.float64)
    G = rhs.shape[0]
    phi = np.array(faces, dtype=np.float64, copy=True)
    phi[1:-1, 1:-1, 1:-1] = 0.0
    # move the boundary contribution to the right-hand side
    b = rhs[1:-1, 1:-1, 1:-1].copy()
    inv = 1.0 / dx**2
    b -= inv * (phi[2:, 1:-1, 1:-1] + phi[:-2, 1:-1, 1:-1] + phi[1:-1, 2:, 1:-1] + phi[1:-1, :-2, 1:-1]
                + phi[1:-1, 1:-1, 2:] + phi[1:-1, 1:-1, :-2])
    n = G - 2
    k = np.arange(1, n + 1)
    lam1 = (2.0 * np.cos(np.pi * k / (n + 1)) - 2.0) * inv
    lam = lam1[:, None, None] + lam1[None, :, None] + lam1[None, None, :]
    bh = dstn(b, type=1)
    u = idstn(bh / lam, type=1)
    phi[1:-1, 1:-1, 1:-1] = u
    return phi


def solve_reference_problem(rho, dx, grav):
    """FP64 exact solution of the reference's discrete problem for f32 density rho:
    rhs = f32(4 pi G) * rho (in f32, multigrid.py:463), FP64 multipole faces."""
    rho32 = np.asarray(rho, dtype=np.float32)
    rhs = (np.float32(4.0 * np.pi * grav) * rho32).astype(np.float64)
    faces = multipole_faces64(rho32, dx, grav)
    return solve_dirichlet(rhs, faces, dx)
