"""Host FP64 conservation diagnostics (the reference's src/galaxy_collision/diagnostics.py:69-173).

Used at cadence for quantities that need all pairs or all positions on the
host (the O(N^2) softened pair-sum potential energy for small validation runs,
the exact Lagrangian radius); the per-step sums are reduced on the device
(:mod:`galaxy_collision_gb300.diagnostics_device`).
"""

from __future__ import annotations

import numpy as np

from galaxy_collision_gb300 import units


def kinetic_energy(mass, vel) -> float:
    mass = np.asarray(mass, np.float64)
    vel = np.asarray(vel, np.float64)
    return float(0.5 * np.sum(mass * np.sum(vel**2, axis=1)))


def linear_momentum(mass, vel) -> np.ndarray:
    return (np.asarray(mass, np.float64)[:, None] * np.asarray(vel, np.float64)).sum(axis=0)


def angular_momentum(mass, pos, vel, center=None) -> np.ndarray:
    pos = np.asarray(pos, np.float64)
    r = pos if center is None else pos - np.asarray(center, np.float64)
    return (np.asarray(mass, np.float64)[:, None] * np.cross(r, np.asarray(vel, np.float64))).sum(axis=0)


def center_of_mass(mass, pos) -> np.ndarray:
    mass = np.asarray(mass, np.float64)
    return (mass[:, None] * np.asarray(pos, np.float64)).sum(axis=0) / mass.sum()


def lagrangian_radius(mass, pos, fraction: float = 0.5, center=None) -> float:
    mass = np.asarray(mass, np.float64)
    pos = np.asarray(pos, np.float64)
    c = center_of_mass(mass, pos) if center is None else np.asarray(center, np.float64)
    r = np.linalg.norm(pos - c, axis=1)
    order = np.argsort(r)
    cum = np.cumsum(mass[order])
    idx = int(np.searchsorted(cum, fraction * mass.sum()))
    return float(r[order][min(idx, len(r) - 1)])


def potential_energy_direct(mass, pos, softening: float = 0.0, grav: float | None = None,
                            block: int = 2048) -> float:
    """-1/2 G sum_{i != j} m_i m_j / sqrt(r_ij^2 + eps^2), in row blocks to bound memory."""
    g = units.G if grav is None else grav
    mass = np.asarray(mass, np.float64)
    pos = np.asarray(pos, np.float64)
    total = 0.0
    for s in range(0, len(mass), block):
        d = pos[s:s + block, None, :] - pos[None, :, :]
        r2 = (d**2).sum(-1) + softening**2
        idx = np.arange(s, min(s + block, len(mass)))
        r2[idx - s, idx] = np.inf
        total += float(np.sum(mass[s:s + block, None] * mass[None, :] / np.sqrt(r2)))
    return -0.5 * g * total


def potential_energy_grid(rho, phi, dx: float = 1.0) -> float:
    return float(0.5 * np.sum(np.asarray(rho, np.float64) * np.asarray(phi, np.float64)) * dx**3)


def virial_ratio(kinetic: float, potential: float) -> float:
    return kinetic / abs(potential) if potential != 0.0 else float("nan")


__all__ = ["kinetic_energy", "linear_momentum", "angular_momentum", "center_of_mass", "lagrangian_radius",
           "potential_energy_direct", "potential_energy_grid", "virial_ratio"]
