"""Host FP64 diagnostics (test infrastructure only): the formulas of
src/galaxy_collision/diagnostics.py:69-173."""

from __future__ import annotations

import numpy as np


def kinetic_energy(mass, vel):
    mass = np.asarray(mass, np.float64)
    vel = np.asarray(vel, np.float64)
    return float(0.5 * np.sum(mass * np.sum(vel**2, axis=1)))


def linear_momentum(mass, vel):
    return (np.asarray(mass, np.float64)[:, None] * np.asarray(vel, np.float64)).sum(axis=0)


def angular_momentum(mass, pos, vel, center=None):
    pos = np.asarray(pos, np.float64)
    r = pos if center is None else pos - np.asarray(center, np.float64)
    return (np.asarray(mass, np.float64)[:, None] * np.cross(r, np.asarray(vel, np.float64))).sum(axis=0)


def center_of_mass(mass, pos):
    mass = np.asarray(mass, np.float64)
    return (mass[:, None] * np.asarray(pos, np.float64)).sum(axis=0) / mass.sum()


def lagrangian_radius(mass, pos, fraction=0.5, center=None):
    mass = np.asarray(mass, np.float64)
    pos = np.asarray(pos, np.float64)
    c = center_of_mass(mass, pos) if center is None else np.asarray(center, np.float64)
    r = np.linalg.norm(pos - c, axis=1)
    order = np.argsort(r)
    cum = np.cumsum(mass[order])
    idx = int(np.searchsorted(cum, fraction * mass.sum()))
    return float(r[order][min(idx, len(r) - 1)])


def potential_energy_direct(mass, pos, softening=0.0, grav=1.0):
    mass = np.asarray(mass, np.float64)
    pos = np.asarray(pos, np.float64)
    diff = pos[:, None, :] - pos[None, :, :]
    r2 = (diff**2).sum(axis=-1) + softening**2
    np.fill_diagonal(r2, np.inf)
    return float(-0.5 * grav * np.sum(mass[:, None] * mass[None, :] / np.sqrt(r2)))


def potential_energy_grid(rho, phi, dx=1.0):
    return float(0.5 * np.sum(np.asarray(rho, np.float64) * np.asarray(phi, np.float64)) * dx**3)


def virial_ratio(kinetic, potential):
    return kinetic / abs(potential) if potential != 0.0 else float("nan")
