"""Seeded host samplers of the benchmark workloads (NumPy ``default_rng``, f32 state).

* :func:`plummer` -- an isolated Plummer sphere (G = M = a = 1): radii from
  r = a / sqrt(u^(-2/3) - 1) truncated at 10a (resampled beyond), isotropic
  directions, speeds q * v_esc with q drawn from g(q) = q^2 (1-q^2)^3.5 by
  rejection and v_esc = sqrt(2) (1 + r^2)^(-1/4). The reference's own sampler
  (src/galaxy_collision/ic.py:296-338) clips at 20a and re-centres; this one
  follows the benchmark specification instead.
* :func:`two_disk` -- two exponential disks (surface density exp(-R/Rd),
  truncated at 5 Rd, vertical sech^2(z/z0) with z0 = 0.1 Rd) with a central
  point mass of 1% of each disk's mass, circular velocities from the enclosed
  disk + central mass with one-cell Plummer softening, plus 10% Gaussian
  dispersion; disk 2 inclined 30 degrees about x; centres 20 apart along x and
  2 along y, approaching at relative speed 0.5, in the centre-of-mass frame.

Positions are physical (the benchmark box is [-L/2, L/2]^3); the engine shifts
them to grid-origin coordinates.
"""

from __future__ import annotations

from dataclasses import dataclass

import numpy as np


@dataclass
class ICResult:
    pos: np.ndarray   # (N, 3) f32
    vel: np.ndarray   # (N, 3) f32
    mass: np.ndarray  # (N,) f32
    gid: np.ndarray   # (N,) i32

    @property
    def n(self) -> int:
        return int(self.pos.shape[0])


def _unit_vectors(rng, n):
    v = rng.normal(size=(n, 3))
    v /= np.linalg.norm(v, axis=1, keepdims=True)
    return v


def _plummer_q(rng, n):
    out = np.empty(n)
    filled = 0
    while filled < n:
        m = max(1024, int(1.2 * (n - filled) * 10))
        x = rng.random(m)
        y = rng.random(m)
        ok = x[0.1 * y < x**2 * (1.0 - x**2) ** 3.5]
        k = min(ok.size, n - filled)
        out[filled:filled + k] = ok[:k]
        filled += k
    return out


def plummer(n: int = 131072, seed: int = 0, mass: float = 1.0, a: float = 1.0, rmax: float = 10.0,
            grav: float = 1.0) -> ICResult:
    rng = np.random.default_rng(seed)
    r = np.empty(n)
    filled = 0
    while filled < n:
        u = rng.random(n - filled)
        u = np.clip(u, 1e-300, 1.0 - 1e-16)
        rr = a / np.sqrt(u ** (-2.0 / 3.0) - 1.0)
        rr = rr[rr <= rmax * a]
        r[filled:filled + rr.size] = rr
        filled += rr.size
    pos = r[:, None] * _unit_vectors(rng, n)
    q = _plummer_q(rng, n)
    vesc = np.sqrt(2.0 * grav * mass / a) * (1.0 + (r / a) ** 2) ** (-0.25)
    vel = (q * vesc)[:, None] * _unit_vectors(rng, n)
    return ICResult(pos.astype(np.float32), vel.astype(np.float32), np.full(n, mass / n, np.float32),
                    np.zeros(n, np.int32))


def _disk(rng, n_disk, m_disk, rd, grav, soft, chunk=1 << 22):
    """Positions/velocities of n_disk particles of an exponential sech^2 disk plus
    the central point mass (returned separately)."""
    rcut = 5.0 * rd
    # inverse CDF of the truncated exponential surface density, tabulated
    rt = np.linspace(0.0, rcut, 8192)
    cdf = 1.0 - (1.0 + rt / rd) * np.exp(-rt / rd)
    cdf /= cdf[-1]
    m_bh = 0.01 * m_disk
    z0 = 0.1 * rd
    pos = np.empty((n_disk, 3), np.float32)
    vel = np.empty((n_disk, 3), np.float32)
    for s in range(0, n_disk, chunk):
        k = min(chunk, n_disk - s)
        R = np.interp(rng.random(k), cdf, rt)
        th = rng.random(k) * (2.0 * np.pi)
        z = z0 * np.arctanh(np.clip(2.0 * rng.random(k) - 1.0, -1 + 1e-12, 1 - 1e-12))
        menc = m_disk * np.interp(R, rt, cdf) + m_bh
        vc = np.sqrt(grav * menc * R * R / (R * R + soft * soft) ** 1.5)
        c, sn = np.cos(th), np.sin(th)
        pos[s:s + k, 0] = R * c
        pos[s:s + k, 1] = R * sn
        pos[s:s + k, 2] = z
        disp = rng.normal(size=(k, 3)) * (0.1 * vc)[:, None]
        vel[s:s + k, 0] = -vc * sn + disp[:, 0]
        vel[s:s + k, 1] = vc * c + disp[:, 1]
        vel[s:s + k, 2] = disp[:, 2]
    return pos, vel, m_bh


def two_disk(n1: int = 4_000_000, n2: int = 6_000_000, seed: int = 1, m1: float = 1.0, m2: float = 1.5,
             rd1: float = 1.0, rd2: float = 1.2, incline_deg: float = 30.0, separation=(20.0, 2.0, 0.0),
             approach_speed: float = 0.5, grav: float = 1.0, dx: float = 0.25) -> ICResult:
    """The two-disk collision. n1/n2 count all particles of each galaxy, the
    central point mass included (one particle carrying 1% of the disk mass)."""
    rng = np.random.default_rng(seed)
    parts = []
    for gid, (n, m_disk, rd) in enumerate(((n1, m1, rd1), (n2, m2, rd2))):
        nd = n - 1
        p, v, m_bh = _disk(rng, nd, m_disk, rd, grav, soft=dx)
        mass = np.full(n, m_disk / nd, np.float32)
        mass[-1] = m_bh
        p = np.concatenate([p, np.zeros((1, 3), np.float32)])
        v = np.concatenate([v, np.zeros((1, 3), np.float32)])
        if gid == 1 and incline_deg:
            a = np.deg2rad(incline_deg)
            rot = np.array([[1, 0, 0], [0, np.cos(a), -np.sin(a)], [0, np.sin(a), np.cos(a)]], np.float32)
            p = p @ rot.T
            v = v @ rot.T
        parts.append((p, v, mass, np.full(n, gid, np.int32)))
    M1 = float(parts[0][2].astype(np.float64).sum())
    M2 = float(parts[1][2].astype(np.float64).sum())
    sep = np.asarray(separation, np.float64)
    off1, off2 = -M2 / (M1 + M2) * sep, M1 / (M1 + M2) * sep
    vrel = np.array([approach_speed, 0.0, 0.0])
    v1, v2 = M2 / (M1 + M2) * vrel, -M1 / (M1 + M2) * vrel
    for (p, v, _, _), off, dv in ((parts[0], off1, v1), (parts[1], off2, v2)):
        p += off.astype(np.float32)
        v += dv.astype(np.float32)
    return ICResult(np.concatenate([q[0] for q in parts]), np.concatenate([q[1] for q in parts]),
                    np.concatenate([q[2] for q in parts]), np.concatenate([q[3] for q in parts]))


# Benchmark configurations (sizes, box, grid, time step, seed).
CONFIGS = {
    "plummer_131k": dict(kind="plummer", n=131072, seed=0, box=24.0, grid=64, dt=0.01, steps=200),
    "two_disk_10M": dict(kind="two_disk", n1=4_000_000, n2=6_000_000, seed=1, box=64.0, grid=256, dt=0.005,
                         steps=500),
    "two_disk_100M": dict(kind="two_disk", n1=40_000_000, n2=60_000_000, seed=2, box=64.0, grid=256, dt=0.005,
                          steps=200, fixed_point_bits=40),
}


def build(name: str, scale: float = 1.0) -> tuple[ICResult, dict]:
    """Sample configuration ``name`` (optionally with the particle counts scaled)."""
    cfg = dict(CONFIGS[name])
    dx = cfg["box"] / cfg["grid"]
    if cfg["kind"] == "plummer":
        ic = plummer(max(1, int(cfg["n"] * scale)), seed=cfg["seed"])
    else:
        ic = two_disk(max(2, int(cfg["n1"] * scale)), max(2, int(cfg["n2"] * scale)), seed=cfg["seed"], dx=dx)
    cfg["dx"] = dx
    cfg["origin"] = (-cfg["box"] / 2.0,) * 3
    return ic, cfg


__all__ = ["ICResult", "plummer", "two_disk", "CONFIGS", "build"]
