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


# ---------------------------------------------------------------------------- device samplers
@dataclass
class DeviceIC:
    """Initial conditions resident on the GPU (the layout of :class:`ICResult`)."""

    pos: "torch.Tensor"   # (N, 3) f32, physical coordinates
    vel: "torch.Tensor"   # (N, 3) f32
    mass: "torch.Tensor"  # (N,) f32
    gid: "torch.Tensor"   # (N,) i32

    @property
    def n(self) -> int:
        return int(self.pos.shape[0])

    def to_host(self) -> ICResult:
        return ICResult(self.pos.cpu().numpy(), self.vel.cpu().numpy(), self.mass.cpu().numpy(),
                        self.gid.cpu().numpy())


def _alloc_device(n: int):
    import torch

    dev = torch.device("cuda", torch.cuda.current_device())
    return (torch.empty((n, 3), dtype=torch.float32, device=dev), torch.empty((n, 3), dtype=torch.float32, device=dev),
            torch.empty(n, dtype=torch.float32, device=dev), torch.empty(n, dtype=torch.int32, device=dev))


def plummer_device(n: int = 131072, seed: int = 0, mass: float = 1.0, a: float = 1.0, rmax: float = 10.0,
                   grav: float = 1.0) -> DeviceIC:
    """:func:`plummer` drawn on the GPU (``gc_ic_plummer``): same distributions,
    counter-based random numbers (particle i depends only on seed and i)."""
    from galaxy_collision_gb300._ops import op_context

    pos, vel, m, g = _alloc_device(n)
    op_context(2, 1.0).call("gc_ic_plummer", int(n), int(seed), float(mass), float(a), float(rmax), float(grav),
                            pos.data_ptr(), vel.data_ptr(), m.data_ptr(), g.data_ptr(), what="gc_ic_plummer")
    return DeviceIC(pos, vel, m, g)


def two_disk_device(n1: int = 4_000_000, n2: int = 6_000_000, seed: int = 1, m1: float = 1.0, m2: float = 1.5,
                    rd1: float = 1.0, rd2: float = 1.2, incline_deg: float = 30.0, separation=(20.0, 2.0, 0.0),
                    approach_speed: float = 0.5, grav: float = 1.0, dx: float = 0.25) -> DeviceIC:
    """:func:`two_disk` drawn on the GPU (``gc_ic_disk`` per galaxy): the same
    construction in the centre-of-mass frame; galaxy g fills rows [off_g, off_g + n_g)
    with its central point mass last."""
    import ctypes as C

    from galaxy_collision_gb300._ops import op_context

    n = n1 + n2
    pos, vel, m, g = _alloc_device(n)
    # galaxy masses as the device writes them (f32 particle masses)
    M = [float(np.float32(md / (nk - 1))) * (nk - 1) + float(np.float32(0.01 * md)) for nk, md in ((n1, m1), (n2, m2))]
    sep = np.asarray(separation, np.float64)
    offs = (-M[1] / (M[0] + M[1]) * sep, M[0] / (M[0] + M[1]) * sep)
    vrel = np.array([approach_speed, 0.0, 0.0])
    bulks = (M[1] / (M[0] + M[1]) * vrel, -M[0] / (M[0] + M[1]) * vrel)
    ctx = op_context(2, 1.0)
    row = 0
    for gal, (nk, md, rd, inc) in enumerate(((n1, m1, rd1, 0.0), (n2, m2, rd2, incline_deg))):
        off = (C.c_double * 3)(*offs[gal])
        bulk = (C.c_double * 3)(*bulks[gal])
        ctx.call("gc_ic_disk", int(nk - 1), int(seed), gal, float(md), float(rd), float(grav), float(dx), float(inc),
                 off, bulk, pos[row:].data_ptr(), vel[row:].data_ptr(), m[row:].data_ptr(), g[row:].data_ptr(),
                 what="gc_ic_disk")
        row += nk
    return DeviceIC(pos, vel, m, g)


def equilibrate_disk_velocities(ic, *, dx: float, grid: int, origin, grav: float = 1.0, n_radii: int = 64,
                                n_azimuth: int = 64, tol: float = 1e-6) -> dict:
    """Launch each disk on the circular speed the PM grid gives it
    (equilibrate_disk_velocities, reference ic.py:408-525): for each galaxy, its
    own particles are deposited, solved (cold start) and differentiated on the
    production grid; rings of probes in the plane through its central mass
    sample the azimuthal mean of the inward radial acceleration, v_c(R) =
    sqrt(R <-a_R>); every disk particle gets the tangential speed R omega(R)
    (omega = v_c / R interpolated linearly) plus the galaxy's bulk velocity.
    The central point mass (the galaxy's last particle) keeps its velocity.
    Works on a :class:`DeviceIC` in place; returns {gid: (r_table, vc_table)}."""
    import torch

    from galaxy_collision_gb300.data import Field, ParticleState
    from galaxy_collision_gb300.deposit import deposit_density, gather_acceleration, potential_to_accel
    from galaxy_collision_gb300.solver import make_solver

    dev = ic.pos.device
    org = torch.as_tensor(np.asarray(origin, np.float64), device=dev)
    solver = make_solver("multigrid", grid, dx=dx, grav_constant=grav, tol=tol, n_cycles=60)
    rho, phi = Field((grid,) * 3), Field((grid,) * 3)
    ax, ay, az = Field((grid,) * 3), Field((grid,) * 3), Field((grid,) * 3)
    curves = {}
    gids = torch.unique(ic.gid).tolist()
    for gal in gids:
        idx = torch.nonzero(ic.gid == gal).flatten()
        bh = int(idx[-1])
        center = ic.pos[bh].double()
        bulk = ic.vel[bh].clone()
        disk = idx[:-1]
        rel = (ic.pos[idx].double() - org).float()
        parts = ParticleState(int(idx.numel()))
        for i, k in enumerate(("pos_x", "pos_y", "pos_z")):
            getattr(parts, k).tensor.copy_(rel[:, i])
        parts.mass.tensor.copy_(ic.mass[idx])
        deposit_density(parts, rho, dx)
        solver.solve(rho, phi, warm_start=False)
        potential_to_accel(phi, ax, ay, az, dx)
        dxp = (ic.pos[disk, 0].double() - center[0])
        dyp = (ic.pos[disk, 1].double() - center[1])
        r_disk = torch.hypot(dxp, dyp)
        r_max = float(r_disk.max())
        r_tab = np.linspace(dx, r_max, n_radii)
        th = np.linspace(0.0, 2.0 * np.pi, n_azimuth, endpoint=False)
        rr, tt = np.meshgrid(r_tab, th, indexing="ij")
        c_np = center.cpu().numpy() - np.asarray(origin, np.float64)
        probes = ParticleState(rr.size)
        probes.pos_x.from_numpy((c_np[0] + rr * np.cos(tt)).ravel().astype(np.float32))
        probes.pos_y.from_numpy((c_np[1] + rr * np.sin(tt)).ravel().astype(np.float32))
        probes.pos_z.from_numpy(np.full(rr.size, c_np[2], np.float32))
        pax, pay, paz = Field(rr.size), Field(rr.size), Field(rr.size)
        gather_acceleration(probes, ax, ay, az, pax, pay, paz, dx)
        a_rad = pax.to_numpy().reshape(rr.shape) * np.cos(tt) + pay.to_numpy().reshape(rr.shape) * np.sin(tt)
        inward = np.maximum(-a_rad.mean(axis=1), 0.0)
        vc_tab = np.sqrt(r_tab * inward)
        curves[int(gal)] = (r_tab, vc_tab)
        # omega(R) interpolated linearly (clamped at the table ends), v = R omega tangential + bulk
        rt = torch.as_tensor(r_tab, device=dev)
        om = torch.as_tensor(vc_tab / r_tab, device=dev)
        j = torch.clamp(torch.searchsorted(rt, r_disk) - 1, 0, n_radii - 2)
        w = torch.clamp((r_disk - rt[j]) / (rt[j + 1] - rt[j]), 0.0, 1.0)
        omega = om[j] * (1 - w) + om[j + 1] * w
        vc = r_disk * omega
        safe = torch.clamp(r_disk, min=1e-6)
        ic.vel[disk, 0] = (vc * (-dyp / safe)).float() + bulk[0]
        ic.vel[disk, 1] = (vc * (dxp / safe)).float() + bulk[1]
        ic.vel[disk, 2] = bulk[2]
    return curves


# Benchmark configurations (sizes, box, grid, time step, seed).
CONFIGS = {
    "plummer_131k": dict(kind="plummer", n=131072, seed=0, box=24.0, grid=64, dt=0.01, steps=200),
    "two_disk_10M": dict(kind="two_disk", n1=4_000_000, n2=6_000_000, seed=1, box=64.0, grid=256, dt=0.005,
                         steps=500, fixed_point_bits=44),
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


__all__ = ["ICResult", "DeviceIC", "plummer", "two_disk", "plummer_device", "two_disk_device",
           "equilibrate_disk_velocities", "CONFIGS", "build"]
