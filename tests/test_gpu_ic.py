"""Initial conditions drawn on the GPU: the generator bit for bit against its
NumPy restatement, and the sampled distributions against their definitions and
the host samplers."""

from __future__ import annotations

import ctypes as C

import numpy as np
import pytest
import torch

from oracle import rng as orng

pytestmark = pytest.mark.gpu


def test_device_uniforms_are_the_restated_philox(cuda):
    from galaxy_collision_gb300._ops import op_context

    for seed, stream in ((0, 0), (0x123456789ABCDEF, 3)):
        n = 50000
        out = torch.empty(4 * n, dtype=torch.float32, device="cuda")
        op_context(2, 1.0).call("gc_rng_uniform", seed, stream, n, out.data_ptr(), what="rng")
        np.testing.assert_array_equal(out.cpu().numpy().reshape(n, 4), orng.uniforms(seed, stream, n))


def _plummer_mass_fraction(r, rmax=10.0):
    f = lambda x: x**3 / (1 + x * x) ** 1.5  # noqa: E731
    return f(r) / f(rmax)


def test_plummer_device_distribution(cuda):
    from galaxy_collision_gb300 import ic

    n = 1_000_000
    d = ic.plummer_device(n, seed=4)
    pos, vel = d.pos.double().cpu().numpy(), d.vel.double().cpu().numpy()
    r = np.linalg.norm(pos, axis=1)
    assert r.max() <= 10.0 + 1e-5
    for rr in (0.5, 1.0, 2.0, 5.0):
        p = _plummer_mass_fraction(rr)
        assert abs((r < rr).mean() - p) < 4 * np.sqrt(p * (1 - p) / n)
    u = pos / r[:, None]
    assert np.linalg.norm(u.mean(axis=0)) < 5 / np.sqrt(n)
    # q = |v| / v_esc has density ~ q^2 (1 - q^2)^3.5 on (0, 1)
    q = np.linalg.norm(vel, axis=1) / (np.sqrt(2.0) * (1 + r * r) ** -0.25)
    x = np.linspace(0, 1, 200001)
    g = x * x * (1 - x * x) ** 3.5
    trap = getattr(np, "trapezoid", None) or np.trapz
    mq = trap(x * g, x) / trap(g, x)
    sq = np.sqrt(trap(x * x * g, x) / trap(g, x) - mq * mq)
    assert abs(q.mean() - mq) < 5 * sq / np.sqrt(n)
    np.testing.assert_allclose(d.mass.cpu().numpy(), np.float32(1.0 / n))
    # counter-based: the first particles do not depend on n
    e = ic.plummer_device(1000, seed=4)
    np.testing.assert_array_equal(e.pos.cpu().numpy(), d.pos[:1000].cpu().numpy())
    assert torch.equal(ic.plummer_device(1000, seed=4).vel, e.vel)


def test_two_disk_device_matches_host_statistics(cuda):
    from galaxy_collision_gb300 import ic

    n1, n2 = 300_001, 450_001
    dv = ic.two_disk_device(n1, n2, seed=9).to_host()
    hs = ic.two_disk(n1, n2, seed=9)
    assert dv.n == hs.n and (dv.gid == hs.gid).all()
    np.testing.assert_allclose(dv.mass.astype(np.float64).sum(), hs.mass.astype(np.float64).sum(), rtol=1e-6)
    # the centre-of-mass frame
    for s in (dv, hs):
        com = (s.pos.astype(np.float64) * s.mass[:, None]).sum(0) / s.mass.sum()
        assert np.abs(com).max() < 0.02
    # galaxy 0: disk statistics relative to its point mass
    def stats(s):
        sel = np.nonzero(s.gid == 0)[0]
        c = s.pos[sel[-1]].astype(np.float64)
        p = s.pos[sel[:-1]].astype(np.float64) - c
        v = s.vel[sel[:-1]].astype(np.float64) - s.vel[sel[-1]]
        R = np.hypot(p[:, 0], p[:, 1])
        vphi = (p[:, 0] * v[:, 1] - p[:, 1] * v[:, 0]) / np.maximum(R, 1e-9)
        return np.array([R.mean(), (R < 1.0).mean(), np.abs(p[:, 2]).mean(), vphi.mean(), v[:, 2].std()])
    a, b = stats(dv), stats(hs)
    np.testing.assert_allclose(a, b, rtol=0.02)
    # sech^2 layer: mean |z| = z0 ln 2
    assert abs(a[2] - 0.1 * np.log(2.0)) < 0.002


def test_equilibrated_disk_rotates_on_the_grid_curve(cuda):
    from galaxy_collision_gb300 import ic

    d = ic.two_disk_device(150_001, 150_001, seed=3, separation=(24.0, 0.0, 0.0), dx=1.0)
    v_before = d.vel.clone()
    curves = ic.equilibrate_disk_velocities(d, dx=1.0, grid=64, origin=(-32.0, -32.0, -32.0))
    assert set(curves) == {0, 1}
    r_tab, vc = curves[0]
    assert (vc[r_tab > 2.0] > 0).all()
    # point masses keep their velocities; disk speeds follow R omega(R) tangentially
    sel = torch.nonzero(d.gid == 0).flatten()
    assert torch.equal(d.vel[sel[-1]], v_before[sel[-1]])
    c = d.pos[sel[-1]].double()
    p = d.pos[sel[:-1]].double() - c
    v = d.vel[sel[:-1]].double() - d.vel[sel[-1]].double()
    R = torch.hypot(p[:, 0], p[:, 1])
    vr = (p[:, 0] * v[:, 0] + p[:, 1] * v[:, 1]) / R.clamp(min=1e-9)
    assert float(vr.abs().max()) < 1e-4
    vphi = ((p[:, 0] * v[:, 1] - p[:, 1] * v[:, 0]) / R.clamp(min=1e-9)).cpu().numpy()
    want = np.interp(R.cpu().numpy(), r_tab, vc / r_tab) * R.cpu().numpy()
    np.testing.assert_allclose(vphi, want, rtol=1e-4, atol=1e-5)
    # the measured curve is close to the analytic one outside the softened core
    M = 1.01
    sel_r = (r_tab > 3.0) & (r_tab < 4.5)
    vk = np.sqrt(M / r_tab[sel_r])
    assert np.all(vc[sel_r] < 1.15 * vk) and np.all(vc[sel_r] > 0.6 * vk)
