"""Device view kernels against the restated viewer rules (oracle/viz.py)."""

from __future__ import annotations

import numpy as np
import pytest
import torch

from oracle import viz as ov

pytestmark = pytest.mark.gpu


def _lut():
    t = np.linspace(0.0, 1.0, 256, dtype=np.float32)
    return np.stack([t, t ** 2, np.sqrt(t)], axis=1).astype(np.float32)


def test_colormap_and_max_match_the_rule(cuda):
    from galaxy_collision_gb300 import viz

    rng = np.random.default_rng(1)
    img = (10.0 ** rng.uniform(-6, 3, size=(200, 300))).astype(np.float32)
    img[rng.random(img.shape) < 0.1] = 0.0
    d = torch.from_numpy(img).cuda()
    peak = viz.device_max(d)
    assert peak == float(img.max())
    lo, inv = viz.log_window(peak)
    lut = _lut()
    got = viz.colormap_log(d, torch.from_numpy(lut).cuda(), lo, inv).cpu().numpy()
    ref = ov.colormap_log(img, lut, lo, inv)
    # logf and NumPy's f32 log may differ by an ulp: a LUT index can move by one
    # only where t * 255 + 0.5 falls within ~1e-5 of an integer
    gi = np.argmin(np.abs(got[..., 1:2] - lut[None, None, :, 1]), axis=-1)
    ri = ov.lut_index(img, lo, inv)
    diff = np.abs(gi - ri)
    assert diff.max() <= 1 and (diff > 0).mean() < 1e-3
    same = diff == 0
    np.testing.assert_array_equal(got[same], ref[same])


def test_pack_density_color_and_splat_match_the_rule(cuda):
    from galaxy_collision_gb300 import viz

    rng = np.random.default_rng(2)
    G, dx = 32, 1.0
    n = 40000
    pos = rng.uniform(-1.0, G + 1.0, size=(n, 3)).astype(np.float32)
    rho = (10.0 ** rng.uniform(-4, 2, size=(G, G, G))).astype(np.float32)
    x, y, z = (torch.from_numpy(np.ascontiguousarray(pos[:, i])).cuda() for i in range(3))
    lut = _lut()
    lo, inv = ov.log_window(float(rho.max()))
    stride, m = 7, len(range(0, n, 7))
    p = viz.pack_positions(x, y, z, stride, 1.0 / G, m).cpu().numpy()
    np.testing.assert_array_equal(p, ov.pack_positions(pos[:, 0], pos[:, 1], pos[:, 2], stride, 1.0 / G, m))
    c = viz.density_color(x, y, z, torch.from_numpy(rho).cuda(), stride, m, 1.0 / dx,
                          torch.from_numpy(lut).cuda(), lo, inv).cpu().numpy()
    cr = ov.density_color(pos[:, 0], pos[:, 1], pos[:, 2], rho, stride, m, 1.0 / dx, G, lut, lo, inv)
    assert (np.abs(c - cr).max(axis=1) > 0).mean() < 1e-3  # logf vs NumPy log, see above
    M = viz.look_at((1.2, -1.5, 0.9), aspect=160 / 120)
    pts = torch.from_numpy(p).cuda()
    cols = torch.from_numpy(cr).cuda()
    for r in (0.0, 1.0, 2.5):
        img = viz.splat(pts, cols, M, 160, 120, r).cpu().numpy()
        ref = ov.splat(p, cr, M, 160, 120, r, (0.02, 0.02, 0.04))
        np.testing.assert_array_equal(img, ref)


def test_render_frames_and_png(cuda, tmp_path):
    from galaxy_collision_gb300 import viz
    from galaxy_collision_gb300.data import Field, ParticleState
    from galaxy_collision_gb300.deposit import deposit_density
    from galaxy_collision_gb300.project import scatter_density

    rng = np.random.default_rng(3)
    n, G, dx = 50000, 32, 1.0
    parts = ParticleState(n)
    pos = (rng.normal(size=(n, 3)) * 4 + G / 2).astype(np.float32)
    for i, k in enumerate(("pos_x", "pos_y", "pos_z")):
        getattr(parts, k).from_numpy(pos[:, i])
    parts.mass.from_numpy(np.full(n, 1.0 / n, np.float32))
    rho = Field((G, G, G))
    deposit_density(parts, rho, dx)
    img3 = viz.render_3d(parts, rho.tensor, dx, float(G), max_points=20000, width=64, height=48)
    assert img3.shape == (48, 64, 4) and img3[..., :3].max() > 0
    proj = Field((64, 64))
    scatter_density(parts, proj, (0.0, float(G), 0.0, float(G)))
    img2 = viz.render_2d(proj.tensor)
    assert img2.shape == (64, 64, 4)
    f = viz.write_png(img2, tmp_path / "frame.png")
    assert f.read_bytes()[:8] == b"\x89PNG\r\n\x1a\n"
