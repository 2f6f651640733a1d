"""Device NGP projection against a NumPy restatement of the reference kernel
(viz/project.py:26-46: f32 bin index, out-of-range mass dropped)."""

from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _oracle(a, b, m, extent, bins):
    lo_a, hi_a, lo_b, hi_b = extent
    bw_a, bw_b = np.float32((hi_a - lo_a) / bins), np.float32((hi_b - lo_b) / bins)
    ga = np.floor((a.astype(np.float32) - np.float32(lo_a)) / bw_a)
    gb = np.floor((b.astype(np.float32) - np.float32(lo_b)) / bw_b)
    ok = (ga >= 0) & (ga < bins) & (gb >= 0) & (gb < bins)
    img = np.zeros((bins, bins), np.float64)
    np.add.at(img, (ga[ok].astype(int), gb[ok].astype(int)), m[ok].astype(np.float64))
    return img, float(bw_a), float(bw_b)


def test_projection_matches_oracle(cuda):
    from galaxy_collision_gb300.data import Field, ParticleState
    from galaxy_collision_gb300.project import project_density, scatter_density

    rng = np.random.default_rng(4)
    n, bins = 200000, 128
    pos = (rng.normal(size=(n, 3)) * 6.0 + 16.0).astype(np.float32)
    pos[:10] = [[-5, 3, 3], [40, 3, 3], [np.nan, 1, 1], [0, 0, 0], [32, 32, 0], [0.0, 31.999, 0], [5, 5, 5],
                [16, 16, 16], [31.75, 0.25, 2], [-0.0001, 4, 4]]
    mass = rng.uniform(0.5, 2.0, size=n).astype(np.float32)
    parts = ParticleState(n)
    for f, c in zip((parts.pos_x, parts.pos_y, parts.pos_z), pos.T):
        f.from_numpy(np.ascontiguousarray(c))
    parts.mass.from_numpy(mass)
    extent = (0.0, 32.0, 0.0, 32.0)
    for axes in ((0, 1), (0, 2), (2, 1)):
        img = Field((bins, bins))
        bw = scatter_density(parts, img, extent, axes)
        ref, bwa, bwb = _oracle(pos[:, axes[0]], pos[:, axes[1]], mass, extent, bins)
        np.testing.assert_allclose(img.to_numpy(), ref, rtol=2e-6, atol=1e-4)
        assert bw == pytest.approx((bwa, bwb))
        sd = project_density(parts, img, extent, axes)
        np.testing.assert_allclose(sd, ref.T / (bw[0] * bw[1]), rtol=2e-6, atol=1e-4)
