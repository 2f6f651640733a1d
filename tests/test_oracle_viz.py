"""The viewer's colour and drawing rules, restated in oracle/viz.py, on cases
whose answers follow from the reference's formulas (viewer.py:50-121, 200-283)."""

from __future__ import annotations

import math

import numpy as np

from oracle import viz


def test_log_window_is_four_decades_below_the_peak():
    lo, inv = viz.log_window(1000.0)
    assert math.isclose(lo, math.log(1000.0) - 4 * math.log(10.0))
    assert math.isclose(1.0 / inv, 4 * math.log(10.0))


def test_colormap_ends_and_nonpositive():
    lut = np.stack([np.linspace(0, 1, 256)] * 3, axis=1).astype(np.float32)
    lo, inv = viz.log_window(100.0)
    v = np.array([0.0, -1.0, 100.0, 1e9, 100.0 * 1e-4, 1e-12], np.float32)
    idx = viz.lut_index(v, lo, inv)
    assert list(idx) == [0, 0, 255, 255, 0, 0]
    # halfway in log space: 2 decades below the peak -> t = 0.5 -> int(127.5 + 0.5) = 128
    assert viz.lut_index(np.float32(1.0), lo, inv) == 128
    rgb = viz.colormap_log(v, lut, lo, inv)
    assert rgb.shape == (6, 3) and rgb[2, 0] == 1.0 and rgb[0, 0] == 0.0


def test_pack_and_density_color_indices():
    x = np.array([0.0, 1.0, 2.0, 3.0, 4.0, 63.9], np.float32)
    p = viz.pack_positions(x, x, x, 2, 1.0 / 64.0, 3)
    np.testing.assert_array_equal(p[:, 0], np.float32([0.0, 2.0, 4.0]) / np.float32(64) - np.float32(0.5))
    G = 4
    rho = np.zeros((G, G, G), np.float32)
    rho[1, 1, 1] = 10.0
    lut = np.stack([np.linspace(0, 1, 256)] * 3, axis=1).astype(np.float32)
    lo, inv = viz.log_window(10.0)
    # nearest node of 0.6 (dx 1) is 1; of -3 clamps to 0
    c = viz.density_color(np.float32([0.6, -3.0]), np.float32([0.6, 0.6]), np.float32([0.6, 0.6]), rho, 1, 2, 1.0,
                          G, lut, lo, inv)
    assert c[0, 0] == 1.0 and c[1, 0] == 0.0


def test_splat_nearest_wins_and_ties_to_lower_index():
    I = np.eye(4, dtype=np.float32)  # clip = position; depth = z
    pos = np.array([[0.0, 0.0, 0.5], [0.0, 0.0, 0.25], [0.0, 0.0, 0.25], [0.9, 0.9, 0.1]], np.float32)
    col = np.array([[1, 0, 0], [0, 1, 0], [0, 0, 1], [1, 1, 1]], np.float32)
    img = viz.splat(pos, col, I, 8, 8, 1.0, (0, 0, 0))
    # pixel centre (4.5, 4.5) ... the centre pixels (3..4) see point 1 (nearer than 0, lower index than 2)
    assert tuple(img[4, 4, :3]) == (0, 255, 0) and tuple(img[3, 3, :3]) == (0, 255, 0)
    # point 3 at ndc (0.9, 0.9) -> px 7.6, py 0.4: top-right corner
    assert tuple(img[0, 7, :3]) == (255, 255, 255)
    assert tuple(img[7, 0, :3]) == (0, 0, 0) and img[7, 0, 3] == 255
    # behind the camera (w <= 0) or outside [0, 1] depth: not drawn
    M = I.copy()
    M[3, 3] = -1.0
    assert (viz.splat(pos, col, M, 8, 8, 1.0, (0, 0, 0))[..., :3] == 0).all()
