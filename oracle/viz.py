"""CPU restatement of the viewer's device kernels (test infrastructure only).

Follows src/galaxy_collision/viz/viewer.py of the reference: `_pack_positions`
(:50-65), `_colormap_log` (:76-93), `_density_color` (:104-121), and the
window `log_vmin = ln(peak) - 4 ln 10`, `inv_logspan = 1 / (4 ln 10)`
(:200-210, 265, 282). The reference draws its 3-D points with GGUI
`scene.particles` (:258-272), a graphics API; `splat` restates the CUDA
replacement's documented rule instead (flat discs, nearest point per pixel,
ties to the lower index), in float32 with the kernel's operation order so the
pixels match exactly. Parity of `splat` is pinned to that rule only: the
reference has no CPU rasteriser.
"""

from __future__ import annotations

import math

import numpy as np

LUT_N = 256
LOG_DECADES = 4.0

f32 = np.float32


def log_window(peak: float, decades: float = LOG_DECADES) -> tuple[float, float]:
    """(log_vmin, inv_logspan) of the viewer's fixed log window below the peak."""
    return math.log(peak) - decades * math.log(10.0), 1.0 / (decades * math.log(10.0))


def lut_index(v, log_vmin, inv_logspan):
    v = np.asarray(v, np.float32)
    with np.errstate(divide="ignore", invalid="ignore"):
        t = np.where(v > 0, (np.log(np.where(v > 0, v, f32(1))) - f32(log_vmin)) * f32(inv_logspan), f32(0))
    t = np.minimum(f32(1), np.maximum(f32(0), t.astype(np.float32)))
    idx = (t * f32(LUT_N - 1) + f32(0.5)).astype(np.int32)
    return np.clip(idx, 0, LUT_N - 1)


def colormap_log(img, lut, log_vmin, inv_logspan):
    return np.asarray(lut, np.float32)[lut_index(img, log_vmin, inv_logspan)]


def pack_positions(x, y, z, stride, inv_box, m):
    p = np.arange(m) * stride
    ib = f32(inv_box)
    return np.stack([np.asarray(a, np.float32)[p] * ib - f32(0.5) for a in (x, y, z)], axis=1).astype(np.float32)


def density_color(x, y, z, rho, stride, m, inv_dx, G, lut, log_vmin, inv_logspan):
    p = np.arange(m) * stride
    idx = [np.clip((np.asarray(a, np.float32)[p] * f32(inv_dx) + f32(0.5)).astype(np.int32), 0, G - 1) for a in (x, y, z)]
    v = np.asarray(rho, np.float32).reshape(G, G, G)[idx[0], idx[1], idx[2]]
    return colormap_log(v, lut, log_vmin, inv_logspan)


def splat(pos, col, view_proj, width, height, radius_px, bg):
    """RGBA8 image (height, width, 4) of the discs, nearest point per pixel."""
    pos = np.asarray(pos, np.float32)
    M = np.asarray(view_proj, np.float32).reshape(4, 4)
    x, y, z = pos[:, 0], pos[:, 1], pos[:, 2]

    def row(r):
        return ((M[r, 0] * x + M[r, 1] * y) + M[r, 2] * z) + M[r, 3]

    xc, yc, zc, wc = row(0), row(1), row(2), row(3)
    keep = wc > 0
    with np.errstate(divide="ignore", invalid="ignore"):
        iw = f32(1) / np.where(keep, wc, f32(1))
        depth = zc * iw + f32(0)
    keep &= (depth >= 0) & (depth <= 1)
    px = (xc * iw + f32(1)) * (f32(0.5) * f32(width))
    py = (f32(1) - yc * iw) * (f32(0.5) * f32(height))
    r = f32(radius_px)
    r2 = r * r
    best = np.full(width * height, np.iinfo(np.uint64).max, dtype=np.uint64)
    for i in np.nonzero(keep)[0]:
        u0 = max(0, int(np.floor(px[i] - r)))
        u1 = min(width - 1, int(np.floor(px[i] + r)))
        v0 = max(0, int(np.floor(py[i] - r)))
        v1 = min(height - 1, int(np.floor(py[i] + r)))
        if u0 > u1 or v0 > v1:
            continue
        us = np.arange(u0, u1 + 1, dtype=np.float32)
        vs = np.arange(v0, v1 + 1, dtype=np.float32)
        dx = (us + f32(0.5)) - px[i]
        dy = (vs + f32(0.5)) - py[i]
        cover = (dx[None, :] * dx[None, :] + dy[:, None] * dy[:, None]) <= r2
        vv, uu = np.nonzero(cover)
        pix = (vv + v0) * width + (uu + u0)
        key = (np.uint64(depth[i].view(np.uint32)) << np.uint64(32)) | np.uint64(i)
        best[pix] = np.minimum(best[pix], key)
    col = np.asarray(col, np.float32)
    rgb = np.tile(np.asarray(bg, np.float32), (width * height, 1))
    hit = best != np.iinfo(np.uint64).max
    rgb[hit] = col[(best[hit] & np.uint64(0xFFFFFFFF)).astype(np.int64)]
    u8 = (np.clip(rgb, 0, 1) * f32(255) + f32(0.5)).astype(np.int32).astype(np.uint8)
    out = np.empty((height, width, 4), np.uint8)
    out[..., :3] = u8.reshape(height, width, 3)
    out[..., 3] = 255
    return out


__all__ = ["LUT_N", "LOG_DECADES", "log_window", "lut_index", "colormap_log", "pack_positions", "density_color",
           "splat"]
