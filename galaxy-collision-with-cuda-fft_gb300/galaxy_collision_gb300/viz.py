"""Headless views of the collision: the device kernels of the reference's viewer
(src/galaxy_collision/viz/viewer.py) writing device buffers instead of a GGUI
window.

* 2-D view: the full-N density projection (`project.scatter_density`) coloured
  through a 256-entry LUT on a fixed log window 4 decades below the frame's
  peak (`colormap_log`; viewer.py:76-93, 276-284). Only the peak crosses to the
  host.
* 3-D view: every stride-th particle in a centred unit cube (`pack_positions`,
  viewer.py:50-65) coloured by the local density (`density_color`,
  viewer.py:104-121), drawn by CUDA as flat discs with a per-pixel depth test
  (`splat`), where the reference calls GGUI `scene.particles`.

`render_3d` / `render_2d` return RGBA8 host images; `write_png` stores one
without any imaging library.
"""

from __future__ import annotations

import ctypes as C
import math
import struct
import zlib
from pathlib import Path

import numpy as np
import torch

from galaxy_collision_gb300 import _native
from galaxy_collision_gb300._ops import op_context
from galaxy_collision_gb300.data import as_tensor

LUT_N = 256
LOG_DECADES = 4.0  # the viewer's fixed log dynamic range below the peak (viewer.py:31-36)


def _ctx():
    return op_context(2, 1.0)


def default_lut() -> np.ndarray:
    """256 x 3 f32 colour table: matplotlib's 'inferno' (the reference's LUT,
    viewer.py:124-128) when matplotlib is importable, else a black-red-yellow-
    white ramp of the same monotone lightness."""
    try:
        import matplotlib

        return matplotlib.colormaps["inferno"](np.linspace(0.0, 1.0, LUT_N))[:, :3].astype(np.float32)
    except Exception:
        t = np.linspace(0.0, 1.0, LUT_N)
        r = np.clip(1.6 * t, 0, 1)
        g = np.clip(1.6 * t - 0.55, 0, 1)
        b = np.clip(2.5 * t - 1.5, 0, 1) + 0.25 * np.sin(np.pi * np.clip(2 * t, 0, 1)) * (t < 0.5)
        return np.stack([r, g, np.clip(b, 0, 1)], axis=1).astype(np.float32)


def log_window(peak: float, decades: float = LOG_DECADES) -> tuple[float, float]:
    """(log_vmin, inv_logspan) of the fixed window below the peak (viewer.py:210, 265, 282)."""
    return math.log(peak) - decades * math.log(10.0), 1.0 / (decades * math.log(10.0))


def device_max(a: torch.Tensor) -> float:
    """max(0, max a) reduced on the device; one scalar crosses to the host."""
    a = as_tensor(a, name="array")
    out = torch.empty(1, dtype=torch.float32, device=a.device)
    _ctx().call("gc_max_f32", a.data_ptr(), a.numel(), out.data_ptr(), what="max")
    return float(out.item())


def colormap_log(img: torch.Tensor, lut: torch.Tensor, log_vmin: float, inv_logspan: float) -> torch.Tensor:
    """img (any shape, f32 device) -> RGB f32 of shape img.shape + (3,)."""
    img = as_tensor(img, name="img")
    lut = as_tensor(lut, shape=(LUT_N, 3), name="lut")
    out = torch.empty(tuple(img.shape) + (3,), dtype=torch.float32, device=img.device)
    _ctx().call("gc_colormap_log", img.data_ptr(), img.numel(), lut.data_ptr(), float(log_vmin), float(inv_logspan),
                out.data_ptr(), what="colormap")
    return out


def pack_positions(x, y, z, stride: int, inv_box: float, m: int) -> torch.Tensor:
    """(m, 3) f32 device: particle i*stride in the unit cube centred on the origin."""
    x = as_tensor(x, name="pos_x")
    out = torch.empty((m, 3), dtype=torch.float32, device=x.device)
    _ctx().call("gc_pack_positions", x.data_ptr(), as_tensor(y, name="pos_y").data_ptr(),
                as_tensor(z, name="pos_z").data_ptr(), int(stride), float(inv_box), int(m), out.data_ptr(),
                what="pack_positions")
    return out


def density_color(x, y, z, rho: torch.Tensor, stride: int, m: int, inv_dx: float, lut: torch.Tensor,
                  log_vmin: float, inv_logspan: float) -> torch.Tensor:
    """(m, 3) f32 device colours of particle i*stride from rho at its nearest node."""
    rho = as_tensor(rho, name="rho")
    G = int(rho.shape[0])
    lut = as_tensor(lut, shape=(LUT_N, 3), name="lut")
    x = as_tensor(x, name="pos_x")
    out = torch.empty((m, 3), dtype=torch.float32, device=x.device)
    _ctx().call("gc_density_color", x.data_ptr(), as_tensor(y, name="pos_y").data_ptr(),
                as_tensor(z, name="pos_z").data_ptr(), rho.data_ptr(), G, int(stride), int(m), float(inv_dx),
                lut.data_ptr(), float(log_vmin), float(inv_logspan), out.data_ptr(), what="density_color")
    return out


def look_at(eye, target=(0.0, 0.0, 0.0), up=(0.0, 0.0, 1.0), fov_deg: float = 45.0, aspect: float = 1.0,
            near: float = 0.05, far: float = 10.0) -> np.ndarray:
    """Row-major 4 x 4 perspective view-projection matrix (depth mapped to [0, 1])."""
    eye, target, up = (np.asarray(v, np.float64) for v in (eye, target, up))
    f = target - eye
    f /= np.linalg.norm(f)
    s = np.cross(f, up)
    s /= np.linalg.norm(s)
    u = np.cross(s, f)
    view = np.eye(4)
    view[0, :3], view[1, :3], view[2, :3] = s, u, -f
    view[:3, 3] = -view[:3, :3] @ eye
    t = 1.0 / math.tan(math.radians(fov_deg) / 2)
    proj = np.zeros((4, 4))
    proj[0, 0], proj[1, 1] = t / aspect, t
    proj[2, 2], proj[2, 3] = far / (near - far), near * far / (near - far)
    proj[3, 2] = -1.0
    return (proj @ view).astype(np.float32)


def splat(pos: torch.Tensor, col: torch.Tensor, view_proj, width: int, height: int, radius_px: float = 1.5,
          bg=(0.02, 0.02, 0.04), zbuf: torch.Tensor | None = None) -> torch.Tensor:
    """Draw points as discs: (height, width, 4) uint8 device image."""
    pos = as_tensor(pos, name="pos")
    col = as_tensor(col, name="col")
    m = int(pos.shape[0])
    if zbuf is None or zbuf.numel() < width * height:
        zbuf = torch.empty(width * height, dtype=torch.int64, device=pos.device)
    out = torch.empty((height, width, 4), dtype=torch.uint8, device=pos.device)
    M = (C.c_float * 16)(*np.asarray(view_proj, np.float32).ravel().tolist())
    b = (C.c_float * 3)(*[float(v) for v in bg])
    _ctx().call("gc_splat_points", pos.data_ptr(), col.data_ptr(), m, M, int(width), int(height), float(radius_px),
                b, zbuf.data_ptr(), out.data_ptr(), what="splat")
    return out


def render_3d(parts, rho: torch.Tensor, dx: float, box: float, *, max_points: int = 1_000_000, width: int = 960,
              height: int = 960, eye=(1.3, -1.6, 1.0), radius_px: float = 1.0, lut=None) -> np.ndarray:
    """One 3-D frame of the viewer: subsample (ceil-division stride, viewer.py:189-191),
    density colours on the 4-decade window, discs; RGBA8 host image."""
    n = int(parts.n)
    stride = max(1, -(-n // max_points))
    m = len(range(0, n, stride))
    lut_t = torch.as_tensor(default_lut() if lut is None else lut, dtype=torch.float32, device="cuda")
    lo, inv = log_window(max(device_max(rho), 1e-30))
    pos = pack_positions(parts.pos_x, parts.pos_y, parts.pos_z, stride, 1.0 / box, m)
    col = density_color(parts.pos_x, parts.pos_y, parts.pos_z, rho, stride, m, 1.0 / dx, lut_t, lo, inv)
    img = splat(pos, col, look_at(eye, aspect=width / height), width, height, radius_px)
    return img.cpu().numpy()


def render_2d(img: torch.Tensor, *, lut=None) -> np.ndarray:
    """The 2-D view of a device projection image (img[a, b], viewer.py:276-284):
    RGBA8 host image with b up, as the window shows it."""
    lut_t = torch.as_tensor(default_lut() if lut is None else lut, dtype=torch.float32, device="cuda")
    lo, inv = log_window(max(device_max(img), 1e-30))
    rgb = colormap_log(img, lut_t, lo, inv).cpu().numpy()  # [a, b, 3]
    rgb = np.transpose(rgb, (1, 0, 2))[::-1]  # rows = b, top row = largest b
    out = np.empty(rgb.shape[:2] + (4,), np.uint8)
    out[..., :3] = (np.clip(rgb, 0, 1) * 255 + 0.5).astype(np.uint8)
    out[..., 3] = 255
    return out


def write_png(rgba: np.ndarray, path) -> Path:
    """RGBA8 (height, width, 4) array to a PNG file (zlib only)."""
    rgba = np.ascontiguousarray(rgba, dtype=np.uint8)
    h, w = rgba.shape[:2]
    raw = b"".join(b"\x00" + rgba[y].tobytes() for y in range(h))

    def chunk(tag, data):
        return struct.pack(">I", len(data)) + tag + data + struct.pack(">I", zlib.crc32(tag + data) & 0xFFFFFFFF)

    png = b"\x89PNG\r\n\x1a\n" + chunk(b"IHDR", struct.pack(">IIBBBBB", w, h, 8, 6, 0, 0, 0))
    png += chunk(b"IDAT", zlib.compress(raw, 6)) + chunk(b"IEND", b"")
    p = Path(path)
    p.write_bytes(png)
    return p


__all__ = ["LUT_N", "LOG_DECADES", "default_lut", "log_window", "device_max", "colormap_log", "pack_positions",
           "density_color", "look_at", "splat", "render_3d", "render_2d", "write_png"]
