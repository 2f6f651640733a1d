"""Device 2-D density projection (drop-in for src/galaxy_collision/viz/project.py).

Mass is binned nearest-bin into a ``(bins, bins)`` device image over two
in-plane axes (``gc_project_ngp``); only that image crosses to the host. Same
conventions as the reference: ``img[ia, ib]`` is mass per bin, ``extent =
(a_lo, a_hi, b_lo, b_hi)``, :func:`project_density` returns the surface density
transposed for ``imshow(origin="lower")``.
"""

from __future__ import annotations

import numpy as np

from galaxy_collision_gb300._ops import op_context
from galaxy_collision_gb300.data import as_tensor

_AXIS = {0: "pos_x", 1: "pos_y", 2: "pos_z"}


def scatter_density(parts, img, extent, axes=(0, 1)) -> tuple[float, float]:
    """Fill the device image ``img`` with mass per bin; returns the bin widths."""
    a, b = axes
    t = img.tensor if hasattr(img, "tensor") else img
    bins = int(t.shape[0])
    out = as_tensor(img, shape=(bins, bins), name="img")
    lo_a, hi_a, lo_b, hi_b = (float(v) for v in extent)
    bw_a = (hi_a - lo_a) / bins
    bw_b = (hi_b - lo_b) / bins
    n = int(parts.n)
    pa = as_tensor(getattr(parts, _AXIS[a]), shape=(n,), name=_AXIS[a])
    pb = as_tensor(getattr(parts, _AXIS[b]), shape=(n,), name=_AXIS[b])
    m = as_tensor(parts.mass, shape=(n,), name="mass")
    op_context(2, 1.0).call("gc_project_ngp", pa.data_ptr(), pb.data_ptr(), m.data_ptr(), n, lo_a, lo_b, bw_a, bw_b,
                            bins, out.data_ptr(), what="project")
    return bw_a, bw_b


def project_density(parts, img, extent, axes=(0, 1)) -> np.ndarray:
    """Surface density of the projection, oriented for ``imshow(origin='lower')``."""
    bw_a, bw_b = scatter_density(parts, img, extent, axes)
    t = img.tensor if hasattr(img, "tensor") else img
    return t.detach().cpu().numpy().T / (bw_a * bw_b)


__all__ = ["scatter_density", "project_density"]
