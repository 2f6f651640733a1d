"""The particle-mesh force chain's grid<->particle stages on the GPU.

Drop-in for the reference module src/galaxy_collision/deposit.py: same function
names, arguments and node-centred convention (node (i,j,k) at (i,j,k)*dx;
out-of-box weight dropped, never wrapped). Each call is one launch of a
hand-written sm_103a kernel through ``libgcpm.so``:

* :func:`deposit_density` -- CIC deposit (deposit.py:47-82, 177-182). The
  reference's per-corner f32 contributions are summed in int64 fixed point, so
  rho is bit-identical run to run (the reference's f32 atomics are not).
* :func:`potential_to_accel` -- g = -grad(phi) (deposit.py:132-174, 204-207).
* :func:`gather_acceleration` -- CIC gather (deposit.py:85-129, 185-201).
* :func:`cell_keys` / :func:`sort_by_cell` -- the reference's cell index
  ``floor(x/dx)`` (deposit.py:62-67) as a sort key, and its stable sort.
"""

from __future__ import annotations

import torch

from galaxy_collision_gb300 import _native
from galaxy_collision_gb300._ops import DEFAULT_FIXED_POINT_BITS, op_context
from galaxy_collision_gb300.data import as_tensor


def _grid_size(f) -> int:
    t = f.tensor if hasattr(f, "tensor") else f
    shape = tuple(t.shape)
    if len(shape) != 3 or not (shape[0] == shape[1] == shape[2]):
        raise ValueError(f"grid fields must be cubic (G, G, G), got {shape}")
    return shape[0]


def _parts_arrays(parts):
    n = int(parts.n)
    xs = [as_tensor(getattr(parts, a), shape=(n,), name=f"parts.{a}") for a in ("pos_x", "pos_y", "pos_z")]
    return n, xs


def deposit_density(parts, rho, dx: float = 1.0, *, fixed_point_bits: int = DEFAULT_FIXED_POINT_BITS) -> None:
    """Deposit particle masses onto ``rho`` (mass/dx^3) by CIC. Zeroes ``rho`` first."""
    G = _grid_size(rho)
    r = as_tensor(rho, shape=(G, G, G), name="rho")
    n, (x, y, z) = _parts_arrays(parts)
    m = as_tensor(parts.mass, shape=(n,), name="parts.mass")
    ctx = op_context(G, dx)
    ctx.call("gc_deposit_cic", x.data_ptr(), y.data_ptr(), z.data_ptr(), m.data_ptr(), n, int(fixed_point_bits),
             r.data_ptr(), what="deposit_density")


def gather_acceleration(parts, ax_g, ay_g, az_g, acc_x, acc_y, acc_z, dx: float = 1.0) -> None:
    """CIC-interpolate the node acceleration field (``ax_g``..) to particles (``acc_x``..)."""
    G = _grid_size(ax_g)
    grids = [as_tensor(g, shape=(G, G, G), name=nm) for g, nm in ((ax_g, "ax_g"), (ay_g, "ay_g"), (az_g, "az_g"))]
    n, (x, y, z) = _parts_arrays(parts)
    outs = [as_tensor(a, shape=(n,), name=nm) for a, nm in ((acc_x, "acc_x"), (acc_y, "acc_y"), (acc_z, "acc_z"))]
    ctx = op_context(G, dx)
    ctx.call("gc_gather_accel", x.data_ptr(), y.data_ptr(), z.data_ptr(), n, *(g.data_ptr() for g in grids),
             *(o.data_ptr() for o in outs), what="gather_acceleration")


def potential_to_accel(phi, ax_g, ay_g, az_g, dx: float = 1.0) -> None:
    """Compute the node acceleration field g = -grad(phi) (the "grad" step)."""
    G = _grid_size(phi)
    p = as_tensor(phi, shape=(G, G, G), name="phi")
    outs = [as_tensor(g, shape=(G, G, G), name=nm) for g, nm in ((ax_g, "ax_g"), (ay_g, "ay_g"), (az_g, "az_g"))]
    ctx = op_context(G, dx)
    ctx.call("gc_potential_to_accel", p.data_ptr(), *(o.data_ptr() for o in outs), what="potential_to_accel")


def cell_keys(parts, grid_size: int, dx: float = 1.0) -> torch.Tensor:
    """uint32-valued (stored as int32) cell key per particle, the sentinel (G+1)^3 for no deposit."""
    n, (x, y, z) = _parts_arrays(parts)
    keys = torch.empty(n, dtype=torch.int32, device=x.device)
    ctx = op_context(grid_size, dx)
    ctx.call("gc_cell_keys", x.data_ptr(), y.data_ptr(), z.data_ptr(), n, keys.data_ptr(), what="cell_keys")
    return keys


def sort_keys(keys: torch.Tensor, grid_size: int, dx: float = 1.0):
    """Stable sort of 32-bit keys: returns (sorted_keys, perm) with perm[i] = source index."""
    k = as_tensor(keys, dtype=torch.int32, name="keys")
    n = k.numel()
    sk = torch.empty_like(k)
    perm = torch.empty_like(k)
    ctx = op_context(grid_size, dx)
    ctx.call("gc_sort_keys", k.data_ptr(), n, sk.data_ptr(), perm.data_ptr(), what="sort_keys")
    return sk, perm


__all__ = ["deposit_density", "gather_acceleration", "potential_to_accel", "cell_keys", "sort_keys"]
