"""Particle and grid state on the device, with the reference's field interface.

The reference keeps its state in Taichi fields (src/galaxy_collision/data.py:84-138)
and its functions only use ``.shape``, ``.to_numpy()``, ``.from_numpy()``,
``.fill()`` and element indexing. :class:`Field` provides exactly that over a
contiguous CUDA tensor, so code written against the reference's
``ParticleState``/``GridState`` runs unchanged. Every operator of this package
also accepts a plain ``torch.Tensor``.
"""

from __future__ import annotations

from dataclasses import dataclass

import numpy as np
import torch

BYTES_PER_PARTICLE = 32  # pos(3) + vel(3) + mass f32, gid i32 (data.py:21)
_GRID_FIELDS = 2 + 3 + 3.0 * 8.0 / 7.0  # rho, phi, accel(3), hierarchy (data.py:30-33)


@dataclass(frozen=True)
class MemoryEstimate:
    n_particles: int
    grid_size: int
    particle_bytes: int
    grid_bytes: int

    @property
    def total_bytes(self) -> int:
        return self.particle_bytes + self.grid_bytes

    @property
    def total_gb(self) -> float:
        return self.total_bytes / 1e9

    def summary(self) -> str:
        return (
            f"N={self.n_particles:,} particles, grid={self.grid_size}^3 | "
            f"particles {self.particle_bytes / 1e9:.2f} GB + grid {self.grid_bytes / 1e9:.2f} GB = "
            f"{self.total_gb:.2f} GB"
        )


def estimate_memory(n_particles: int, grid_size: int = 256) -> MemoryEstimate:
    """SoA memory footprint of the production path (reference data.py:61-81)."""
    if n_particles <= 0:
        raise ValueError(f"n_particles must be positive, got {n_particles}")
    if grid_size <= 0:
        raise ValueError(f"grid_size must be positive, got {grid_size}")
    return MemoryEstimate(n_particles, grid_size, n_particles * BYTES_PER_PARTICLE,
                          int(_GRID_FIELDS * grid_size**3 * 4))


def _device() -> torch.device:
    if not torch.cuda.is_available():
        raise RuntimeError("galaxy_collision_gb300 needs a CUDA device")
    return torch.device("cuda", torch.cuda.current_device())


class Field:
    """A contiguous device array with the Taichi-field methods the reference uses."""

    __slots__ = ("tensor",)

    def __init__(self, shape, dtype=torch.float32, tensor: torch.Tensor | None = None):
        if tensor is None:
            tensor = torch.zeros(tuple(shape) if not isinstance(shape, int) else (shape,), dtype=dtype,
                                 device=_device())
        self.tensor = tensor

    @property
    def shape(self):
        return tuple(self.tensor.shape)

    @property
    def dtype(self):
        return self.tensor.dtype

    def to_numpy(self) -> np.ndarray:
        return self.tensor.detach().cpu().numpy()

    def from_numpy(self, arr) -> None:
        a = np.ascontiguousarray(arr)
        if tuple(a.shape) != self.shape:
            raise ValueError(f"shape mismatch: field {self.shape}, array {a.shape}")
        src = torch.from_numpy(a).to(self.tensor.dtype)
        self.tensor.copy_(src.to(self.tensor.device, non_blocking=False))

    def fill(self, value) -> None:
        self.tensor.fill_(value)

    def data_ptr(self) -> int:
        return self.tensor.data_ptr()

    def __getitem__(self, idx):
        if idx is None:
            return self.tensor.item()
        return self.tensor[idx].item()

    def __setitem__(self, idx, value) -> None:
        self.tensor[idx] = value


def as_tensor(f, dtype=torch.float32, shape=None, name: str = "array") -> torch.Tensor:
    """Validate and unwrap a Field/Tensor argument: CUDA, contiguous, given dtype."""
    t = f.tensor if isinstance(f, Field) else f
    if not isinstance(t, torch.Tensor):
        raise TypeError(f"{name}: expected a Field or a CUDA torch.Tensor, got {type(f).__name__}")
    if not t.is_cuda:
        raise ValueError(f"{name}: tensor must be on a CUDA device")
    if t.dtype != dtype:
        raise ValueError(f"{name}: dtype must be {dtype}, got {t.dtype}")
    if not t.is_contiguous():
        raise ValueError(f"{name}: tensor must be contiguous")
    if shape is not None and tuple(t.shape) != tuple(shape):
        raise ValueError(f"{name}: shape must be {tuple(shape)}, got {tuple(t.shape)}")
    return t


class ParticleState:
    """SoA particle fields (reference data.py:84-113): pos, vel, mass f32; gid i32."""

    def __init__(self, n: int):
        if n <= 0:
            raise ValueError(f"particle count must be positive, got {n}")
        self.n = int(n)
        self.pos_x = Field(n)
        self.pos_y = Field(n)
        self.pos_z = Field(n)
        self.vel_x = Field(n)
        self.vel_y = Field(n)
        self.vel_z = Field(n)
        self.mass = Field(n)
        self.gid = Field(n, dtype=torch.int32)

    def fields(self):
        return (self.pos_x, self.pos_y, self.pos_z, self.vel_x, self.vel_y, self.vel_z, self.mass, self.gid)


class GridState:
    """SoA grid fields (reference data.py:116-138): rho, phi and g = -grad(phi)."""

    def __init__(self, grid_size: int = 256):
        if grid_size <= 0:
            raise ValueError(f"grid_size must be positive, got {grid_size}")
        self.grid_size = int(grid_size)
        shape = (grid_size,) * 3
        self.rho = Field(shape)
        self.phi = Field(shape)
        self.ax = Field(shape)
        self.ay = Field(shape)
        self.az = Field(shape)


__all__ = ["BYTES_PER_PARTICLE", "MemoryEstimate", "estimate_memory", "Field", "as_tensor", "ParticleState",
           "GridState"]
