"""Snapshot I/O with the reference's layout (src/galaxy_collision/io.py:25-198).

A snapshot holds ``pos`` (N,3), ``vel`` (N,3), ``mass`` (N,), ``gid`` (N,) int32,
optional ``rho``/``phi`` grids (G,G,G), the metadata ``step``, ``time``, ``dx``
and a ``diagnostics`` dict. ``.npz`` files store the diagnostics with the
``diag__`` key prefix; ``.h5``/``.hdf5`` use h5py (attributes + a
``diagnostics`` group) when h5py is installed. Files written here read back in
the reference and vice versa.
"""

from __future__ import annotations

from dataclasses import dataclass, field
from pathlib import Path

import numpy as np

_PARTICLE_KEYS = ("pos", "vel", "mass", "gid")
_GRID_KEYS = ("rho", "phi")
_META_KEYS = ("step", "time", "dx")
_DIAG_PREFIX = "diag__"


@dataclass
class Snapshot:
    step: int
    time: float
    pos: np.ndarray
    vel: np.ndarray
    mass: np.ndarray
    gid: np.ndarray
    dx: float = 1.0
    rho: np.ndarray | None = None
    phi: np.ndarray | None = None
    diagnostics: dict[str, np.ndarray] = field(default_factory=dict)

    @property
    def n(self) -> int:
        return self.pos.shape[0]


def _np(f):
    if f is None:
        return None
    if hasattr(f, "to_numpy"):
        return f.to_numpy()
    if hasattr(f, "detach"):
        return f.detach().cpu().numpy()
    return np.asarray(f)


def snapshot_from_states(step, time, parts, grid=None, diagnostics=None, dx=1.0) -> Snapshot:
    """Pull a ParticleState (+ optional GridState) to the host (io.py:51-76)."""
    pos = np.stack([_np(parts.pos_x), _np(parts.pos_y), _np(parts.pos_z)], axis=1)
    vel = np.stack([_np(parts.vel_x), _np(parts.vel_y), _np(parts.vel_z)], axis=1)
    return Snapshot(step=int(step), time=float(time), pos=pos, vel=vel, mass=_np(parts.mass), gid=_np(parts.gid),
                    dx=float(dx), rho=_np(grid.rho) if grid is not None else None,
                    phi=_np(grid.phi) if grid is not None else None,
                    diagnostics={k: np.asarray(v) for k, v in (diagnostics or {}).items()})


def snapshot_from_engine(step, time, engine, diagnostics=None, with_phi: bool = True) -> Snapshot:
    """Snapshot of a synchronised :class:`~galaxy_collision_gb300.engine.PMEngine` in
    original particle order and physical coordinates (phi in the grid frame)."""
    pos, vel, mass, gid = engine.state_arrays(physical=True)
    return Snapshot(step=int(step), time=float(time), pos=pos.cpu().numpy().astype(np.float32),
                    vel=vel.cpu().numpy(), mass=mass.cpu().numpy(), gid=gid.cpu().numpy(), dx=float(engine.dx),
                    phi=engine.potential().cpu().numpy() if with_phi else None,
                    diagnostics={k: np.asarray(v) for k, v in (diagnostics or {}).items()})


def write_snapshot(snap: Snapshot, path: str | Path) -> Path:
    path = Path(path)
    path.parent.mkdir(parents=True, exist_ok=True)
    suffix = path.suffix.lower()
    if suffix in (".h5", ".hdf5"):
        _write_hdf5(snap, path)
    elif suffix == ".npz":
        _write_npz(snap, path)
    else:
        raise ValueError(f"unsupported snapshot extension {path.suffix!r} (use .h5/.hdf5/.npz)")
    return path


def read_snapshot(path: str | Path) -> Snapshot:
    path = Path(path)
    if not path.is_file():
        raise FileNotFoundError(f"snapshot not found: {path}")
    suffix = path.suffix.lower()
    if suffix in (".h5", ".hdf5"):
        return _read_hdf5(path)
    if suffix == ".npz":
        return _read_npz(path)
    raise ValueError(f"unsupported snapshot extension {path.suffix!r} (use .h5/.hdf5/.npz)")


def _write_npz(snap: Snapshot, path: Path) -> None:
    arrays = {"step": np.asarray(snap.step), "time": np.asarray(snap.time), "dx": np.asarray(snap.dx)}
    for key in _PARTICLE_KEYS:
        arrays[key] = getattr(snap, key)
    for key in _GRID_KEYS:
        arr = getattr(snap, key)
        if arr is not None:
            arrays[key] = arr
    for key, val in snap.diagnostics.items():
        arrays[_DIAG_PREFIX + key] = np.asarray(val)
    np.savez_compressed(path, **arrays)


def _read_npz(path: Path) -> Snapshot:
    with np.load(path) as data:
        diag = {k[len(_DIAG_PREFIX):]: np.asarray(data[k]) for k in data.files if k.startswith(_DIAG_PREFIX)}
        return Snapshot(step=int(data["step"]), time=float(data["time"]), pos=data["pos"], vel=data["vel"],
                        mass=data["mass"], gid=data["gid"], dx=float(data["dx"]),
                        rho=data["rho"] if "rho" in data.files else None,
                        phi=data["phi"] if "phi" in data.files else None, diagnostics=diag)


def _write_hdf5(snap: Snapshot, path: Path) -> None:
    try:
        import h5py
    except ImportError as e:  # pragma: no cover - depends on the environment
        raise RuntimeError("HDF5 snapshots need h5py, which is not installed; use .npz") from e
    with h5py.File(path, "w") as f:
        for key in _META_KEYS:
            f.attrs[key] = getattr(snap, key)
        for key in _PARTICLE_KEYS:
            f.create_dataset(key, data=getattr(snap, key), compression="gzip")
        for key in _GRID_KEYS:
            arr = getattr(snap, key)
            if arr is not None:
                f.create_dataset(key, data=arr, compression="gzip")
        if snap.diagnostics:
            grp = f.create_group("diagnostics")
            for key, val in snap.diagnostics.items():
                grp.create_dataset(key, data=np.asarray(val))


def _read_hdf5(path: Path) -> Snapshot:
    try:
        import h5py
    except ImportError as e:  # pragma: no cover
        raise RuntimeError("HDF5 snapshots need h5py, which is not installed; use .npz") from e
    with h5py.File(path, "r") as f:
        kw = {key: f.attrs[key] for key in _META_KEYS}
        for key in _PARTICLE_KEYS:
            kw[key] = f[key][()]
        for key in _GRID_KEYS:
            kw[key] = f[key][()] if key in f else None
        diag = {k: np.asarray(f["diagnostics"][k][()]) for k in f["diagnostics"]} if "diagnostics" in f else {}
    return Snapshot(step=int(kw["step"]), time=float(kw["time"]), pos=kw["pos"], vel=kw["vel"], mass=kw["mass"],
                    gid=kw["gid"], dx=float(kw["dx"]), rho=kw["rho"], phi=kw["phi"], diagnostics=diag)


__all__ = ["Snapshot", "snapshot_from_states", "snapshot_from_engine", "write_snapshot", "read_snapshot"]
