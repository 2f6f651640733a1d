"""Run configuration: the reference's ``SimConfig`` schema and YAML files.

Same fields, defaults, validation and error type as src/galaxy_collision/config.py:35-147
(``ConfigError`` is a ``ValueError``; unknown keys are rejected; exactly one of
``n_particles`` / ``particle_mass``). A few keys are added for the GPU engine,
all optional with defaults: ``box_lo`` (physical position of node 0; the
reference's box starts at 0), ``grav_constant`` (None = the reference's G),
``solver_tol``, ``solver_max_cycles``, ``fixed_point_bits`` and ``sort_every``.

PyYAML is optional: without it the loader reads the flat ``key: value  # comment``
subset that run configurations use (scalars only).
"""

from __future__ import annotations

from dataclasses import asdict, dataclass, fields
from pathlib import Path
from typing import Any

BACKENDS = ("cpu", "cuda", "metal")
SOLVERS = ("multigrid", "fft")
IC_PRESETS = ("hello", "two_galaxy_4v", "two_galaxy_2v", "plummer", "plummer_131k", "two_disk")
GALAXY_MASS_MSUN = 2.32e11


class ConfigError(ValueError):
    """Raised when a configuration is structurally or semantically invalid."""


@dataclass
class SimConfig:
    name: str = "hello-sim"
    backend: str = "cuda"
    n_particles: int | None = None
    particle_mass: float | None = None
    dt: float = 0.01
    steps: int = 1
    ic_preset: str = "hello"
    solver: str = "multigrid"
    grid_size: int = 256
    separation: float = 90.0
    impact_parameter: float = 0.0
    output_cadence: int = 0
    output_dir: str = "outputs"
    seed: int = 0
    # GPU-engine additions (optional)
    box_lo: float = 0.0
    dx: float = 1.0
    grav_constant: float | None = None
    solver_tol: float = 1e-6
    solver_max_cycles: int = 50
    fixed_point_bits: int = 52
    sort_every: int = 20

    def __post_init__(self) -> None:
        self.validate()

    def validate(self) -> None:
        if self.backend not in BACKENDS:
            raise ConfigError(f"backend must be one of {BACKENDS}, got {self.backend!r}")
        if self.solver not in SOLVERS:
            raise ConfigError(f"solver must be one of {SOLVERS}, got {self.solver!r}")
        if self.ic_preset not in IC_PRESETS:
            raise ConfigError(f"ic_preset must be one of {IC_PRESETS}, got {self.ic_preset!r}")
        if self.n_particles is not None and self.particle_mass is not None:
            raise ConfigError("set only one resolution knob: n_particles OR particle_mass, not both")
        if self.n_particles is not None and self.n_particles <= 0:
            raise ConfigError(f"n_particles must be positive, got {self.n_particles}")
        if self.particle_mass is not None and self.particle_mass <= 0:
            raise ConfigError(f"particle_mass must be positive, got {self.particle_mass}")
        if self.dt <= 0:
            raise ConfigError(f"dt must be positive, got {self.dt}")
        if self.steps < 0:
            raise ConfigError(f"steps must be non-negative, got {self.steps}")
        if self.grid_size <= 0:
            raise ConfigError(f"grid_size must be positive, got {self.grid_size}")
        if self.separation <= 0:
            raise ConfigError(f"separation must be positive, got {self.separation}")
        if self.impact_parameter < 0:
            raise ConfigError(f"impact_parameter must be non-negative, got {self.impact_parameter}")
        if self.output_cadence < 0:
            raise ConfigError(f"output_cadence must be non-negative, got {self.output_cadence}")
        if self.dx <= 0:
            raise ConfigError(f"dx must be positive, got {self.dx}")
        if not (0 < self.solver_tol < 1):
            raise ConfigError(f"solver_tol must be in (0, 1), got {self.solver_tol}")
        if not (24 <= self.fixed_point_bits <= 60):
            raise ConfigError(f"fixed_point_bits must be in [24, 60], got {self.fixed_point_bits}")

    def resolve_n_particles(self) -> int | None:
        if self.n_particles is not None:
            return self.n_particles
        if self.particle_mass is not None:
            return round(2 * GALAXY_MASS_MSUN / self.particle_mass)
        return None

    def to_dict(self) -> dict[str, Any]:
        return asdict(self)


def from_dict(data: dict[str, Any]) -> SimConfig:
    """Build a :class:`SimConfig` from a plain dict, rejecting unknown keys."""
    if not isinstance(data, dict):
        raise ConfigError(f"config must be a mapping, got {type(data).__name__}")
    known = {f.name for f in fields(SimConfig)}
    unknown = set(data) - known
    if unknown:
        raise ConfigError(f"unknown config keys: {sorted(unknown)}")
    return SimConfig(**data)


def _scalar(text: str):
    t = text.strip()
    if t in ("", "~", "null", "Null", "NULL", "None"):
        return None
    if t in ("true", "True", "TRUE", "yes", "on"):
        return True
    if t in ("false", "False", "FALSE", "no", "off"):
        return False
    if len(t) >= 2 and t[0] == t[-1] and t[0] in "'\"":
        return t[1:-1]
    try:
        return int(t)
    except ValueError:
        pass
    try:
        return float(t)
    except ValueError:
        return t


def parse_flat_yaml(text: str) -> dict[str, Any]:
    """The flat ``key: value  # comment`` subset of YAML used by run configs."""
    out: dict[str, Any] = {}
    for lineno, raw in enumerate(text.splitlines(), 1):
        line = raw
        # strip comments that are not inside quotes
        q = None
        for i, ch in enumerate(line):
            if ch in "'\"":
                q = None if q == ch else (ch if q is None else q)
            elif ch == "#" and q is None and (i == 0 or line[i - 1].isspace()):
                line = line[:i]
                break
        if not line.strip() or line.strip() == "---":
            continue
        if line[0].isspace() or ":" not in line:
            raise ConfigError(f"line {lineno}: only flat 'key: value' entries are supported: {raw!r}")
        key, val = line.split(":", 1)
        out[key.strip()] = _scalar(val)
    return out


def load_config(path: str | Path) -> SimConfig:
    """Load and validate a YAML run configuration from ``path``."""
    path = Path(path)
    if not path.is_file():
        raise ConfigError(f"config file not found: {path}")
    text = path.read_text(encoding="utf-8")
    try:
        import yaml  # type: ignore

        data = yaml.safe_load(text) or {}
    except ImportError:
        data = parse_flat_yaml(text)
    return from_dict(data)


def dump_config(config: SimConfig, path: str | Path) -> None:
    """Write a config as flat YAML (round-trips through :func:`load_config`)."""
    lines = []
    for k, v in config.to_dict().items():
        if v is None:
            s = "null"
        elif isinstance(v, bool):
            s = "true" if v else "false"
        elif isinstance(v, str):
            s = repr(v) if (":" in v or "#" in v or v.strip() != v or v == "") else v
        else:
            s = repr(v)
        lines.append(f"{k}: {s}")
    Path(path).write_text("\n".join(lines) + "\n", encoding="utf-8")


__all__ = ["SimConfig", "ConfigError", "load_config", "dump_config", "from_dict", "parse_flat_yaml", "BACKENDS",
           "SOLVERS", "IC_PRESETS"]
