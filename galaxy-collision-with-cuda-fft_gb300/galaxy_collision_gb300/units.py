"""Internal units (kpc, Myr, M_sun) and the gravitational constant.

Same unit system as the reference (src/galaxy_collision/units.py:23-46): G is
derived from G = 4.30091e-3 pc (km/s)^2 / M_sun, giving ~4.498e-12
kpc^3 M_sun^-1 Myr^-2. The configurations of this package's benchmark use G = 1
model units instead and pass ``grav_constant`` explicitly.
"""

from __future__ import annotations

M_PER_PC = 3.0856775814913673e16
PC_PER_KPC = 1.0e3
M_PER_KPC = M_PER_PC * PC_PER_KPC
KM_PER_KPC = M_PER_KPC * 1.0e-3
S_PER_MYR = 365.25 * 86400.0 * 1.0e6
KMS_PER_KPC_PER_MYR = KM_PER_KPC / S_PER_MYR
G_STANDARD_PC_KMS = 4.30091e-3

G = G_STANDARD_PC_KMS / PC_PER_KPC / KMS_PER_KPC_PER_MYR**2
"""Gravitational constant in kpc^3 M_sun^-1 Myr^-2."""


def kms_to_kpc_per_myr(v_kms: float) -> float:
    return v_kms / KMS_PER_KPC_PER_MYR


def kpc_per_myr_to_kms(v: float) -> float:
    return v * KMS_PER_KPC_PER_MYR
