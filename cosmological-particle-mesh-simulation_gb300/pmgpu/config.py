"""Simulation configuration: the constants of the reference's src/configure_me.py."""
from __future__ import annotations

import dataclasses

from ._lib import PM_FLAG_FIX_COSMO_F, PM_FLAG_KEEP_DENSITY, PM_FLAG_SPECTRAL_GRADIENT, PMConfigC


@dataclasses.dataclass
class Config:
    """Fields and meaning follow configure_me.py:7-40 (plot / save switches live in the
    driver, not here)."""

    n_parts: int = 256          # N_PARTS
    n_cells: int = 512          # N_CELLS
    box_size: float = 250.0     # BOX_SIZE [Mpc/h]
    random_seed: int = 0        # RANDOM_SEED
    steps: int = 1000           # STEPS
    power: float = 0.96         # POWER
    lcdm_transfer_function: bool = True  # LCDM_TRANSFER_FUNCTION
    omega_m0: float = 0.3       # OMEGA_M0
    omega_b0: float = 0.04      # OMEGA_B0
    omega_k0: float = 0.0       # OMEGA_K0
    omega_lambda0: float = 0.7  # OMEGA_LAMBDA0
    h0: float = 0.7             # H0
    a_init: float = 0.02        # A_INIT
    a_end: float = 1.0          # A_END
    fix_cosmo_f: bool = False   # evaluate f(a) with Omega_m in its slot (reference passes H0)
    keep_density: bool = False  # batch engine: keep the density grid apart from the potential
    spectral_gradient: bool = False  # drop-in step: force from -i sin(k) phi_k grids, not 32 taps

    @property
    def mass(self) -> float:
        """Particle mass in code units, pmesh.py:28."""
        return (self.n_cells / self.n_parts) ** 3

    @property
    def da(self) -> float:
        """pmesh.py:30."""
        return (self.a_end - self.a_init) / self.steps

    @property
    def np_total(self) -> int:
        return self.n_parts ** 3

    def c_struct(self) -> PMConfigC:
        flags = (PM_FLAG_FIX_COSMO_F if self.fix_cosmo_f else 0) | (
            PM_FLAG_KEEP_DENSITY if self.keep_density else 0) | (
            PM_FLAG_SPECTRAL_GRADIENT if self.spectral_gradient else 0)
        return PMConfigC(self.n_cells, self.n_parts, float(self.box_size), self.omega_m0, self.omega_b0,
                         self.omega_k0, self.omega_lambda0, self.h0, self.a_init, self.a_end, self.steps,
                         flags)

    @classmethod
    def from_module(cls, m) -> "Config":
        """Build from a configure_me-style module (upper-case constants)."""
        kw = {}
        for f in dataclasses.fields(cls):
            name = f.name.upper()
            if hasattr(m, name):
                kw[f.name] = getattr(m, name)
        return cls(**kw)


def step_count(a_init: float, a_end: float, steps: int) -> int:
    """Iterations of the driver loop ``while a < A_END - da: a += da`` (pmesh.py:56,63)."""
    da = (a_end - a_init) / steps
    a, n = a_init, 0
    while a < a_end - da:
        a += da
        n += 1
    return n
