"""Drop-in for zeldovich.py (host numpy, runs once per simulation)."""
from pmgpu import ics
from pmgpu.dropin import config


def zeldovich(density):
    """Lattice + Zel'dovich displacement (+ seeded +-2 cell jitter): positions, velocities (3, N_PARTS^3)."""
    return ics.zeldovich(density, config())
