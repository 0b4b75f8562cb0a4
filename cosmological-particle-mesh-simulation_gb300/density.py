"""Drop-in for density.py: CIC mass deposit on the GPU (deterministic, sorted)."""
from pmgpu import dropin


def density(positions, mass):
    """positions (3, Np) float32 -> grid (N_CELLS,)*3 float32 indexed [z, y, x]."""
    return dropin.density(positions, mass)
