"""Drop-in for potential.py: FFT Poisson solve on the GPU."""
from pmgpu import dropin


def potential(density, fgrid, a):
    """phi = IFFT(-3 OMEGA_M0 / (8 a) * fgrid * FFT(density)).real"""
    return dropin.potential(density, fgrid, a)
