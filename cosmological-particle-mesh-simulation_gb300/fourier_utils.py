"""Drop-in for fourier_utils.py."""
from pmgpu import dropin


def fourier_grid():
    """1 / sum_i sin^2(k_i / 2) on the N_CELLS^3 grid, k = 2 pi fftfreq(N_CELLS); k = 0 -> 0."""
    return dropin.fourier_grid()
