"""Initial conditions: Gaussian random field + Zel'dovich displacement (host, numpy).

Follows src/gaussian_random_field.py:9-123 and src/zeldovich.py:10-100 of the
reference operation for operation (same random stream, same float32/float64 mix), with
three decisions that make the result well defined:

* entries that the reference computes with ``np.divide``/``np.power`` ``where=`` and no
  ``out=`` (k = 0; left uninitialised there) are 0;
* the Zel'dovich jitter (uniform in [-2, 2) cells, zeldovich.py:89-91), drawn from the
  unseeded stdlib ``random`` in the reference, is drawn from
  ``numpy.random.Generator(PCG64(seed))``: x-jitter, then y, then z;
* a polar Box-Muller pair whose float32 u^2 + v^2 rounds up to >= 1 (NaN or a negative
  square root in the reference's float32 expression) is evaluated in float64, clamped at 0.

This runs once per simulation and is not part of the per-step path.
"""
from __future__ import annotations

import numpy as np

try:  # multithreaded FFTs when scipy is present
    import scipy.fft as _sfft

    def _fftn(a):
        return _sfft.fftn(a, workers=-1)

    def _ifftn(a):
        return _sfft.ifftn(a, workers=-1)
except ImportError:  # pragma: no cover
    _fftn, _ifftn = np.fft.fftn, np.fft.ifftn

from .config import Config


def cosmo_H(a, h0, om, ol, ok):
    """cosmology.py:11-18."""
    return np.sqrt(h0 ** 2 * (om / a ** 3 + ok / a ** 2 + ol))


def cosmo_f(a, om, ol, ok):
    """cosmology.py:20-27."""
    return 1 / np.sqrt((om + ok * a + ol * a ** 3) / a)


def cosmo_Dt(a, om, ol, ok):
    """cosmology.py:29-36."""
    return 5 / 2 / om / (om ** (4 / 7) - ol + (1 + om / 2) * (1 + ol / 70)) * a


def uniform_pairs(n_parts: int, seed: int):
    """gaussian_random_field.py:35-50: the accepted (u, v) of the rejection loop, float32,
    flat (N_PARTS^3,) each, from numpy's RandomState(seed)."""
    rs = np.random.RandomState(seed)
    total = n_parts ** 3
    u = np.zeros(total, dtype=np.float32)
    v = np.zeros(total, dtype=np.float32)
    acc = 0
    while acc < total:
        u1 = rs.uniform(-1, 1, total - acc)
        v1 = rs.uniform(-1, 1, total - acc)
        sq = u1 ** 2 + v1 ** 2
        keep = np.nonzero((0. < sq) & (sq < 1.))
        u1, v1 = u1[keep], v1[keep]
        u[acc:acc + len(u1)] = u1
        v[acc:acc + len(v1)] = v1
        acc += len(u1)
    return u, v


def jitter_state(seed: int):
    """The 128-bit state and increment of numpy's PCG64(seed), the generator of the
    Zel'dovich jitter, as (high, low) 64-bit word pairs."""
    st = np.random.PCG64(seed).state["state"]
    m = (1 << 64) - 1
    return ((st["state"] >> 64) & m, st["state"] & m), ((st["inc"] >> 64) & m, st["inc"] & m)


def gaussian_random_numbers(n_parts: int, seed: int):
    """gaussian_random_field.py:31-63: rejection-sampled polar Box-Muller, float32."""
    u, v = uniform_pairs(n_parts, seed)
    s = u ** 2 + v ** 2
    shape = (n_parts,) * 3
    u, v, s = u.reshape(shape), v.reshape(shape), s.reshape(shape)
    with np.errstate(invalid="ignore", divide="ignore"):
        t = -2 * np.log(s) / s
    # float32 rounding can take u^2 + v^2 (< 1 in float64) to >= 1, making t <= 0 or NaN
    # (the reference computes the same float32 expression); those rare entries are
    # recomputed in float64 and clamped at 0
    bad = ~(t > 0)
    if bad.any():
        s64 = u[bad].astype(np.float64) ** 2 + v[bad].astype(np.float64) ** 2
        with np.errstate(invalid="ignore", divide="ignore"):
            t64 = -2.0 * np.log(s64) / s64
        t[bad] = np.where(np.isfinite(t64) & (t64 > 0), t64, 0.0).astype(np.float32)
    f1 = u * t ** 0.5
    f2 = v * t ** 0.5
    return f1, f2


def _kaxes(cfg: Config):
    scale = 2 * np.pi * cfg.n_parts / cfg.box_size
    return scale * np.fft.fftfreq(cfg.n_parts)


def power_spectrum(cfg: Config):
    """gaussian_random_field.py:65-123 (LCDM transfer function, power-law normalisation)."""
    ax = _kaxes(cfg)
    lz, ly, lx = np.meshgrid(ax, ax, ax, indexing="ij")
    k = np.sqrt(lx ** 2 + ly ** 2 + lz ** 2)
    del lx, ly, lz
    nz = k != 0
    if cfg.lcdm_transfer_function:
        gamma = cfg.omega_m0 * cfg.h0 * np.exp(-cfg.omega_b0 - cfg.omega_b0 / cfg.omega_m0)
        q = k / gamma
        factor1 = np.sqrt(1 + 3.89 * q + (16.1 * q) ** 2 + (5.46 * q) ** 3 + (6.71 * q) ** 4)
        factor2 = np.zeros_like(q)
        np.divide(np.log(1 + 2.34 * q) ** 2, (2.34 * q) ** 2, out=factor2, where=q != 0)
        lcdm = factor2 / factor1
    else:
        lcdm = 0.
    npix = cfg.n_parts ** 3
    sigma2 = 64 * cfg.h0 ** 2
    if cfg.power >= 0.:
        kp = np.zeros_like(k)
        np.power(k, cfg.power, out=kp, where=nz)
        if cfg.lcdm_transfer_function:
            summ = np.sum(kp * lcdm)
            amp = sigma2 * npix ** 2 / summ
            return amp * k ** cfg.power * lcdm
        summ = np.sum(kp)
        amp = sigma2 * npix ** 2 / summ
        return amp * k ** cfg.power
    kinv = np.zeros_like(k)
    np.power(k, -cfg.power, out=kinv, where=nz)
    div = np.zeros_like(k)
    np.divide(1, kinv, out=div, where=kinv != 0)
    amp = sigma2 * npix ** 2 / np.sum(div)
    return amp * div


def gaussian_random_field(cfg: Config) -> np.ndarray:
    """gaussian_random_field.py:9-29: float32 (N_PARTS,)*3 real density field."""
    d = cosmo_Dt(cfg.a_init, cfg.omega_m0, cfg.omega_lambda0, cfg.omega_k0)
    f1, f2 = gaussian_random_numbers(cfg.n_parts, cfg.random_seed)
    p = power_spectrum(cfg)
    amp = np.sqrt(p * d ** 2)
    rho_k = amp * f1 + 1j * (amp * f2)
    del p, amp, f1, f2
    return _ifftn(rho_k).real.astype("float32")


def zeldovich(density: np.ndarray, cfg: Config):
    """zeldovich.py:10-100: positions, velocities (3, N_PARTS^3) float32."""
    n = cfg.n_parts
    npart = n ** 3
    positions = np.zeros((3, npart), dtype=np.float32)
    velocities = np.zeros((3, npart), dtype=np.float32)
    dens_k = _fftn(density)
    ax = _kaxes(cfg)
    lz, ly, lx = np.meshgrid(ax, ax, ax, indexing="ij")
    del_sq = -(lx ** 2 + ly ** 2 + lz ** 2)
    del lx, ly, lz
    pot_k = np.zeros_like(dens_k)
    np.divide(dens_k, del_sq, out=pot_k, where=del_sq != 0)
    del dens_k, del_sq
    force_resolution = cfg.n_cells / cfg.box_size
    resolution = cfg.n_cells / cfg.n_parts
    lin = cosmo_Dt(cfg.a_init, cfg.omega_m0, cfg.omega_lambda0, cfg.omega_k0)
    h_0 = cosmo_H(cfg.a_init, cfg.h0, cfg.omega_m0, cfg.omega_lambda0, cfg.omega_k0)
    f_0 = cosmo_f(cfg.a_init, cfg.omega_m0, cfg.omega_lambda0, cfg.omega_k0)
    jitter = np.random.Generator(np.random.PCG64(cfg.random_seed)).uniform(-2.0, 2.0, 3 * npart)
    space = np.linspace(0, cfg.n_cells - resolution, n) + 0.5
    shape = (n, n, n)
    for direction in range(3):
        bshape = [1, 1, 1]
        bshape[direction] = n
        l_dir = ax.reshape(bshape)
        df_k = -1.j * l_dir * pot_k * resolution
        disp = _ifftn(df_k).reshape(npart).real * force_resolution
        del df_k
        lattice = np.broadcast_to(space.reshape(bshape), shape).reshape(npart)
        pos = lattice + lin * disp
        pos += jitter[direction * npart:(direction + 1) * npart]
        positions[direction] = pos % cfg.n_cells
        velocities[direction] = cfg.a_init * f_0 * h_0 * lin * disp
    return positions, velocities


def initial_conditions(cfg: Config):
    """GRF then Zel'dovich (pmesh.py:46-47)."""
    return zeldovich(gaussian_random_field(cfg), cfg)
