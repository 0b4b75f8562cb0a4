"""FP64 torch copy of the oracle's PM step, for full-size checks on a GPU.

TEST INFRASTRUCTURE ONLY (part of the oracle): used by tests/ to run the reference algorithm in
float64 at sizes the numpy oracle cannot reach (512^3 grids, 1000 steps).  It follows
oracle/pm_oracle.py function for function -- density (density.py:7-48), potential
(potential.py:7-29, FFTs in complex128), integrate (integrate.py:15-97) and the step
coefficients (integrate.py:11-13, cosmology.py:20-27) -- and is validated against it at
small sizes in tests/test_gpu_pk.py.  Positions are absolute float64 coordinates, as in the
reference (which stores them in float32).
"""
from __future__ import annotations

import math

import torch

from . import pm_oracle as O

CORNERS = O.CORNERS


def cic(pos, n):
    """Base cells (int64) and offsets (float64) of float64 positions wrapped into [0, n)."""
    p = torch.remainder(pos, float(n))
    fl = torch.floor(p)
    cells = fl.to(torch.int64) % n
    return cells, p - fl


def weights(d):
    dx, dy, dz = d
    tx, ty, tz = 1.0 - dx, 1.0 - dy, 1.0 - dz
    return [tx * ty * tz, dx * ty * tz, tx * dy * tz, tx * ty * dz, dx * dy * tz, dx * ty * dz, tx * dy * dz,
            dx * dy * dz]


def density(pos, mass, n):
    """density.py:7-48 in float64 (scatter-add)."""
    cells, d = cic(pos, n)
    w = weights(d)
    xc, yc, zc = cells
    grid = torch.zeros(n ** 3, dtype=torch.float64, device=pos.device)
    for k, (ox, oy, oz) in enumerate(CORNERS):
        idx = (((zc + oz) % n) * n + (yc + oy) % n) * n + (xc + ox) % n
        grid.index_add_(0, idx, w[k] * mass)
    return grid.view(n, n, n)


def green(n, device):
    """fourier_utils.py:5-16 on the rfft half spectrum (k = 0 -> 0), float64."""
    k = 2.0 * math.pi * torch.fft.fftfreq(n, dtype=torch.float64, device=device)
    s2 = torch.sin(k / 2.0) ** 2
    kx = torch.arange(n // 2 + 1, device=device)
    ksq = s2[:, None, None] + s2[None, :, None] + s2[kx][None, None, :]
    g = torch.where(ksq != 0, 1.0 / torch.where(ksq != 0, ksq, torch.ones_like(ksq)), torch.zeros_like(ksq))
    return g


def potential(rho, a, omega_m0, g=None):
    """potential.py:7-29: phi = IFFT(-3 Om/(8a) * G * FFT(rho)).real, float64."""
    n = rho.shape[0]
    if g is None:
        g = green(n, rho.device)
    rk = torch.fft.rfftn(rho)
    rk *= (-3.0 * omega_m0 / 8.0 / a) * g
    return torch.fft.irfftn(rk, s=rho.shape)


def integrate(pos, vel, a, f_a1, da, phi):
    """integrate.py:15-97 in float64; returns new (pos, vel)."""
    n = phi.shape[0]
    cells, d = cic(pos, n)
    w = weights(d)
    xc, yc, zc = cells
    flat = phi.reshape(-1)
    g = torch.zeros_like(vel)
    for axis in range(3):
        e = [0, 0, 0]
        e[axis] = 1
        acc = torch.zeros_like(vel[0])
        for k, (ox, oy, oz) in enumerate(CORNERS):
            im = (((zc + oz - e[2]) % n) * n + (yc + oy - e[1]) % n) * n + (xc + ox - e[0]) % n
            ip = (((zc + oz + e[2]) % n) * n + (yc + oy + e[1]) % n) * n + (xc + ox + e[0]) % n
            acc += w[k] * (flat[im] - flat[ip])
        g[axis] = acc / 2.0
    vel = vel + da * f_a1 * g
    pos = torch.remainder(pos + da * vel / (a + da) ** 2 * f_a1, float(n))
    return pos, vel


def run(pos, vel, cfg, nsteps, device="cuda"):
    """nsteps iterations of the pmesh.py:60-63 loop body from a = cfg.a_init, float64."""
    n = cfg.n_cells
    p = torch.as_tensor(pos, dtype=torch.float64, device=device)
    v = torch.as_tensor(vel, dtype=torch.float64, device=device)
    g = green(n, device)
    mass = cfg.mass
    a = cfg.a_init
    da = cfg.da
    slot = cfg.omega_m0 if cfg.fix_cosmo_f else cfg.h0
    for _ in range(nsteps):
        rho = density(p, mass, n)
        phi = potential(rho, a, cfg.omega_m0, g)
        del rho
        fa1 = O.cosmo_f(a + da, [slot, cfg.omega_lambda0, cfg.omega_k0])
        p, v = integrate(p, v, a, fa1, da, phi)
        del phi
        a += da
    return p, v, a


def power_spectrum(rho, box_size, nbins=None):
    """P(k) of delta = rho/mean - 1 on the GPU in float64, same estimator and bins as
    pm_oracle.power_spectrum (rfft half space, modes with 0 < kx < N/2 counted twice)."""
    rho = rho.to(torch.float64)
    n = rho.shape[0]
    delta = rho / rho.mean() - 1.0
    dk = torch.fft.rfftn(delta)
    p3 = (dk.real ** 2 + dk.imag ** 2) * (box_size ** 3) / float(n) ** 6
    m = torch.fft.fftfreq(n, dtype=torch.float64, device=rho.device) * n
    mx = torch.arange(n // 2 + 1, dtype=torch.float64, device=rho.device)
    mm = torch.sqrt(m[:, None, None] ** 2 + m[None, :, None] ** 2 + mx[None, None, :] ** 2)
    wgt = torch.full((n // 2 + 1,), 2.0, dtype=torch.float64, device=rho.device)
    wgt[0] = 1.0
    if n % 2 == 0:
        wgt[-1] = 1.0
    wgt = wgt.expand_as(mm)
    b = torch.floor(mm + 0.5).to(torch.int64)
    if nbins is None:
        nbins = n // 2 + 1
    sel = (b > 0) & (b < nbins)
    cnt = torch.bincount(b[sel], weights=wgt[sel], minlength=nbins)
    psum = torch.bincount(b[sel], weights=(p3 * wgt)[sel], minlength=nbins)
    ksum = torch.bincount(b[sel], weights=(mm * wgt)[sel], minlength=nbins)
    pk = psum / cnt
    kc = ksum / cnt * 2.0 * math.pi / box_size
    return kc[1:].cpu().numpy(), pk[1:].cpu().numpy(), cnt[1:].cpu().numpy()
