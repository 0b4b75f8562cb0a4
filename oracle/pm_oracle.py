"""FP64 CPU oracle for the particle-mesh hot path.

TEST INFRASTRUCTURE ONLY.  This module is the oracle: only ``tests/``,
``__graft_entry__.smoke()`` and the ``cpu_baseline`` / ``--impl reference`` leg of
``bench.py`` may import it.  The product path (the CUDA library and its Python
host layer) never calls into it.

It restates, vectorised with numpy and in float64, the reference functions of
grkooij/Cosmological-Particle-Mesh-Simulation that make up one PM step:

* ``density``        -- src/density.py:7-48         (CIC mass deposit)
* ``fourier_grid``   -- src/fourier_utils.py:5-16    (discrete-Laplacian Green table)
* ``potential``      -- src/potential.py:7-29        (FFT Poisson solve)
* ``cosmo_f``        -- src/cosmology.py:20-27       (leapfrog coefficient f(a))
* ``integrate``      -- src/integrate.py:15-97       (CIC force gather, kick, drift)
* ``advance_time``   -- src/integrate.py:9-13
* ``step_count``     -- src/pmesh.py:30,56,63        (loop count of the driver)

plus the deterministic parts the GPU engine adds (cell keys in deposit-tile
order, the displacement representation of positions) and a matter power
spectrum estimator that the reference does not have.

Reference quirks and the decision taken for each (identical in the CUDA path):

* Q1 ``integrate.py:12`` passes ``[H0, OMEGA_LAMBDA0, OMEGA_K0]`` to ``f``, i.e. H0
  sits in the Omega_m slot.  Kept by default (``fix_cosmo_f=False``).
* Q2 ``fourier_utils.py:16`` leaves k=0 of the Green table uninitialised
  (``np.divide`` with ``where=`` and no ``out=``).  Defined as 0 (mean removed).
* Q3 ``density.py:17,37-47`` deposits with non-atomic ``+=`` inside ``prange``.
  The oracle deposits serially in float64.
* Q4 A float32 position can equal ``N`` exactly after ``% N`` in float64
  (``integrate.py:95``, ``zeldovich.py:93``).  The reference then gets
  ``x_c = 0, d = N``.  Positions are canonicalised (``x >= N -> x - N``) before
  the cell and weights are formed; ``canonical=False`` reproduces the reference.
* Q5 the Zel'dovich jitter (``zeldovich.py:89-91``) uses the unseeded stdlib
  ``random``; the IC generator used with this oracle draws it from a seeded PCG64.
* Q6 the driver loop ``while a < A_END - da`` runs a float-accumulated count of
  steps; ``step_count`` reproduces it exactly.
"""
from __future__ import annotations

import math

import numpy as np

# Deposit tile shape shared with the CUDA engine: a tile is TZ x TY full x-rows.
TILE_Y = 4
TILE_Z = 4


# --------------------------------------------------------------------------------------
# cosmology.py
# --------------------------------------------------------------------------------------
def cosmo_H(a, h0, cosmology):
    """cosmology.py:11-18."""
    om, ol, ok = cosmology
    return np.sqrt(h0 ** 2 * (om / a ** 3 + ok / a ** 2 + ol))


def cosmo_f(a, cosmology):
    """cosmology.py:20-27: 1/sqrt((om + ok a + ol a^3)/a)."""
    om, ol, ok = cosmology
    return 1.0 / math.sqrt((om + ok * a + ol * a ** 3) / a)


def cosmo_Dt(a, cosmology):
    """cosmology.py:29-36 (growth-factor approximation)."""
    om, ol, ok = cosmology
    return 5.0 / 2.0 / om / (om ** (4.0 / 7.0) - ol + (1.0 + om / 2.0) * (1.0 + ol / 70.0)) * a


def step_coefficients(a, da, omega_m0, omega_lambda0, omega_k0, h0, fix_cosmo_f=False):
    """integrate.py:11-13 and :94-95.

    Returns (green, kick, drift) with green = -3*Om/(8a) (potential.py:15, without the
    1/N^3 of the inverse FFT), kick = da*f(a+da) and drift = da*f(a+da)/(a+da)^2.
    With ``fix_cosmo_f=False`` f is evaluated with H0 in the Omega_m slot (Q1).
    """
    cos = [omega_m0 if fix_cosmo_f else h0, omega_lambda0, omega_k0]
    fa1 = cosmo_f(a + da, cos)
    green = -3.0 * omega_m0 / 8.0 / a
    return green, da * fa1, da / (a + da) ** 2 * fa1


def step_count(a_init, a_end, steps):
    """pmesh.py:30,56,63: number of iterations of ``while a < A_END - da: a += da``."""
    da = (a_end - a_init) / steps
    a = a_init
    n = 0
    while a < a_end - da:
        a += da
        n += 1
    return n


# --------------------------------------------------------------------------------------
# cells, weights, keys
# --------------------------------------------------------------------------------------
def canonicalise(x, n):
    """Q4: map float32 positions into [0, n) (x == n -> 0).  Exact in float32."""
    x = np.asarray(x, dtype=np.float32)
    x = np.where(x >= n, x - np.float32(n), x)
    x = np.where(x < 0, x + np.float32(n), x)
    return x.astype(np.float32)


def cic_cells(positions, n, canonical=True):
    """Base cell and offsets per axis.

    density.py:19-30 / integrate.py:20,36-38: ``x_c = floor(x) % N``, ``d = x - x_c``.
    Returns (cells int64 (3,Np), d float64 (3,Np)).  With ``canonical`` (default) the
    positions are first mapped into [0, N) (Q4), so ``d`` is in [0, 1).
    """
    p = np.asarray(positions, dtype=np.float32)
    if canonical:
        p = canonicalise(p, n)
    fl = np.floor(p.astype(np.float64))
    cells = fl.astype(np.int64) % n
    d = p.astype(np.float64) - cells
    return cells, d


def cic_weights(d):
    """integrate.py:27-52: the 8 weights ordered [ttt, dtt, tdt, ttd, ddt, dtd, tdd, ddd]."""
    dx, dy, dz = d
    tx, ty, tz = 1.0 - dx, 1.0 - dy, 1.0 - dz
    return np.stack([tx * ty * tz, dx * ty * tz, tx * dy * tz, tx * ty * dz,
                     dx * dy * tz, dx * ty * dz, tx * dy * dz, dx * dy * dz])


# corner offsets (ox, oy, oz) in the weight order above
CORNERS = [(0, 0, 0), (1, 0, 0), (0, 1, 0), (0, 0, 1), (1, 1, 0), (1, 0, 1), (0, 1, 1), (1, 1, 1)]


def row_index(y, z, n, ty=TILE_Y, tz=TILE_Z):
    """Deposit-tile-major row number of the x-row (y, z).

    Tiles are ``tz`` planes x ``ty`` rows of full x-rows, numbered z-major; rows inside a
    tile are numbered ``(z % tz) * ty + (y % ty)``.
    """
    y = np.asarray(y, dtype=np.int64)
    z = np.asarray(z, dtype=np.int64)
    tile = (z // tz) * (n // ty) + (y // ty)
    return tile * (tz * ty) + (z % tz) * ty + (y % ty)


def key_xbits(n):
    """Bits reserved for x in a cell key: ceil(log2(n))."""
    return max(1, int(math.ceil(math.log2(n))))


def cell_keys(positions, n, row_base=0, xbits=None, canonical=True):
    """Sort key of each particle: ``(row_base + row_index(y_c, z_c)) << xbits | x_c``.

    The key orders cells x-fastest inside an x-row and rows in deposit-tile order; the
    cells are those of density.py:19-21.
    """
    if xbits is None:
        xbits = key_xbits(n)
    cells, _ = cic_cells(positions, n, canonical)
    r = row_index(cells[1], cells[2], n) + row_base
    return ((r << xbits) | cells[0]).astype(np.uint64)


# --------------------------------------------------------------------------------------
# density.py
# --------------------------------------------------------------------------------------
def density(positions, mass, n, canonical=True):
    """density.py:7-48, serial float64 CIC deposit onto grid[z, y, x] (float64)."""
    cells, d = cic_cells(positions, n, canonical)
    w = cic_weights(d) * float(mass)
    xc, yc, zc = cells
    grid = np.zeros(n * n * n, dtype=np.float64)
    for c, (ox, oy, oz) in enumerate(CORNERS):
        idx = (((zc + oz) % n) * n + (yc + oy) % n) * n + (xc + ox) % n
        grid += np.bincount(idx, weights=w[c], minlength=n ** 3)
    return grid.reshape(n, n, n)


# --------------------------------------------------------------------------------------
# fourier_utils.py / potential.py
# --------------------------------------------------------------------------------------
def fourier_grid(n):
    """fourier_utils.py:5-16 in float64, with the k=0 entry defined as 0 (Q2)."""
    k = 2.0 * np.pi * np.fft.fftfreq(n)
    s2 = np.sin(k / 2.0) ** 2
    ksq = s2[:, None, None] + s2[None, :, None] + s2[None, None, :]
    out = np.zeros_like(ksq)
    np.divide(1.0, ksq, out=out, where=ksq != 0)
    return out


def potential(density, fgrid, a, omega_m0, workers=None):
    """potential.py:7-29: complex128 forward FFT, x(-3 Om/(8a) fgrid), normalised
    backward FFT, real part.  ``workers`` threads the FFTs through scipy.fft (the
    reference threads FFTW with N_CPU)."""
    if workers:
        import scipy.fft as sfft
        fftn = lambda x: sfft.fftn(x, workers=workers)  # noqa: E731
        ifftn = lambda x: sfft.ifftn(x, workers=workers)  # noqa: E731
    else:
        fftn, ifftn = np.fft.fftn, np.fft.ifftn
    rho_k = fftn(np.asarray(density, dtype=np.complex128))
    phi_k = -3.0 * omega_m0 / 8.0 / a * np.asarray(fgrid, dtype=np.float64) * rho_k
    del rho_k
    return ifftn(phi_k).real


# --------------------------------------------------------------------------------------
# integrate.py
# --------------------------------------------------------------------------------------
def gather_gradient(phi, cells, d):
    """integrate.py:54-92: the CIC-interpolated central-difference gradient per axis.

    For axis ``a`` and corner ``o`` the reference forms
    ``phi[c + o - e_a] - phi[c + o + e_a]`` and sums ``t_o * g_o / 2``.
    Returns g (3, Np) float64.
    """
    n = phi.shape[0]
    ph = np.asarray(phi, dtype=np.float64)
    w = cic_weights(d)
    xc, yc, zc = cells
    g = np.zeros((3, xc.size), dtype=np.float64)
    for axis in range(3):
        e = [0, 0, 0]
        e[axis] = 1
        acc = np.zeros(xc.size, dtype=np.float64)
        for c, (ox, oy, oz) in enumerate(CORNERS):
            xm, ym, zm = (xc + ox - e[0]) % n, (yc + oy - e[1]) % n, (zc + oz - e[2]) % n
            xp, yp, zp = (xc + ox + e[0]) % n, (yc + oy + e[1]) % n, (zc + oz + e[2]) % n
            acc += w[c] * (ph[zm, ym, xm] - ph[zp, yp, xp])
        g[axis] = acc / 2.0
    return g


def integrate(positions, velocities, a_val, f_a1, da, phi, canonical=True):
    """integrate.py:15-97 in float64.  Returns new (positions, velocities) as float64.

    Cell centres and weights come from the positions before the step (integrate.py:20-21)
    and are shared by the three sweeps; each sweep kicks then drifts its axis
    (integrate.py:94-95) and wraps into [0, N).
    """
    n = phi.shape[0]
    cells, d = cic_cells(positions, n, canonical)
    g = gather_gradient(phi, cells, d)
    v = np.asarray(velocities, dtype=np.float64) + da * f_a1 * g
    x = np.asarray(positions, dtype=np.float32).astype(np.float64)
    x = np.mod(x + da * v / (a_val + da) ** 2 * f_a1, n)
    return x, v


def advance_time(density, positions, velocities, fgrid, a, da, omega_m0, omega_lambda0,
                 omega_k0, h0, fix_cosmo_f=False, canonical=True, workers=None):
    """integrate.py:9-13."""
    phi = potential(density, fgrid, a, omega_m0, workers=workers)
    cos = [omega_m0 if fix_cosmo_f else h0, omega_lambda0, omega_k0]
    fa1 = cosmo_f(a + da, cos)
    return integrate(positions, velocities, a, fa1, da, phi, canonical)


# --------------------------------------------------------------------------------------
# displacement representation (GPU resident engine): x = q(lattice) + d
# --------------------------------------------------------------------------------------
def lattice_q(np1, n):
    """zeldovich.py:79-83: lattice coordinate of particle index i along one axis,
    ``i * (N_CELLS/N_PARTS) + 0.5``, split into integer and float32 fractional part."""
    r = n / np1
    q = np.arange(np1, dtype=np.float64) * r + 0.5
    qi = np.floor(q).astype(np.int64)
    qf = (q - qi).astype(np.float32)
    return qi, qf


def particle_axes(np1):
    """Particle index -> (ix, iy, iz): zeldovich.py:83 meshgrid('ij') + C-order reshape."""
    i = np.arange(np1 ** 3, dtype=np.int64)
    return i // (np1 * np1), (i // np1) % np1, i % np1


def disp_cells(disp, ids, np1, n):
    """Cell and in-cell offset of displacement-stored particles.

    Per axis: ``cell = (q_int + floor(q_frac + d)) mod N`` and
    ``f = (q_frac + d) - floor(q_frac + d)`` with ``q_frac + d`` rounded to float32 --
    the formula of the CUDA engine (keys bit-exact).
    """
    qi, qf = lattice_q(np1, n)
    ids = np.asarray(ids, dtype=np.int64)
    axes = [ids // (np1 * np1), (ids // np1) % np1, ids % np1]
    cells = np.empty((3, ids.size), dtype=np.int64)
    frac = np.empty((3, ids.size), dtype=np.float64)
    for a in range(3):
        s = (qf[axes[a]] + np.asarray(disp[a], dtype=np.float32)).astype(np.float32)
        fl = np.floor(s)
        cells[a] = (qi[axes[a]] + fl.astype(np.int64)) % n
        frac[a] = (s - fl).astype(np.float32)
    return cells, frac


# --------------------------------------------------------------------------------------
# matter power spectrum (not in the reference)
# --------------------------------------------------------------------------------------
def power_spectrum(rho, box_size, nbins=None):
    """Shell-averaged P(k) of delta = rho/mean(rho) - 1 (float64).

    Bins are integer shells of width k_f = 2 pi / box in |m| (mode index); returns
    (k_centres [h/Mpc], P(k) [(Mpc/h)^3], modes per bin).  rfft half-space modes with
    0 < kx < N/2 count twice.  No CIC window correction: compared spectra are taken
    with the same estimator on the same kind of grid.
    """
    rho = np.asarray(rho, dtype=np.float64)
    n = rho.shape[0]
    delta = rho / rho.mean() - 1.0
    dk = np.fft.rfftn(delta)
    p3 = (np.abs(dk) ** 2) * (box_size ** 3) / float(n) ** 6
    m = np.fft.fftfreq(n) * n
    mx = np.arange(n // 2 + 1, dtype=np.float64)
    mm = np.sqrt(m[:, None, None] ** 2 + m[None, :, None] ** 2 + mx[None, None, :] ** 2)
    weight = np.full(n // 2 + 1, 2.0)
    weight[0] = 1.0
    if n % 2 == 0:
        weight[-1] = 1.0
    wgt = np.broadcast_to(weight[None, None, :], mm.shape)
    b = np.floor(mm + 0.5).astype(np.int64)
    if nbins is None:
        nbins = n // 2 + 1
    sel = (b > 0) & (b < nbins)
    cnt = np.bincount(b[sel], weights=wgt[sel], minlength=nbins)
    psum = np.bincount(b[sel], weights=(p3 * wgt)[sel], minlength=nbins)
    ksum = np.bincount(b[sel], weights=(mm * wgt)[sel], minlength=nbins)
    with np.errstate(invalid="ignore", divide="ignore"):
        pk = psum / cnt
        kc = ksum / cnt * 2.0 * np.pi / box_size
    return kc[1:], pk[1:], cnt[1:]
