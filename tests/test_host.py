"""Host-side checks that need no GPU: the C ABI library builds and exports every
symbol the header declares, configuration and IC generation match the reference."""
import ctypes
import os
import re
import shutil

import numpy as np
import pytest

from conftest import GOLDEN_CASES, ROOT, golden_config, load_golden, periodic_maxdiff

HEADER = os.path.join(ROOT, "include", "pm_gb300.h")


def declared_symbols():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(pm_[a-z0-9_]+)\s*\(", text)))


@pytest.fixture(scope="module")
def libpath():
    if shutil.which("nvcc") is None and not os.path.exists("/usr/local/cuda/bin/nvcc"):
        pytest.skip("nvcc not available")
    import pmgpu
    return pmgpu.build()


def test_library_exports_every_declared_symbol(libpath):
    lib = ctypes.CDLL(libpath)
    syms = declared_symbols()
    assert len(syms) >= 20
    missing = [s for s in syms if not hasattr(lib, s)]
    assert not missing, missing


def test_binding_covers_header():
    from pmgpu import _lib
    assert set(declared_symbols()) <= set(_lib.SIGNATURES)


def test_supported_sizes_and_cosmo_f(libpath):
    from pmgpu import _lib
    lib = _lib.load(libpath)
    for n in (16, 24, 32, 48, 64, 96, 128, 192, 256, 384, 512, 768, 1024):
        assert lib.pm_supported_n(n) == 1
    for n in (8, 20, 100, 2048, 40):
        assert lib.pm_supported_n(n) == 0
    from oracle import pm_oracle as O
    for a in (0.02, 0.5, 1.0):
        assert lib.pm_cosmo_f(a, 0.7, 0.7, 0.0) == pytest.approx(O.cosmo_f(a, [0.7, 0.7, 0.0]), rel=1e-15)


def test_ctx_create_rejects_bad_sizes(libpath):
    # argument validation happens before any CUDA call
    from pmgpu import _lib
    from pmgpu.config import Config
    lib = _lib.load(libpath)
    h = ctypes.c_void_p()
    rc = lib.pm_ctx_create(ctypes.byref(Config(n_cells=100).c_struct()), 0, ctypes.byref(h))
    assert rc == _lib.PM_ERR_ARG and not h.value


def test_config_from_module_and_step_count():
    import types
    from pmgpu.config import Config, step_count
    from oracle import pm_oracle as O
    m = types.SimpleNamespace(N_PARTS=64, N_CELLS=128, BOX_SIZE=100, STEPS=100, OMEGA_M0=0.31, H0=0.68,
                              A_INIT=0.01, A_END=1.0)
    cfg = Config.from_module(m)
    assert (cfg.n_parts, cfg.n_cells, cfg.box_size, cfg.steps) == (64, 128, 100, 100)
    assert cfg.mass == 8.0 and cfg.da == pytest.approx(0.0099)
    for a0, steps in ((0.02, 1000), (0.01, 100), (0.02, 200), (0.02, 500)):
        assert step_count(a0, 1.0, steps) == O.step_count(a0, 1.0, steps)


@pytest.mark.parametrize("name", GOLDEN_CASES)
def test_initial_conditions_match_reference(name):
    from pmgpu import ics
    f, c = load_golden(name)
    cfg = golden_config(c)
    grf = ics.gaussian_random_field(cfg)
    assert np.array_equal(grf, f["grf"])  # same random stream and arithmetic
    pos, vel = ics.zeldovich(f["grf"], cfg)
    assert periodic_maxdiff(pos, f["pos0"], cfg.n_cells) < 8 * np.spacing(np.float32(cfg.n_cells))
    assert np.abs(vel - f["vel0"]).max() < 1e-6 * np.abs(f["vel0"]).max()


# ---- the arithmetic the device initial conditions rely on (pm_ics.cu), checked on the host

PCG_MULT = 0x2360ED051FC65DA44385DF649FCCF645
M128 = (1 << 128) - 1


def pcg_advance(state, inc, delta):
    """Jump-ahead of the 128-bit LCG state' = state * M + inc by delta steps."""
    cur_mult, cur_plus, acc_mult, acc_plus = PCG_MULT, inc, 1, 0
    while delta > 0:
        if delta & 1:
            acc_mult = (acc_mult * cur_mult) & M128
            acc_plus = (acc_plus * cur_mult + cur_plus) & M128
        cur_plus = ((cur_mult + 1) * cur_plus) & M128
        cur_mult = (cur_mult * cur_mult) & M128
        delta >>= 1
    return (acc_mult * state + acc_plus) & M128


def xsl_rr(s):
    x = ((s >> 64) ^ s) & ((1 << 64) - 1)
    rot = s >> 122
    return ((x >> rot) | (x << ((64 - rot) & 63))) & ((1 << 64) - 1)


@pytest.mark.parametrize("seed", [0, 3, 38, 2 ** 31 - 5])
def test_pcg64_jump_matches_numpy_jitter_stream(seed):
    """Draw j of Generator(PCG64(seed)).uniform(-2, 2) = -2 + 4 * (xsl_rr(state after j + 1
    steps) >> 11) * 2^-53 -- the formula k_zeld_particles evaluates per particle."""
    from pmgpu.ics import jitter_state
    (sh, sl), (ih, il) = jitter_state(seed)
    state, inc = (sh << 64) | sl, (ih << 64) | il
    draws = np.random.Generator(np.random.PCG64(seed)).uniform(-2.0, 2.0, 5000)
    for j in (0, 1, 2, 7, 8, 9, 999, 4095, 4999):
        s = pcg_advance(state, inc, j)
        s = (s * PCG_MULT + inc) & M128
        val = -2.0 + 4.0 * ((xsl_rr(s) >> 11) * (1.0 / 9007199254740992.0))
        assert val == draws[j], (seed, j)


def test_uniform_pairs_feed_the_host_box_muller():
    from pmgpu import ics
    u, v = ics.uniform_pairs(8, 5)
    assert u.dtype == np.float32 and u.shape == (512,)
    s = u.astype(np.float64) ** 2 + v.astype(np.float64) ** 2
    assert np.all((s > 0) & (s < 1))
    f1, f2 = ics.gaussian_random_numbers(8, 5)
    t = -2 * np.log(u ** 2 + v ** 2) / (u ** 2 + v ** 2)
    assert np.allclose(f1.ravel(), u * t ** 0.5, rtol=1e-6)


def test_real_part_of_inverse_fft_is_inverse_rfft_of_hermitian_part():
    """Re(ifftn(X)) = irfftn of (X[k] + conj(X[-k])) / 2 on the half spectrum (the GRF fill)."""
    rng = np.random.default_rng(1)
    n = 12
    x = rng.standard_normal((n,) * 3) + 1j * rng.standard_normal((n,) * 3)
    neg = x[np.ix_(*[(-np.arange(n)) % n] * 3)]
    herm = 0.5 * (x + np.conj(neg))
    ref = np.fft.ifftn(x).real
    got = np.fft.irfftn(herm[:, :, : n // 2 + 1], s=(n,) * 3, axes=(0, 1, 2))
    assert np.allclose(got, ref, atol=1e-12)


@pytest.mark.parametrize("direction", [0, 1, 2])
def test_displacement_spectrum_drops_the_nyquist_plane(direction):
    """Re(ifftn(-i l_d pot_k)) of a real field = irfftn of i l_d rho_k / |l|^2 with the plane
    where axis `direction` is at the Nyquist index set to zero (k_zeld_spectrum)."""
    rng = np.random.default_rng(2)
    n = 8
    rho = rng.standard_normal((n,) * 3)
    ax = 2 * np.pi * np.fft.fftfreq(n)
    lz, ly, lx = np.meshgrid(ax, ax, ax, indexing="ij")
    l2 = lx ** 2 + ly ** 2 + lz ** 2
    rk = np.fft.fftn(rho)
    pot = np.zeros_like(rk)
    np.divide(rk, -l2, out=pot, where=l2 != 0)
    ld = (lz, ly, lx)[direction]
    ref = np.fft.ifftn(-1j * ld * pot).real
    half = np.fft.rfftn(rho)
    lh = [a[:, :, : n // 2 + 1] for a in (lz, ly, lx)]
    l2h = lh[0] ** 2 + lh[1] ** 2 + lh[2] ** 2
    g = np.zeros_like(l2h)
    np.divide(lh[direction], l2h, out=g, where=l2h != 0)
    idx = [slice(None)] * 3
    idx[direction] = n // 2
    g[tuple(idx)] = 0.0
    got = np.fft.irfftn(1j * g * half, s=(n,) * 3, axes=(0, 1, 2))
    assert np.allclose(got, ref, atol=1e-12)


def test_snapshot_units_and_file_roundtrip(tmp_path):
    """save_data.py:10-11 conversions and the dataset names; files read back unchanged."""
    from pmgpu.snapshot import host_snapshot, read_file, units, write_file
    up, uv = units(0.5, 250.0, 512, 0.7)
    assert up == 7.8 * (250.0 / (512 / 128)) / 10 ** 3
    assert uv == 0.781 * 250.0 * 0.7 / (0.5 * 512 / 128)
    rng = np.random.default_rng(0)
    pos = rng.uniform(0, 512, (3, 100)).astype(np.float32)
    vel = rng.standard_normal((3, 100)).astype(np.float32)
    d = host_snapshot(pos, vel, 0.5, 250.0, 512, 0.7)
    assert d["x2"].dtype == np.float32 and np.array_equal(d["x2"], pos[1] * up)
    path = str(tmp_path / "data.3.npz")
    write_file(path, d)
    back = read_file(path)
    assert set(back) == set(d) and all(np.array_equal(back[k], d[k]) for k in d)


# ---- index algebra of the shared-memory transforms (pm_fft.cuh), restated in numpy ----------
def _fft_plans():
    """The radix plans as pm_fft.cuh declares them (PM_PLAN(L, r0, r1, ...))."""
    src = open(os.path.join(ROOT, "cosmological-particle-mesh-simulation_gb300", "csrc", "pm_fft.cuh")).read()
    plans = {}
    for m in re.finditer(r"^PM_PLAN\((\d+),\s*([\d,\s]+)\)", src, re.M):
        plans[int(m.group(1))] = [int(x) for x in m.group(2).split(",")]
    return plans


def _stockham_pass(x, L, R, NS, inv, swap=False):
    """One pass as stockham_pass / stockham_pass_pairs index it: task j loads x[j + r L/R],
    twiddles by w^(r k L/(NS R)) (k = j mod NS), a radix-R DFT, stores at (j - k) R + k + r NS;
    with `swap` (stride-1 passes of 4-pair bundles) odd j store output r ^ 1 at step r."""
    NB = L // R
    y = np.empty_like(x)
    sgn = 1 if inv else -1
    dft = np.exp(sgn * 2j * np.pi * np.outer(np.arange(R), np.arange(R)) / R)
    for j in range(NB):
        k = j % NS
        v = x[j + NB * np.arange(R)].copy()
        if NS > 1:
            v[1:] *= np.exp(sgn * 2j * np.pi * (np.arange(1, R) * k * (L // (NS * R))) / L)
        out = dft @ v
        base = (j - k) * R + k
        for r in range(R):
            rr = r ^ 1 if (swap and NS == 1 and (j & 1)) else r
            y[base + rr * NS] = out[rr]
    return y


@pytest.mark.parametrize("L", sorted(_fft_plans()))
def test_stockham_plans_and_z_turn(L):
    """Each plan is a DFT; the z pass's turn (last forward pass, the Green multiply and the
    first pass of an inverse run on the reversed plan, all on one thread's registers) equals
    ifft(fft(x) g) L; the pair-swapped store order changes nothing but the order."""
    plan = _fft_plans()[L]
    assert int(np.prod(plan)) == L
    pairs = L % 3 != 0  # blocked_pairs(L): the pair passes, which may swap their store order
    rng = np.random.default_rng(L)
    x = rng.standard_normal(L) + 1j * rng.standard_normal(L)
    g = rng.standard_normal(L)
    y, NS = x, 1
    for R in plan:
        y = _stockham_pass(y, L, R, NS, False, swap=pairs)
        NS *= R
    assert np.allclose(y, np.fft.fft(x), atol=1e-9 * L)
    # the turn
    y, NS = x, 1
    for R in plan[:-1]:
        y = _stockham_pass(y, L, R, NS, False, swap=pairs)
        NS *= R
    R = plan[-1]
    NSL = L // R
    t = np.empty_like(y)
    for j in range(NSL):
        v = y[j + NSL * np.arange(R)].copy()
        if NSL > 1:
            v[1:] *= np.exp(-2j * np.pi * np.arange(1, R) * j / L)
        v = np.exp(-2j * np.pi * np.outer(np.arange(R), np.arange(R)) / R) @ v  # forward, last pass
        v *= g[j + NSL * np.arange(R)]                                            # the Green multiply
        v = np.exp(2j * np.pi * np.outer(np.arange(R), np.arange(R)) / R) @ v     # inverse, first pass
        t[j * R + np.arange(R)] = v
    y, NS = t, R
    for R2 in plan[-2::-1]:
        y = _stockham_pass(y, L, R2, NS, True, swap=pairs)
        NS *= R2
    assert np.allclose(y, np.fft.ifft(np.fft.fft(x) * g) * L, atol=1e-9 * L)
