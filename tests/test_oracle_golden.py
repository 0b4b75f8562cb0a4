"""Pin the FP64 oracle against the reference's own outputs (golden fixtures made by
running the reference source, see tests/golden/make_golden.py).  CPU only."""
import numpy as np
import pytest

from conftest import COMPACT_CASES, GOLDEN_CASES, load_golden, periodic_maxdiff, rel_l2
from oracle import pm_oracle as O


@pytest.mark.parametrize("name", GOLDEN_CASES)
def test_density_matches_reference(name):
    f, c = load_golden(name)
    n = c["N_CELLS"]
    mass = (n / c["N_PARTS"]) ** 3
    for s in range(c["steps"]):
        rho = O.density(f[f"pos{s}"], mass, n)
        # the reference accumulates in float32: agreement to float32 rounding
        assert rel_l2(rho, f[f"rho{s}"]) < 1e-6
        assert abs(rho.sum() - mass * c["N_PARTS"] ** 3) < 1e-6 * mass * c["N_PARTS"] ** 3


@pytest.mark.parametrize("name", ["n8_g16", "n12_g24"])
def test_fourier_grid_matches_reference(name):
    f, c = load_golden(name)
    g = O.fourier_grid(c["N_CELLS"])
    assert np.abs(g - f["fgrid"]).max() / np.abs(g).max() < 1e-6
    assert g[0, 0, 0] == 0.0


@pytest.mark.parametrize("name", GOLDEN_CASES)
def test_potential_matches_reference(name):
    f, c = load_golden(name)
    n = c["N_CELLS"]
    fg = O.fourier_grid(n)
    for s in range(c["steps"]):
        phi = O.potential(f[f"rho{s}"], fg, f["a"][s], c["OMEGA_M0"])
        assert rel_l2(phi, f[f"phi{s}"]) < 1e-6


@pytest.mark.parametrize("name", GOLDEN_CASES)
def test_advance_time_matches_reference(name):
    f, c = load_golden(name)
    n = c["N_CELLS"]
    fg = O.fourier_grid(n)
    da = (c["A_END"] - c["A_INIT"]) / c["STEPS"]
    for s in range(c["steps"]):
        x, v = O.advance_time(f[f"rho{s}"], f[f"pos{s}"], f[f"vel{s}"], fg, f["a"][s], da, c["OMEGA_M0"],
                              c["OMEGA_LAMBDA0"], c["OMEGA_K0"], c["H0"])
        assert periodic_maxdiff(x, f[f"pos{s + 1}"], n) < 4 * np.spacing(np.float32(n))
        assert rel_l2(v, f[f"vel{s + 1}"]) < 1e-6


def test_step_count_matches_driver_loop():
    # pmesh.py:56,63 runs one step fewer than STEPS for these configurations (Q6)
    assert O.step_count(0.02, 1.0, 1000) in (999, 1000)
    n = O.step_count(0.01, 1.0, 100)
    a, da, k = 0.01, 0.99 / 100, 0
    while a < 1.0 - da:
        a += da
        k += 1
    assert n == k


def test_cosmo_f_quirk_q1():
    # the reference passes [H0, OL, OK] to f (integrate.py:12)
    g, kick, drift = O.step_coefficients(0.5, 0.01, 0.3, 0.7, 0.0, 0.7)
    fa1 = O.cosmo_f(0.51, [0.7, 0.7, 0.0])
    assert kick == pytest.approx(0.01 * fa1, rel=1e-15)
    assert drift == pytest.approx(0.01 / 0.51 ** 2 * fa1, rel=1e-15)
    g2, kick2, _ = O.step_coefficients(0.5, 0.01, 0.3, 0.7, 0.0, 0.7, fix_cosmo_f=True)
    assert kick2 == pytest.approx(0.01 * O.cosmo_f(0.51, [0.3, 0.7, 0.0]), rel=1e-15)


def test_canonical_position_quirk_q4():
    n = 16
    pos = np.array([[16.0, 3.25], [2.5, 2.5], [1.5, 1.5]], dtype=np.float32)
    cells, d = O.cic_cells(pos, n, canonical=True)
    assert cells[0, 0] == 0 and d[0, 0] == 0.0
    cells_r, d_r = O.cic_cells(pos, n, canonical=False)
    assert cells_r[0, 0] == 0 and d_r[0, 0] == 16.0  # reference behaviour: weights outside [0, 1]
    rho = O.density(pos, 1.0, n)
    assert rho.sum() == pytest.approx(2.0)


def test_uniform_lattice_gives_uniform_density():
    n = 16
    g = (np.arange(n) + 0.5).astype(np.float32)
    z, y, x = np.meshgrid(g, g, g, indexing="ij")
    pos = np.stack([x.ravel(), y.ravel(), z.ravel()])
    rho = O.density(pos, 1.0, n)
    assert np.allclose(rho, 1.0, rtol=0, atol=1e-12)


def test_plane_wave_potential():
    n, m, eps, a, om = 32, 3, 0.01, 0.5, 0.3
    x = np.arange(n)
    rho = np.broadcast_to(1.0 + eps * np.cos(2 * np.pi * m * x / n), (n, n, n))
    phi = O.potential(rho, O.fourier_grid(n), a, om)
    expect = -3 * om / (8 * a) * eps * np.cos(2 * np.pi * m * x / n) / np.sin(np.pi * m / n) ** 2
    assert np.abs(phi - np.broadcast_to(expect, (n, n, n))).max() < 1e-12


def test_cell_keys_order_rows_by_tile():
    n = 16
    rng = np.random.default_rng(0)
    pos = rng.uniform(0, n, (3, 1000)).astype(np.float32)
    keys = O.cell_keys(pos, n)
    cells, _ = O.cic_cells(pos, n)
    xb = O.key_xbits(n)
    assert np.array_equal(keys & ((1 << xb) - 1), cells[0])
    rows = keys >> xb
    assert np.array_equal(rows, O.row_index(cells[1], cells[2], n))
    assert rows.max() < n * n


@pytest.mark.parametrize("name", COMPACT_CASES)
def test_oracle_matches_reference_64p_128g(name):
    """The 64^3-particle / 128^3-grid configuration (box 100 Mpc/h, seed 0, 100 STEPS): one
    step of the oracle against the reference's own outputs, at the fixture's sampled cells and
    particles and through whole-grid sums."""
    f, c = load_golden(name)
    n = c["N_CELLS"]
    mass = (n / c["N_PARTS"]) ** 3
    idx, pidx = f["cell_idx"], f["part_idx"]
    rho = O.density(f["pos0"], mass, n)
    assert rel_l2(rho.reshape(-1)[idx], f["rho0_s"]) < 1e-6
    assert rel_l2(rho.sum(axis=0), f["rho0_proj"]) < 1e-6
    assert abs(rho.sum() - f["rho0_sum"]) < 1e-6 * f["rho0_sum"]
    fg = O.fourier_grid(n)
    phi = O.potential(rho, fg, f["a"][0], c["OMEGA_M0"])
    assert rel_l2(phi.reshape(-1)[idx], f["phi0_s"]) < 1e-6
    assert rel_l2(phi.sum(axis=0), f["phi0_proj"]) < 1e-6
    da = (c["A_END"] - c["A_INIT"]) / c["STEPS"]
    x, v = O.advance_time(rho, f["pos0"], f["vel0"], fg, f["a"][0], da, c["OMEGA_M0"], c["OMEGA_LAMBDA0"],
                          c["OMEGA_K0"], c["H0"])
    assert periodic_maxdiff(x[:, pidx], f["pos1_s"], n) < 4 * np.spacing(np.float32(n))
    assert rel_l2(v[:, pidx], f["vel1_s"]) < 1e-6
    assert rel_l2((v.astype(np.float64) ** 2).sum(axis=1), f["vel1_sq"]) < 1e-6
