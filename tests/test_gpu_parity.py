"""Parity of the CUDA hot path (through the C ABI) with the reference and the FP64 oracle.

Tolerances: cell keys, sorted keys and permutation bit-exact; density
and potential within 1e-5 relative L2 of the FP64 oracle; total mass exact to float32
rounding.  Kick/drift: velocities within 1e-5 relative L2, positions within a few
float32 ulps of the grid size.
"""
import numpy as np
import pytest

from conftest import GOLDEN_CASES, golden_config, load_golden, periodic_maxdiff, rel_l2
from oracle import pm_oracle as O

pytestmark = pytest.mark.gpu

DENS_TOL = 1e-5
PHI_TOL = 1e-5
VEL_TOL = 1e-5


def pos_tol(n):
    return 16 * float(np.spacing(np.float32(n)))


def ctx_for(cfg):
    from pmgpu.context import PMContext
    return PMContext(cfg)


def dev(torch, a):
    return torch.from_numpy(np.ascontiguousarray(a, dtype=np.float32)).cuda()


@pytest.mark.parametrize("name", GOLDEN_CASES)
def test_keys_sort_bit_exact(cuda, name):
    torch = cuda
    f, c = load_golden(name)
    cfg = golden_config(c)
    ctx = ctx_for(cfg)
    for s in range(c["steps"] + 1):
        pos = f[f"pos{s}"]
        keys, skeys, perm = ctx.sort_keys(dev(torch, pos))
        ctx.check_device()
        ok = O.cell_keys(pos, cfg.n_cells)
        k = keys.cpu().numpy().view(np.uint32).astype(np.uint64)
        assert np.array_equal(k, ok)
        order = np.argsort(ok, kind="stable")
        assert np.array_equal(skeys.cpu().numpy().view(np.uint32).astype(np.uint64), ok[order])
        assert np.array_equal(perm.cpu().numpy().view(np.uint32).astype(np.int64), order)


@pytest.mark.parametrize("name", GOLDEN_CASES)
def test_density_parity(cuda, name):
    torch = cuda
    f, c = load_golden(name)
    cfg = golden_config(c)
    ctx = ctx_for(cfg)
    for s in range(c["steps"]):
        pos = f[f"pos{s}"]
        rho = ctx.density(dev(torch, pos), cfg.mass)
        ctx.check_device()
        r = rho.cpu().numpy()
        assert rel_l2(r, O.density(pos, cfg.mass, cfg.n_cells)) < DENS_TOL
        assert rel_l2(r, f[f"rho{s}"]) < DENS_TOL  # the reference's own float32 output
        total = r.sum(dtype=np.float64)
        expect = cfg.mass * cfg.np_total
        assert abs(total - expect) <= 2e-7 * expect


def test_density_deterministic(cuda):
    torch = cuda
    from pmgpu.config import Config
    cfg = Config(n_parts=32, n_cells=64)
    ctx = ctx_for(cfg)
    rng = np.random.default_rng(1)
    # clustered input: many particles share cells (same-address atomics)
    centres = rng.uniform(0, 64, (3, 50))
    pos = (centres[:, rng.integers(0, 50, 32768)] + rng.normal(0, 0.3, (3, 32768))) % 64
    p = dev(torch, pos)
    a = ctx.density(p, 8.0).cpu().numpy()
    b = ctx.density(p, 8.0).cpu().numpy()
    assert np.array_equal(a, b)
    assert rel_l2(a, O.density(pos.astype(np.float32), 8.0, 64)) < DENS_TOL


@pytest.mark.parametrize("name", GOLDEN_CASES)
def test_potential_parity(cuda, name):
    torch = cuda
    f, c = load_golden(name)
    cfg = golden_config(c)
    ctx = ctx_for(cfg)
    fg_o = O.fourier_grid(cfg.n_cells)
    fg = ctx.fourier_grid()
    assert np.abs(fg.cpu().numpy() - fg_o).max() / fg_o.max() < 1e-6
    for s in range(c["steps"]):
        rho = f[f"rho{s}"]
        a = f["a"][s]
        expect = O.potential(rho, fg_o, a, cfg.omega_m0)
        phi = ctx.potential(dev(torch, rho), None, a).cpu().numpy()
        assert rel_l2(phi, expect) < PHI_TOL
        assert rel_l2(phi, f[f"phi{s}"]) < PHI_TOL
        phi_t = ctx.potential(dev(torch, rho), fg, a).cpu().numpy()  # caller's Green table
        assert rel_l2(phi_t, expect) < PHI_TOL


@pytest.mark.parametrize("name", GOLDEN_CASES)
def test_integrate_parity(cuda, name):
    torch = cuda
    f, c = load_golden(name)
    cfg = golden_config(c)
    ctx = ctx_for(cfg)
    n = cfg.n_cells
    for s in range(c["steps"]):
        a = f["a"][s]
        fa1 = O.cosmo_f(a + cfg.da, [cfg.h0, cfg.omega_lambda0, cfg.omega_k0])
        phi = f[f"phi{s}"]
        x_o, v_o = O.integrate(f[f"pos{s}"], f[f"vel{s}"], a, fa1, cfg.da, phi)
        p, v = dev(torch, f[f"pos{s}"]), dev(torch, f[f"vel{s}"])
        ctx.integrate(p, v, a, fa1, cfg.da, dev(torch, phi))
        ctx.check_device()
        assert rel_l2(v.cpu().numpy(), v_o) < VEL_TOL
        assert periodic_maxdiff(p.cpu().numpy(), x_o, n) < pos_tol(n)


@pytest.mark.parametrize("name", GOLDEN_CASES)
def test_advance_time_matches_reference(cuda, name):
    torch = cuda
    f, c = load_golden(name)
    cfg = golden_config(c)
    ctx = ctx_for(cfg)
    for s in range(c["steps"]):
        p, v = dev(torch, f[f"pos{s}"]), dev(torch, f[f"vel{s}"])
        ctx.advance_time(dev(torch, f[f"rho{s}"]), p, v, None, f["a"][s], cfg.da)
        ctx.check_device()
        assert rel_l2(v.cpu().numpy(), f[f"vel{s + 1}"]) < VEL_TOL
        assert periodic_maxdiff(p.cpu().numpy(), f[f"pos{s + 1}"], cfg.n_cells) < pos_tol(cfg.n_cells)


@pytest.mark.parametrize("name", GOLDEN_CASES)
def test_step_chain_matches_reference(cuda, name):
    """pmesh.py loop body (density -> advance_time) chained over the fixture's steps."""
    torch = cuda
    f, c = load_golden(name)
    cfg = golden_config(c)
    ctx = ctx_for(cfg)
    p, v = dev(torch, f["pos0"]), dev(torch, f["vel0"])
    rho = ctx.grid()
    for s in range(c["steps"]):
        ctx.step(p, v, cfg.mass, f["a"][s], cfg.da, rho_out=rho)
        ctx.check_device()
        assert rel_l2(rho.cpu().numpy(), f[f"rho{s}"]) < DENS_TOL
        assert rel_l2(v.cpu().numpy(), f[f"vel{s + 1}"]) < 10 * VEL_TOL * (s + 1)
        assert periodic_maxdiff(p.cpu().numpy(), f[f"pos{s + 1}"], cfg.n_cells) < pos_tol(cfg.n_cells) * (s + 1)


# ---- known-answer and edge cases -------------------------------------------------------
def test_uniform_lattice_and_edges(cuda):
    torch = cuda
    from pmgpu.config import Config
    n = 32
    ctx = ctx_for(Config(n_parts=32, n_cells=n))
    g = (np.arange(n) + 0.5).astype(np.float32)
    z, y, x = np.meshgrid(g, g, g, indexing="ij")
    pos = np.stack([x.ravel(), y.ravel(), z.ravel()])
    rho = ctx.density(dev(torch, pos), 1.0).cpu().numpy()
    assert np.array_equal(rho, np.ones_like(rho))
    # edge (oracle quirk Q4): x == N exactly, x = N - eps, x = 0 (periodic wrap of the CIC corners)
    edge = np.array([[n, n - 1e-4, 0.0, 31.999998], [0.5, 5.5, n - 0.25, 7.0], [3.0, n, 0.0, 31.5]],
                    dtype=np.float32)
    r = ctx.density(dev(torch, edge), 2.0)
    ctx.check_device()
    r = r.cpu().numpy()
    assert rel_l2(r, O.density(edge, 2.0, n)) < DENS_TOL
    assert r.sum(dtype=np.float64) == pytest.approx(8.0, rel=1e-6)


def test_plane_wave_potential_gpu(cuda):
    torch = cuda
    from pmgpu.config import Config
    for n in (48, 64, 96, 128):
        ctx = ctx_for(Config(n_parts=n // 2, n_cells=n, omega_m0=0.3))
        m, eps, a = 3, 0.01, 0.5
        x = np.arange(n)
        rho = np.ascontiguousarray(np.broadcast_to(1.0 + eps * np.cos(2 * np.pi * m * x / n), (n, n, n)))
        phi = ctx.potential(dev(torch, rho), None, a).cpu().numpy()
        expect = -3 * 0.3 / (8 * a) * eps * np.cos(2 * np.pi * m * x / n) / np.sin(np.pi * m / n) ** 2
        assert rel_l2(phi, np.broadcast_to(expect, (n, n, n))) < PHI_TOL


def test_nonfinite_position_flagged(cuda):
    torch = cuda
    from pmgpu.config import Config
    from pmgpu import PMError
    ctx = ctx_for(Config(n_parts=16, n_cells=32))
    pos = np.full((3, 8), 3.5, dtype=np.float32)
    pos[0, 3] = np.nan
    rho = ctx.density(dev(torch, pos), 1.0)
    with pytest.raises(PMError):
        ctx.check_device()
    r = rho.cpu().numpy()
    assert r.sum(dtype=np.float64) == pytest.approx(7.0)  # the bad particle is skipped
    ctx.check_device()  # flags were cleared


# ---- larger sizes: oracle comparison and size-independent properties ----------------------
@pytest.mark.parametrize("nparts,ncells", [(48, 96), (64, 128), (96, 192), (128, 256), (192, 384)])
def test_density_potential_large(cuda, nparts, ncells):
    torch = cuda
    from pmgpu.config import Config
    from pmgpu import ics
    cfg = Config(n_parts=nparts, n_cells=ncells, box_size=200.0, random_seed=11)
    pos, vel = ics.initial_conditions(cfg)
    ctx = ctx_for(cfg)
    rho = ctx.density(dev(torch, pos), cfg.mass)
    ctx.check_device()
    r = rho.cpu().numpy()
    ro = O.density(pos, cfg.mass, ncells)
    assert rel_l2(r, ro) < DENS_TOL
    a = 0.05
    phi = ctx.potential(rho, None, a).cpu().numpy()
    po = O.potential(ro, O.fourier_grid(ncells), a, cfg.omega_m0)
    assert rel_l2(phi, po) < PHI_TOL


def test_full_size_properties(cuda):
    """At the 512^3 grid: mass conservation, determinism and linearity of the solve."""
    torch = cuda
    from pmgpu.config import Config
    n, npart = 512, 1 << 24
    ctx = ctx_for(Config(n_parts=256, n_cells=n))
    gen = torch.Generator(device="cuda").manual_seed(5)
    pos = torch.rand((3, npart), device="cuda", generator=gen) * n
    rho = ctx.density(pos, 8.0)
    ctx.check_device()
    total = rho.double().sum().item()
    assert total == pytest.approx(8.0 * npart, rel=1e-6)
    rho2 = ctx.density(pos, 8.0)
    assert torch.equal(rho, rho2)
    phi = ctx.potential(rho, None, 0.3)
    phi2 = ctx.potential(rho * 2.0, None, 0.3)
    err = ((phi2 - 2.0 * phi).double().norm() / (2.0 * phi).double().norm()).item()
    assert err < 1e-6
    # constant density has zero potential (k = 0 removed)
    const = torch.full((n, n, n), 3.0, device="cuda")
    assert ctx.potential(const, None, 0.3).abs().max().item() < 1e-6


def test_step_fused_deposit_matches_unfused(cuda):
    """pm_step without a density output deposits straight into the x-transformed spectrum;
    the arithmetic per element is the same, so the step is bit-identical."""
    torch = cuda
    from pmgpu.config import Config
    from pmgpu import ics
    cfg = Config(n_parts=64, n_cells=128, box_size=150.0, random_seed=4)
    pos, vel = ics.initial_conditions(cfg)
    ctx = ctx_for(cfg)
    out = []
    for want_rho in (True, False):
        p, v = dev(torch, pos), dev(torch, vel)
        for s in range(3):
            ctx.step(p, v, cfg.mass, cfg.a_init + s * cfg.da, cfg.da, rho_out=ctx.grid() if want_rho else None)
        ctx.check_device()
        out.append((p.cpu().numpy(), v.cpu().numpy()))
    assert np.array_equal(out[0][0], out[1][0])
    assert np.array_equal(out[0][1], out[1][1])


def test_step_fused_deposit_clustered(cuda):
    """Clustered particles (hundreds per cell, very uneven tiles) through the fused deposit,
    whose tiles are handed out by a counter: the step is bit-identical to the unfused one,
    and the density matches the oracle."""
    torch = cuda
    from pmgpu.config import Config
    cfg = Config(n_parts=32, n_cells=64, box_size=100.0)
    rng = np.random.default_rng(7)
    centres = rng.uniform(0, 64, (3, 12))
    pos = ((centres[:, rng.integers(0, 12, cfg.np_total)] + rng.normal(0, 0.4, (3, cfg.np_total))) % 64)
    pos = pos.astype(np.float32)
    vel = rng.normal(0, 0.5, (3, cfg.np_total)).astype(np.float32)
    ctx = ctx_for(cfg)
    rho = ctx.density(dev(torch, pos), cfg.mass).cpu().numpy()
    assert rel_l2(rho, O.density(pos, cfg.mass, cfg.n_cells)) < DENS_TOL
    out = []
    for want_rho in (True, False):
        p, v = dev(torch, pos), dev(torch, vel)
        for s in range(2):
            ctx.step(p, v, cfg.mass, cfg.a_init + s * cfg.da, cfg.da, rho_out=ctx.grid() if want_rho else None)
        ctx.check_device()
        out.append((p.cpu().numpy(), v.cpu().numpy()))
    assert np.array_equal(out[0][0], out[1][0])
    assert np.array_equal(out[0][1], out[1][1])


@pytest.mark.parametrize("n_parts,n_cells", [(32, 64), (128, 256)])
def test_step_host_pinned_and_pageable_match_device_step(cuda, n_parts, n_cells):
    """pm_step_host on pinned arrays (positions read over the host link by the keys kernel,
    the result gathered straight into host memory) and on pageable arrays (copy engines)
    give the device step's bits."""
    torch = cuda
    from pmgpu.config import Config
    from pmgpu import ics
    cfg = Config(n_parts=n_parts, n_cells=n_cells, box_size=180.0, random_seed=6)
    pos, vel = ics.initial_conditions(cfg)
    ctx = ctx_for(cfg)
    p, v = dev(torch, pos), dev(torch, vel)
    hp = torch.from_numpy(pos.copy()).pin_memory()
    hv = torch.from_numpy(vel.copy()).pin_memory()
    pp, pv = pos.copy(), vel.copy()
    for s in range(3):
        a = cfg.a_init + s * cfg.da
        ctx.step(p, v, cfg.mass, a, cfg.da)
        ctx.step_host(hp, hv, cfg.mass, a, cfg.da)
        ctx.step_host(pp, pv, cfg.mass, a, cfg.da)
    ctx.check_device()
    assert np.array_equal(hp.numpy(), p.cpu().numpy()) and np.array_equal(hv.numpy(), v.cpu().numpy())
    assert np.array_equal(pp, p.cpu().numpy()) and np.array_equal(pv, v.cpu().numpy())
