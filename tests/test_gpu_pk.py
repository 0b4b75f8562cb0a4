"""Accuracy after a whole run: matter power spectrum of the GPU engine (float32, displacement
storage) against the float64 oracle (oracle/torch64.py, the reference algorithm in float64
on the GPU), started from the same initial conditions.

Gate: P(k) within 0.5% for k < k_Nyquist / 2, total mass exact to float32
rounding.  Trajectories themselves are not compared after many steps: N-body dynamics
amplify rounding differences, the power spectrum is the statistic that must agree."""
import json
import os

import numpy as np
import pytest

from conftest import load_golden

pytestmark = pytest.mark.gpu

PK_TOL = 0.005


def test_torch64_copy_matches_numpy_oracle(cuda):
    """The float64 torch copy reproduces the numpy oracle (and so the reference)."""
    torch = cuda
    from oracle import pm_oracle as O
    from oracle import torch64 as T
    from conftest import golden_config
    f, c = load_golden("n16_g32")
    cfg = golden_config(c)
    p, v, a = T.run(f["pos0"], f["vel0"], cfg, 2)
    x, vv = f["pos0"], f["vel0"]
    fg = O.fourier_grid(cfg.n_cells)
    aa = cfg.a_init
    for _ in range(2):
        rho = O.density(x, cfg.mass, cfg.n_cells)
        x, vv = O.advance_time(rho, x, vv, fg, aa, cfg.da, cfg.omega_m0, cfg.omega_lambda0, cfg.omega_k0, cfg.h0)
        aa += cfg.da
    # the numpy oracle stores positions as float32 between steps, as the reference does;
    # the torch copy keeps them in float64: they agree to float32 rounding of the positions
    d = np.abs(p.cpu().numpy() - x) % cfg.n_cells
    assert np.minimum(d, cfg.n_cells - d).max() < 1e-5
    assert np.abs(v.cpu().numpy() - vv).max() < 1e-5 * np.abs(vv).max()
    rho = T.density(p, cfg.mass, cfg.n_cells).cpu().numpy()
    k1, p1, _ = T.power_spectrum(torch.from_numpy(rho).cuda(), cfg.box_size)
    k2, p2, _ = O.power_spectrum(rho, cfg.box_size)
    assert np.allclose(p1, p2, rtol=1e-10) and np.allclose(k1, k2, rtol=1e-12)


def run_pk_case(torch, n_parts, n_cells, box, steps, seed=0):
    from oracle import torch64 as T
    from pmgpu import ics
    from pmgpu.batch import Batch
    from pmgpu.config import Config, step_count
    cfg = Config(n_parts=n_parts, n_cells=n_cells, box_size=box, random_seed=seed, steps=steps)
    if n_parts > 256:  # the initial conditions on the device (the host restatement takes minutes)
        from pmgpu.device_ics import DeviceICs
        g = DeviceICs(n_parts)
        pos, vel = g.generate(cfg)
        g.close()
    else:
        pos, vel = ics.initial_conditions(cfg)
    nsteps = step_count(cfg.a_init, cfg.a_end, cfg.steps)
    b = Batch()
    sid = b.add(cfg, pos, vel)
    b.step(nsteps + 10)
    b.check_device()
    gp, gv, a_gpu, done = b.get(sid, device=True)
    assert done == nsteps
    b.close()
    p64, v64, a64 = T.run(pos, vel, cfg, nsteps)
    assert abs(a64 - a_gpu) < 1e-12
    rho_gpu = T.density(gp.double(), cfg.mass, n_cells)
    rho_64 = T.density(p64, cfg.mass, n_cells)
    mass = cfg.mass * cfg.np_total
    k, pk_gpu, _ = T.power_spectrum(rho_gpu, box)
    _, pk_64, _ = T.power_spectrum(rho_64, box)
    sel = np.arange(1, len(k) + 1) < n_cells // 4  # |m| < N/4: k < k_Nyquist / 2
    rel = np.abs(pk_gpu[sel] / pk_64[sel] - 1.0)
    # the engine's own (float32, sorted, integer-accumulated) deposit of the final state
    from pmgpu.context import PMContext
    rho_f32 = PMContext(cfg).density(gp, cfg.mass)
    total = rho_f32.double().sum().item()
    return {"n_parts": n_parts, "n_cells": n_cells, "box": box, "steps": nsteps, "a_end": a_gpu,
            "pk_max_rel_dev": float(rel.max()), "pk_mean_rel_dev": float(rel.mean()), "bins": int(sel.sum()),
            "mass_rel_err": abs(total - mass) / mass, "k": k[sel].tolist(), "pk_gpu": pk_gpu[sel].tolist(),
            "pk_fp64": pk_64[sel].tolist()}


def record(res):
    """Write the spectra to $PM_RESULTS_DIR (when set) for the record."""
    out = os.environ.get("PM_RESULTS_DIR")
    if out and os.path.isdir(out):
        name = f"pk_{res['n_parts']}p_{res['n_cells']}g.json"
        with open(os.path.join(out, name), "w") as fh:
            json.dump(res, fh)


def test_pk_after_full_run_128p_256g(cuda):
    res = run_pk_case(cuda, 128, 256, 200.0, 1000)
    record(res)
    print("P(k) 128^3/256^3:", {k: v for k, v in res.items() if not isinstance(v, list)})
    assert res["pk_max_rel_dev"] < PK_TOL
    assert res["mass_rel_err"] < 1e-6


@pytest.mark.slow
def test_pk_after_full_run_256p_512g(cuda):
    """The README workload: 256^3 particles, 512^3 grid, box 250 Mpc/h, 1000 steps."""
    res = run_pk_case(cuda, 256, 512, 250.0, 1000)
    record(res)
    print("P(k) 256^3/512^3:", {k: v for k, v in res.items() if not isinstance(v, list)})
    assert res["pk_max_rel_dev"] < PK_TOL
    assert res["mass_rel_err"] < 1e-6


@pytest.mark.slow
@pytest.mark.skipif(not os.environ.get("PM_FULL_RUNS"),
                    reason="500 float64 oracle steps at 1024^3 take minutes: set PM_FULL_RUNS=1")
def test_pk_after_full_run_512p_1024g(cuda):
    """The large configuration: 512^3 particles, 1024^3 grid, box 500 Mpc/h, seed 1, 500 steps."""
    res = run_pk_case(cuda, 512, 1024, 500.0, 500, seed=1)
    record(res)
    print("P(k) 512^3/1024^3:", {k: v for k, v in res.items() if not isinstance(v, list)})
    assert res["pk_max_rel_dev"] < PK_TOL
    assert res["mass_rel_err"] < 1e-6


# ---- the device estimator (pm_power_spectrum) against the oracle's -------------------------

@pytest.mark.parametrize("name", ["n16_g32", "n24_g48", "n32_g64"])
def test_device_power_spectrum_matches_oracle(cuda, name):
    torch = cuda
    from oracle import pm_oracle as O
    from pmgpu.context import PMContext
    from conftest import golden_config
    f, c = load_golden(name)
    cfg = golden_config(c)
    rho = f["rho0"]
    ctx = PMContext(cfg)
    k, p, m = ctx.power_spectrum(torch.from_numpy(rho).cuda())
    k2, p2, m2 = O.power_spectrum(rho, cfg.box_size)
    assert np.array_equal(m, m2)
    assert np.allclose(k, k2, rtol=1e-12)
    assert np.abs(p / p2 - 1).max() < 1e-5
    # deterministic, and a reduced bin count is the prefix of the full one
    k3, p3, _ = ctx.power_spectrum(torch.from_numpy(rho).cuda())
    assert np.array_equal(p, p3) and np.array_equal(k, k3)
    kb, pb, mb = ctx.power_spectrum(torch.from_numpy(rho).cuda(), nbins=cfg.n_cells // 4)
    assert len(pb) == cfg.n_cells // 4 - 1
    assert np.array_equal(mb, m[: len(mb)])
    assert np.allclose(pb, p[: len(pb)], rtol=1e-12)
    ctx.close()


@pytest.mark.parametrize("n_parts,n_cells", [(64, 128), (128, 256), (256, 512)])
def test_device_power_spectrum_of_evolved_grid(cuda, n_parts, n_cells):
    """A deposited density after some steps (strongly non-Gaussian) at larger sizes: the
    float32 spectrum gives P(k) within 1e-4 of the float64 oracle on the same grid."""
    torch = cuda
    from oracle import torch64 as T
    from pmgpu import ics
    from pmgpu.batch import Batch
    from pmgpu.config import Config
    from pmgpu.context import PMContext
    cfg = Config(n_parts=n_parts, n_cells=n_cells, box_size=150.0, random_seed=2, steps=60)
    b = Batch()
    sid = b.add(cfg, *ics.initial_conditions(cfg))
    b.step(40)
    pos, _, _, _ = b.get(sid, device=True)
    b.close()
    ctx = PMContext(cfg)
    rho = ctx.density(pos, cfg.mass)
    k, p, m = ctx.power_spectrum(rho)
    k2, p2, m2 = T.power_spectrum(rho.double(), cfg.box_size)
    assert np.array_equal(m, m2)
    assert np.allclose(k, k2, rtol=1e-12)
    assert np.abs(p / p2 - 1).max() < 1e-4
    ctx.close()


def test_device_power_spectrum_rejects_bad_arguments(cuda):
    torch = cuda
    from pmgpu import _lib
    from pmgpu.config import Config
    from pmgpu.context import PMContext
    ctx = PMContext(Config(n_parts=16, n_cells=32))
    rho = torch.ones((32,) * 3, device="cuda")
    with pytest.raises(_lib.PMError):
        ctx.power_spectrum(rho, nbins=40)
    with pytest.raises(_lib.PMError):
        ctx.power_spectrum(rho, box_size=-1.0)
    ctx.close()


@pytest.mark.slow
def test_config3_512p_1024g_short_run_against_fp64(cuda):
    """The 512^3-particle / 1024^3-grid configuration (box 500 Mpc/h, seed 1): initial
    conditions on the device, 5 resident steps, against the float64 copy of the reference
    algorithm from the same initial conditions."""
    torch = cuda
    from oracle import torch64 as T
    from pmgpu.batch import Batch
    from pmgpu.config import Config
    from pmgpu.device_ics import DeviceICs
    cfg = Config(n_parts=512, n_cells=1024, box_size=500.0, random_seed=1, steps=500)
    g = DeviceICs(512)
    pos, vel = g.generate(cfg)
    g.close()
    b = Batch()
    sid = b.add(cfg, pos, vel)
    b.step(5)
    b.check_device()
    gp, gv, a_gpu, done = b.get(sid, device=True)
    b.close()
    assert done == 5
    p64, v64, a64 = T.run(pos, vel, cfg, 5)
    assert abs(a64 - a_gpu) < 1e-12
    n = cfg.n_cells
    d = torch.remainder(gp.double() - p64, float(n))
    assert torch.minimum(d, n - d).max().item() < 1e-2
    assert ((gv.double() - v64).norm() / v64.norm()).item() < 5e-4
    del d, gv, v64
    k, pk_gpu, _ = T.power_spectrum(T.density(gp.double(), cfg.mass, n), cfg.box_size)
    _, pk_64, _ = T.power_spectrum(T.density(p64, cfg.mass, n), cfg.box_size)
    sel = np.arange(1, len(k) + 1) < n // 4
    assert np.abs(pk_gpu[sel] / pk_64[sel] - 1.0).max() < 1e-3
