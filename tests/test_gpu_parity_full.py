"""Per-kernel parity at the sizes the metric is quoted on, through the C ABI.

* The 64^3-particle / 128^3-grid configuration against the reference's own outputs
  (tests/golden/n64_g128.npz: inputs whole, outputs sampled and summed).
* The README workload (256^3 particles, 512^3 grid, box 250 Mpc/h) and the large
  configuration (512^3 particles, 1024^3 grid, box 500 Mpc/h, seed 1) against the oracle:
  cell keys, sorted keys and permutation bit-exact (oracle/pm_oracle.cell_keys, stable order);
  density and potential within 1e-5 relative L2 of the float64 oracle (oracle/torch64.py on the
  GPU, validated against the numpy oracle in test_gpu_pk.py).
* Step 1 of the resident engine (displacement storage, keys from displacements, counting
  sort, fused deposit + x transform, kick writing the next keys) against one float64 step of the
  oracle from the same initial conditions: the density of the admitted state (pm_batch_density),
  positions within POS_TOL_CELLS, velocities within 1e-5 relative L2, and the velocity change of
  the step (the kick, the part that depends on the deposit and the solve) within KICK_TOL.
"""
import numpy as np
import pytest

from conftest import COMPACT_CASES, golden_config, load_golden, periodic_maxdiff, rel_l2
from oracle import pm_oracle as O

pytestmark = pytest.mark.gpu

DENS_TOL = 1e-5
PHI_TOL = 1e-5
VEL_TOL = 1e-5
# relative L2 of the velocity change of one step: a difference of neighbouring potential
# values, so it carries the potential's relative error times |phi| / |grad phi|
KICK_TOL = 1e-4
# displacements are float32 offsets from the lattice point, so the absolute position of a
# resident particle carries the rounding of q + d, a few ulps of N
POS_TOL_CELLS = 1e-3


def dev(torch, a):
    return torch.from_numpy(np.ascontiguousarray(a, dtype=np.float32)).cuda()


# ---- 64^3 particles, 128^3 grid: against the reference's outputs -------------------------
@pytest.mark.parametrize("name", COMPACT_CASES)
def test_64p_128g_against_reference(cuda, name):
    torch = cuda
    from pmgpu.context import PMContext
    f, c = load_golden(name)
    cfg = golden_config(c)
    n = cfg.n_cells
    idx, pidx = f["cell_idx"], f["part_idx"]
    ctx = PMContext(cfg)
    pos0 = f["pos0"]
    keys, skeys, perm = ctx.sort_keys(dev(torch, pos0))
    ctx.check_device()
    ok = O.cell_keys(pos0, n)
    assert np.array_equal(keys.cpu().numpy().view(np.uint32).astype(np.uint64), ok)
    assert np.array_equal(perm.cpu().numpy().view(np.uint32).astype(np.int64), np.argsort(ok, kind="stable"))
    rho = ctx.density(dev(torch, pos0), cfg.mass)
    r = rho.cpu().numpy()
    assert rel_l2(r.reshape(-1)[idx], f["rho0_s"]) < DENS_TOL
    assert rel_l2(r.sum(axis=0, dtype=np.float64), f["rho0_proj"]) < DENS_TOL
    assert abs(r.sum(dtype=np.float64) - f["rho0_sum"]) < 1e-6 * f["rho0_sum"]
    phi = ctx.potential(rho, None, float(f["a"][0])).cpu().numpy()
    assert rel_l2(phi.reshape(-1)[idx], f["phi0_s"]) < PHI_TOL
    assert rel_l2(phi.sum(axis=0, dtype=np.float64), f["phi0_proj"]) < PHI_TOL
    p, v = dev(torch, pos0), dev(torch, f["vel0"])
    ctx.step(p, v, cfg.mass, float(f["a"][0]), cfg.da)
    ctx.check_device()
    x, vv = p.cpu().numpy(), v.cpu().numpy()
    assert periodic_maxdiff(x[:, pidx], f["pos1_s"], n) < 16 * float(np.spacing(np.float32(n)))
    assert rel_l2(vv[:, pidx], f["vel1_s"]) < VEL_TOL
    assert rel_l2((vv.astype(np.float64) ** 2).sum(axis=1), f["vel1_sq"]) < VEL_TOL
    ctx.close()


# ---- full sizes: against the float64 oracle ----------------------------------------------
def _initial_conditions(cfg):
    if cfg.n_parts <= 256:
        from pmgpu import ics
        return ics.initial_conditions(cfg)
    from pmgpu.device_ics import DeviceICs
    g = DeviceICs(cfg.n_parts)
    pos, vel = g.generate(cfg)
    g.close()
    return pos.cpu().numpy(), vel.cpu().numpy()


def _config(n_parts):
    from pmgpu.config import Config
    if n_parts == 256:
        return Config(n_parts=256, n_cells=512, box_size=250.0, random_seed=0, steps=1000)
    return Config(n_parts=512, n_cells=1024, box_size=500.0, random_seed=1, steps=500)


def _stable_order(torch, keys_u64):
    """Stable ascending order of the oracle keys (the permutation a stable sort gives)."""
    t = torch.from_numpy(keys_u64.astype(np.int64)).cuda()
    return torch.sort(t, stable=True).indices.cpu().numpy()


def _keys_density_potential(torch, n_parts):
    from oracle import torch64 as T
    from pmgpu.context import PMContext
    cfg = _config(n_parts)
    n = cfg.n_cells
    pos, vel = _initial_conditions(cfg)
    ctx = PMContext(cfg)
    pd = dev(torch, pos)
    keys, skeys, perm = ctx.sort_keys(pd)
    ctx.check_device()
    ok = O.cell_keys(pos, n)
    assert np.array_equal(keys.cpu().numpy().view(np.uint32).astype(np.uint64), ok)
    order = _stable_order(torch, ok)
    assert np.array_equal(skeys.cpu().numpy().view(np.uint32).astype(np.uint64), ok[order])
    assert np.array_equal(perm.cpu().numpy().view(np.uint32).astype(np.int64), order)
    del keys, skeys, perm, order, ok
    rho = ctx.density(pd, cfg.mass)
    ctx.check_device()
    rho64 = T.density(pd.double(), cfg.mass, n)
    e_rho = ((rho.double() - rho64).norm() / rho64.norm()).item()
    total = rho.double().sum().item()
    a = 0.35
    phi = ctx.potential(rho, None, a)
    phi64 = T.potential(rho64, a, cfg.omega_m0)
    e_phi = ((phi.double() - phi64).norm() / phi64.norm()).item()
    ctx.close()
    print(f"{n_parts}^3/{n}^3: density rel-L2 {e_rho:.2e}, potential rel-L2 {e_phi:.2e}")
    assert e_rho < DENS_TOL
    assert e_phi < PHI_TOL
    assert total == pytest.approx(cfg.mass * cfg.np_total, rel=1e-6)


def _resident_step1(torch, n_parts):
    from oracle import torch64 as T
    from pmgpu.batch import Batch
    cfg = _config(n_parts)
    n = cfg.n_cells
    pos, vel = _initial_conditions(cfg)
    b = Batch()
    sid = b.add(cfg, pos, vel)
    rho0 = b.density(sid)
    b.check_device()
    p64 = torch.as_tensor(pos, dtype=torch.float64, device="cuda")
    v64 = torch.as_tensor(vel, dtype=torch.float64, device="cuda")
    rho64 = T.density(p64, cfg.mass, n)
    e_rho = ((rho0.double() - rho64).norm() / rho64.norm()).item()
    del rho0, rho64
    b.step(1)
    b.check_device()
    gp, gv, a_gpu, done = b.get(sid, device=True)
    assert done == 1
    q, w, a64 = T.run(pos, vel, cfg, 1)
    assert abs(a64 - a_gpu) < 1e-12
    d = torch.remainder(gp.double() - q, float(n))
    e_pos = torch.minimum(d, n - d).max().item()
    e_vel = ((gv.double() - w).norm() / w.norm()).item()
    e_kick = ((gv.double() - v64 - (w - v64)).norm() / (w - v64).norm()).item()
    b.close()
    print(f"resident step 1 at {n_parts}^3/{n}^3: density rel-L2 {e_rho:.2e}, positions {e_pos:.2e} cells, "
          f"velocities rel-L2 {e_vel:.2e}, kick rel-L2 {e_kick:.2e}")
    assert e_rho < DENS_TOL
    assert e_pos < POS_TOL_CELLS
    assert e_vel < VEL_TOL
    assert e_kick < KICK_TOL


def test_headline_keys_density_potential(cuda):
    """256^3 particles, 512^3 grid: keys and permutation bit-exact, density and potential
    within 1e-5 of float64."""
    _keys_density_potential(cuda, 256)


def test_headline_resident_step1(cuda):
    """Step 1 of the resident engine at 256^3 / 512^3 against one float64 oracle step."""
    _resident_step1(cuda, 256)


@pytest.mark.slow
def test_large_keys_density_potential(cuda):
    """512^3 particles, 1024^3 grid: keys and permutation bit-exact, density and potential
    within 1e-5 of float64."""
    _keys_density_potential(cuda, 512)


@pytest.mark.slow
def test_large_resident_step1(cuda):
    """Step 1 of the resident engine at 512^3 / 1024^3 against one float64 oracle step."""
    _resident_step1(cuda, 512)
