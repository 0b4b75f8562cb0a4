"""Generate the golden fixtures under tests/golden/ from the reference itself.

Run in a container that has the reference source, naming its src/ directory:

    PM_REFERENCE_SRC=<reference checkout>/src python tests/golden/make_golden.py [case ...]

For each case the reference's own functions are run (through ``ref_shim``):
gaussian_random_field -> zeldovich (jitter seeded, see ref_shim) -> fourier_grid ->
then ``steps`` iterations of the pmesh.py:60-63 loop body
(``density`` -> ``advance_time`` -> ``a += da``).  Saved per case (float32 unless noted):

  grf            gaussian_random_field() output (N_PARTS^3)
  pos0, vel0     zeldovich() output (3, N_PARTS^3)
  fgrid          fourier_grid() with the k=0 entry forced to 0 (see Q2); grids <= 24 only
  rho{s}         density() at step s
  phi{s}         potential(rho{s}, fgrid, a_s)  (the potential advance_time uses)
  pos{s+1}, vel{s+1}  advance_time() output
  a              float64 scale factors a_0 .. a_steps
  cfg            json string of the configure_me overrides

Compact cases (the 64^3-particle / 128^3-grid configuration, whose full grids would make a
fixture of tens of MB) keep the inputs pos0 / vel0 whole and the outputs as samples and
sums, with the indices they were taken at:

  cell_idx       SAMPLE_CELLS flat cell indices (seeded, sorted)
  rho0_s, phi0_s density / potential at cell_idx
  rho0_proj      density summed over z (float64, N x N); rho0_sum its total
  phi0_proj      potential summed over z (float64, N x N)
  part_idx       SAMPLE_PARTS particle indices (seeded, sorted)
  pos1_s, vel1_s advance_time() output at part_idx (3, SAMPLE_PARTS)
  vel1_sq        per-axis float64 sums of squares of the whole advance_time() velocity output
"""
from __future__ import annotations

import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
import ref_shim  # noqa: E402

COSMO = dict(OMEGA_M0=0.3, OMEGA_B0=0.04, OMEGA_K0=0.0, OMEGA_LAMBDA0=0.7, H0=0.7,
             POWER=0.96, LCDM_TRANSFER_FUNCTION=True, A_INIT=0.02, A_END=1.0, N_CPU=1)

CASES = {
    "n8_g16": dict(N_PARTS=8, N_CELLS=16, BOX_SIZE=100, RANDOM_SEED=0, STEPS=100, steps=3),
    "n16_g32": dict(N_PARTS=16, N_CELLS=32, BOX_SIZE=100, RANDOM_SEED=0, STEPS=100, steps=3),
    "n12_g24": dict(N_PARTS=12, N_CELLS=24, BOX_SIZE=150, RANDOM_SEED=5, STEPS=40, steps=2),
    "n24_g48": dict(N_PARTS=24, N_CELLS=48, BOX_SIZE=200, RANDOM_SEED=7, STEPS=60, steps=2),
    "n32_g64": dict(N_PARTS=32, N_CELLS=64, BOX_SIZE=250, RANDOM_SEED=3, STEPS=50, steps=1),
    # the CPU configuration of the reference's own path: 64^3 particles, 128^3 grid, box 100
    "n64_g128": dict(N_PARTS=64, N_CELLS=128, BOX_SIZE=100, RANDOM_SEED=0, STEPS=100, steps=1, compact=True),
}
SAMPLE_CELLS = 1 << 16
SAMPLE_PARTS = 1 << 15


def compact(out, cfg):
    """Keep the inputs whole and the outputs of step 0 as seeded samples and sums."""
    n, npart = cfg["N_CELLS"], cfg["N_PARTS"] ** 3
    rng = np.random.default_rng(20241)
    cell_idx = np.sort(rng.choice(n ** 3, SAMPLE_CELLS, replace=False)).astype(np.int64)
    part_idx = np.sort(rng.choice(npart, SAMPLE_PARTS, replace=False)).astype(np.int64)
    rho, phi = out["rho0"], out["phi0"]
    c = {"pos0": out["pos0"], "vel0": out["vel0"], "a": out["a"], "cell_idx": cell_idx, "part_idx": part_idx,
         "rho0_s": rho.reshape(-1)[cell_idx], "phi0_s": phi.reshape(-1)[cell_idx],
         "rho0_proj": rho.sum(axis=0, dtype=np.float64), "rho0_sum": np.float64(rho.sum(dtype=np.float64)),
         "phi0_proj": phi.sum(axis=0, dtype=np.float64),
         "pos1_s": out["pos1"][:, part_idx], "vel1_s": out["vel1"][:, part_idx],
         "vel1_sq": (out["vel1"].astype(np.float64) ** 2).sum(axis=1)}
    return c


def run_case(name, spec):
    spec = dict(spec)
    steps = spec.pop("steps")
    is_compact = spec.pop("compact", False)
    cfg = dict(COSMO, **spec)
    ref = ref_shim.load(cfg)
    npart = cfg["N_PARTS"] ** 3
    ref.zeldovich.random = ref_shim.SeededUniform(cfg["RANDOM_SEED"], 3 * npart)
    out = {}
    grf = ref.gaussian_random_field.gaussian_random_field()
    out["grf"] = grf.astype(np.float32)
    pos, vel = ref.zeldovich.zeldovich(grf)
    out["pos0"], out["vel0"] = pos.copy(), vel.copy()
    fgrid = np.array(ref.fourier_utils.fourier_grid(), dtype=np.float32)
    fgrid[0, 0, 0] = 0.0  # Q2: uninitialised entry defined as 0
    if cfg["N_CELLS"] <= 24:
        out["fgrid"] = fgrid
    mass = (cfg["N_CELLS"] / cfg["N_PARTS"]) ** 3
    da = (cfg["A_END"] - cfg["A_INIT"]) / cfg["STEPS"]
    a = cfg["A_INIT"]
    avals = [a]
    for s in range(steps):
        rho = ref.density.density(pos, mass)
        out[f"rho{s}"] = np.asarray(rho, dtype=np.float32)
        out[f"phi{s}"] = np.asarray(ref.potential.potential(rho, fgrid, a), dtype=np.float32)
        pos, vel = ref.integrate.advance_time(rho, pos, vel, fgrid, a, da)
        out[f"pos{s + 1}"], out[f"vel{s + 1}"] = pos.copy(), vel.copy()
        a += da
        avals.append(a)
    out["a"] = np.array(avals, dtype=np.float64)
    if is_compact:
        out = compact(out, cfg)
    cfg["steps"] = steps
    cfg["compact"] = bool(is_compact)
    out["cfg"] = np.array(json.dumps(cfg))
    path = os.path.join(HERE, f"{name}.npz")
    np.savez_compressed(path, **out)
    print(name, "->", path, os.path.getsize(path), "bytes")


if __name__ == "__main__":
    only = sys.argv[1:]
    for name, spec in CASES.items():
        if not only or name in only:
            run_case(name, spec)
