"""The spectral gradient (PM_FLAG_SPECTRAL_GRADIENT): the force from three grids, -i sin(k_d)
phi_k transformed back, instead of the reference's central differences of phi
(src/integrate.py:84-92).  The two are the same linear map of phi -- the Fourier symbol of
(phi[x - e_d] - phi[x + e_d]) / 2 is -i sin(k_d) -- so a step agrees with the central-difference
step and with the oracle to rounding: velocity changes within 1e-4 relative L2 (the kick is a
difference of neighbouring potential values), velocities within 1e-5, positions within 1e-4
cells."""
import dataclasses

import numpy as np
import pytest

from conftest import periodic_maxdiff, rel_l2
from oracle import pm_oracle as O

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("n_parts,n_cells", [(16, 32), (32, 64), (48, 96), (64, 128)])
def test_spectral_gradient_step_matches_central_differences(cuda, n_parts, n_cells):
    torch = cuda
    from pmgpu import ics
    from pmgpu.config import Config
    from pmgpu.context import PMContext
    cfg = Config(n_parts=n_parts, n_cells=n_cells, box_size=150.0, random_seed=3, steps=50)
    pos, vel = ics.initial_conditions(cfg)
    fd = PMContext(cfg)
    sp = PMContext(dataclasses.replace(cfg, spectral_gradient=True))
    out = []
    for ctx in (fd, sp):
        p = torch.from_numpy(pos.copy()).cuda()
        v = torch.from_numpy(vel.copy()).cuda()
        for s in range(2):
            ctx.step(p, v, cfg.mass, cfg.a_init + s * cfg.da, cfg.da)
        ctx.check_device()
        out.append((p.cpu().numpy(), v.cpu().numpy()))
    (p1, v1), (p2, v2) = out
    assert rel_l2(v2 - vel, v1 - vel) < 1e-4
    assert rel_l2(v2, v1) < 1e-5
    assert periodic_maxdiff(p2, p1, n_cells) < 1e-4
    # one step against the oracle (float64, central differences)
    p = torch.from_numpy(pos.copy()).cuda()
    v = torch.from_numpy(vel.copy()).cuda()
    sp.step(p, v, cfg.mass, cfg.a_init, cfg.da)
    rho = O.density(pos, cfg.mass, n_cells)
    x_o, v_o = O.advance_time(rho, pos, vel, O.fourier_grid(n_cells), cfg.a_init, cfg.da, cfg.omega_m0,
                              cfg.omega_lambda0, cfg.omega_k0, cfg.h0)
    assert rel_l2(v.cpu().numpy() - vel, v_o - vel) < 1e-4
    assert periodic_maxdiff(p.cpu().numpy(), x_o, n_cells) < 1e-4
    fd.close()
    sp.close()
