"""The multi-threaded CPU port (oracle/cpu_step.c, the CPU baseline of bench.py) against the
float64 numpy oracle and the reference's own golden outputs."""
import numpy as np
import pytest

from conftest import golden_config, load_golden, periodic_maxdiff, rel_l2


@pytest.mark.parametrize("name", ["n16_g32", "n24_g48"])
def test_cpu_port_step_matches_oracle_and_reference(name):
    from oracle import cpu_port as C
    from oracle import pm_oracle as O
    f, c = load_golden(name)
    cfg = golden_config(c)
    rho = C.density(f["pos0"], cfg.mass, cfg.n_cells)
    assert np.allclose(rho, O.density(f["pos0"], cfg.mass, cfg.n_cells), rtol=1e-12, atol=1e-12)
    assert rel_l2(rho, f["rho0"]) < 1e-6
    p, v = f["pos0"].copy(), f["vel0"].copy()
    fg = O.fourier_grid(cfg.n_cells)
    C.step(p, v, cfg.mass, cfg.a_init, cfg.da, cfg, fg, workers=2)
    x_o, v_o = O.advance_time(O.density(f["pos0"], cfg.mass, cfg.n_cells), f["pos0"], f["vel0"], fg, cfg.a_init,
                              cfg.da, cfg.omega_m0, cfg.omega_lambda0, cfg.omega_k0, cfg.h0)
    assert periodic_maxdiff(p, x_o, cfg.n_cells) < 4 * np.spacing(np.float32(cfg.n_cells))
    assert np.abs(v - v_o).max() <= 1e-6 * np.abs(v_o).max()
    assert rel_l2(v, f["vel1"]) < 1e-5
