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
