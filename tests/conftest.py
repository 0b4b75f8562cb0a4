import json
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "cosmological-particle-mesh-simulation_gb300")
GOLDEN = os.path.join(ROOT, "tests", "golden")
for p in (ROOT, PKG):
    if p not in sys.path:
        sys.path.insert(0, p)

GOLDEN_CASES = ["n8_g16", "n12_g24", "n16_g32", "n24_g48", "n32_g64"]
# the 64^3-particle / 128^3-grid configuration: inputs whole, outputs sampled (make_golden.py)
COMPACT_CASES = ["n64_g128"]


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built engine")
    config.addinivalue_line("markers", "slow: long-running GPU test")


def load_golden(name):
    """Golden fixture made by tests/golden/make_golden.py from the reference itself."""
    f = np.load(os.path.join(GOLDEN, f"{name}.npz"))
    cfg = json.loads(str(f["cfg"]))
    return f, cfg


def golden_config(c):
    from pmgpu.config import Config
    return Config(n_parts=c["N_PARTS"], n_cells=c["N_CELLS"], box_size=c["BOX_SIZE"],
                  random_seed=c["RANDOM_SEED"], steps=c["STEPS"], power=c["POWER"],
                  omega_m0=c["OMEGA_M0"], omega_b0=c["OMEGA_B0"], omega_k0=c["OMEGA_K0"],
                  omega_lambda0=c["OMEGA_LAMBDA0"], h0=c["H0"], a_init=c["A_INIT"], a_end=c["A_END"])


def rel_l2(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def periodic_maxdiff(a, b, n):
    d = np.abs(np.asarray(a, dtype=np.float64) - np.asarray(b, dtype=np.float64)) % n
    return float(np.minimum(d, n - d).max())


@pytest.fixture(scope="session")
def cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import pmgpu
    pmgpu.build()
    return torch
