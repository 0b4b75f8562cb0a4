"""The drop-in modules (density.py, fourier_utils.py, potential.py, integrate.py, pmesh.py)
used exactly as the reference's driver uses its own modules, on numpy arrays."""
import importlib
import sys
import types

import numpy as np
import pytest

from conftest import load_golden, periodic_maxdiff, rel_l2

pytestmark = pytest.mark.gpu

DROPIN = ["configure_me", "density", "fourier_utils", "potential", "integrate", "cosmology",
          "gaussian_random_field", "zeldovich", "save_data", "pmesh", "plot_helper"]


def install_config(c, **extra):
    for m in DROPIN:
        sys.modules.pop(m, None)
    cm = types.ModuleType("configure_me")
    for k, v in c.items():
        if k.isupper():
            setattr(cm, k, v)
    cm.N_SAVE_FILES, cm.N_PLOTS = 10, 10
    cm.PLOT_STEPS = cm.PLOT_PROJECTIONS = cm.PLOT_GRF = False
    cm.SAVE_DATA = cm.SAVE_DENSITY = False
    cm.PRINT_STATUS = False
    cm.RESTART, cm.RESTART_FROM_N = False, 0
    cm.RESIDENT = False
    for k, v in extra.items():
        setattr(cm, k, v)
    sys.modules["configure_me"] = cm
    return cm


@pytest.fixture
def restore_modules():
    yield
    for m in DROPIN:
        sys.modules.pop(m, None)


def test_reference_loop_body_on_dropin_modules(cuda, restore_modules):
    f, c = load_golden("n16_g32")
    install_config(c)
    density = importlib.import_module("density")
    fourier_utils = importlib.import_module("fourier_utils")
    integrate = importlib.import_module("integrate")
    potential = importlib.import_module("potential")
    n = c["N_CELLS"]
    mass = (n / c["N_PARTS"]) ** 3
    da = (c["A_END"] - c["A_INIT"]) / c["STEPS"]
    fg = fourier_utils.fourier_grid()
    assert isinstance(fg, np.ndarray) and fg.shape == (n, n, n)
    pos, vel = f["pos0"].copy(), f["vel0"].copy()
    a = c["A_INIT"]
    for s in range(c["steps"]):
        rho = density.density(pos, mass)
        assert isinstance(rho, np.ndarray) and rho.dtype == np.float32
        assert rel_l2(rho, f[f"rho{s}"]) < 1e-5
        phi = potential.potential(rho, fg, a)
        assert rel_l2(phi, f[f"phi{s}"]) < 1e-5
        p2, v2 = integrate.advance_time(rho, pos, vel, fg, a, da)
        assert p2 is pos and v2 is vel  # updated in place, like the reference
        assert rel_l2(vel, f[f"vel{s + 1}"]) < 1e-4
        assert periodic_maxdiff(pos, f[f"pos{s + 1}"], n) < 1e-3
        a += da


def test_pmesh_driver_resident_and_loop_agree(cuda, restore_modules):
    f, c = load_golden("n16_g32")
    c = dict(c, STEPS=20)
    results = []
    for resident in (False, True):
        install_config(c, RESIDENT=resident)
        pmesh = importlib.import_module("pmesh")
        pos, vel = pmesh.simulator()
        results.append((np.asarray(pos), np.asarray(vel)))
    (p0, v0), (p1, v1) = results
    # the resident engine stores displacements (more precise): small differences only
    assert periodic_maxdiff(p0, p1, c["N_CELLS"]) < 5e-3
    assert rel_l2(v0, v1) < 1e-3


def test_projection_is_the_reference_loop(cuda, restore_modules):
    """plot_helper.py:65-72: float64 sum of the first planes, in plane order (bit-identical)."""
    f, c = load_golden("n32_g64")
    install_config(c)
    plot_helper = importlib.import_module("plot_helper")
    rho = f["rho0"]
    for n_slices in (0, 1, 15, rho.shape[0]):
        expect = np.zeros(rho.shape[1:], dtype=np.float64)
        for i in range(n_slices):
            expect += rho[i, :, :]
        got = plot_helper.project(rho, n_slices)
        assert got.dtype == np.float64 and np.array_equal(got, expect)


def test_pmesh_resident_writes_snapshots_in_the_background(cuda, restore_modules, tmp_path, monkeypatch):
    """SAVE_DATA with the resident engine: snapshot files with the reference's datasets,
    written by the background writer while the run continues."""
    from pmgpu.snapshot import read_file
    f, c = load_golden("n16_g32")
    c = dict(c, STEPS=20)
    monkeypatch.chdir(tmp_path)
    install_config(c, RESIDENT=True, SAVE_DATA=True, N_SAVE_FILES=4)
    pmesh = importlib.import_module("pmesh")
    pos, vel = pmesh.simulator()
    files = sorted(p.name for p in (tmp_path / "Data").iterdir())
    assert len(files) >= 4 and files[0].startswith("data.0.")
    last = read_file(str(tmp_path / "Data" / files[-1]))
    assert set(last) >= {"x1", "x2", "x3", "vx1", "vx2", "vx3", "a"}
    assert last["x1"].dtype == np.float32 and last["x1"].shape == (c["N_PARTS"] ** 3,)
    assert np.isfinite(last["vx3"]).all() and 0 < float(last["a"]) <= c["A_END"]


def test_pmesh_snapshots_carry_the_density_in_both_modes(cuda, restore_modules, tmp_path, monkeypatch):
    """SAVE_DENSITY: the resident engine writes the `density` dataset (save_data.py:17-18), the
    density the last step before the snapshot was computed from (pmesh.py:60-67), as the loop
    over the drop-in modules does."""
    from pmgpu.snapshot import read_file
    f, c = load_golden("n16_g32")
    c = dict(c, STEPS=20)
    out = {}
    for resident in (False, True):
        d = tmp_path / ("resident" if resident else "loop")
        d.mkdir()
        monkeypatch.chdir(d)
        install_config(c, RESIDENT=resident, SAVE_DATA=True, SAVE_DENSITY=True, N_SAVE_FILES=4)
        pmesh = importlib.import_module("pmesh")
        pmesh.simulator()
        for m in DROPIN:
            sys.modules.pop(m, None)
        out[resident] = {p.name: read_file(str(p)) for p in sorted((d / "Data").iterdir())}
    assert sorted(out[True]) == sorted(out[False]) and len(out[True]) >= 4
    mass = (c["N_CELLS"] / c["N_PARTS"]) ** 3 * c["N_PARTS"] ** 3
    for name, snap in out[True].items():
        if name.startswith("data.0."):  # the initial-conditions file holds the random field
            continue
        rho = snap["density"]
        assert rho.shape == (c["N_CELLS"],) * 3
        assert float(rho.sum(dtype=np.float64)) == pytest.approx(mass, rel=1e-6)
        assert rel_l2(rho, out[False][name]["density"]) < 1e-4, name
