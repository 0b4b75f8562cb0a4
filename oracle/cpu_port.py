"""Multi-threaded CPU port of the reference step, the CPU baseline of bench.py.

TEST INFRASTRUCTURE ONLY (part of the oracle): the particle loops run in
oracle/cpu_step.c (C + OpenMP, float64 arithmetic, float32 state as in the reference), the
FFT Poisson solve in scipy.fft with the same number of threads (oracle/pm_oracle.potential;
the reference threads pyFFTW with N_CPU).  Checked against oracle/pm_oracle.py by
tests/test_cpu_port.py.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

from . import pm_oracle as O

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "cpu_step.c")
LIB = os.path.join(os.path.dirname(HERE), "_build", "libpm_cpu_step.so")

_lib = None


def build(force: bool = False) -> str:
    """gcc -O3 -fopenmp; the library goes to _build/ (not tracked)."""
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= os.path.getmtime(SRC):
        return LIB
    os.makedirs(os.path.dirname(LIB), exist_ok=True)
    tmp = LIB + ".tmp"
    subprocess.run(["gcc", "-O3", "-fopenmp", "-shared", "-fPIC", SRC, "-o", tmp, "-lm"], check=True)
    os.replace(tmp, LIB)
    return LIB


def load():
    global _lib
    if _lib is None:
        lib = ctypes.CDLL(build())
        f32p, f64p = ctypes.POINTER(ctypes.c_float), ctypes.POINTER(ctypes.c_double)
        lib.cpu_density.argtypes = [f32p, ctypes.c_longlong, ctypes.c_int, ctypes.c_double, f64p]
        lib.cpu_density.restype = None
        lib.cpu_integrate.argtypes = [f32p, f32p, ctypes.c_longlong, ctypes.c_int, f64p, ctypes.c_double,
                                      ctypes.c_double, ctypes.c_double]
        lib.cpu_integrate.restype = None
        _lib = lib
    return _lib


def _f32(a):
    return np.ascontiguousarray(a, dtype=np.float32)


def density(positions, mass, n):
    """density.py:7-48 (float64 grid)."""
    lib = load()
    p = _f32(positions)
    grid = np.empty(n ** 3, dtype=np.float64)
    lib.cpu_density(p.ctypes.data_as(ctypes.POINTER(ctypes.c_float)), p.shape[1], n, float(mass),
                    grid.ctypes.data_as(ctypes.POINTER(ctypes.c_double)))
    return grid.reshape(n, n, n)


def integrate(positions, velocities, a, fa1, da, phi):
    """integrate.py:15-97 on float32 arrays, in place; returns them."""
    lib = load()
    ph = np.ascontiguousarray(phi, dtype=np.float64)
    lib.cpu_integrate(positions.ctypes.data_as(ctypes.POINTER(ctypes.c_float)),
                      velocities.ctypes.data_as(ctypes.POINTER(ctypes.c_float)), positions.shape[1], ph.shape[0],
                      ph.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), float(a), float(fa1), float(da))
    return positions, velocities


def step(positions, velocities, mass, a, da, cfg, fgrid, workers):
    """pmesh.py:60-61: density then advance_time, state float32 in place."""
    rho = density(positions, mass, cfg.n_cells)
    phi = O.potential(rho, fgrid, a, cfg.omega_m0, workers=workers)
    del rho
    slot = cfg.omega_m0 if getattr(cfg, "fix_cosmo_f", False) else cfg.h0
    fa1 = O.cosmo_f(a + da, [slot, cfg.omega_lambda0, cfg.omega_k0])
    return integrate(positions, velocities, a, fa1, da, phi)
