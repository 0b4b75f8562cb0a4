"""Load the reference's own Python modules without numba / pyFFTW / h5py.

Used only by ``make_golden.py`` (fixture generation) in a container that has the
reference checked out; nothing at test time imports this file.

* the reference's ``src/*.py`` are copied to a temporary directory with the text
  ``'cfloat'`` replaced by ``'complex128'`` (numpy >= 2 removed the alias, used by
  gaussian_random_field.py:27 and zeldovich.py:49-50);
* ``numba`` is stubbed: ``njit`` is the identity, ``prange`` is ``range``;
* ``pyfftw.FFTW`` is stubbed with numpy: FFTW_FORWARD -> ``np.fft.fftn``,
  FFTW_BACKWARD -> ``np.fft.ifftn`` (1/N normalised, pyFFTW's default);
* ``configure_me`` executes the reference's own file, then applies overrides;
* ``zeldovich.random`` (stdlib, unseeded in the reference: zeldovich.py:89-91) is
  replaced by a seeded PCG64 stream so that the jitter is reproducible.
"""
from __future__ import annotations

import importlib
import os
import shutil
import sys
import tempfile
import types

import numpy as np

# the reference's src/ directory (required: e.g. PM_REFERENCE_SRC=<checkout>/src)
REF_SRC = os.environ.get("PM_REFERENCE_SRC")
REF_MODULES = ["configure_me", "cosmology", "density", "fourier_utils", "potential",
               "integrate", "gaussian_random_field", "zeldovich"]


def _numba_stub():
    m = types.ModuleType("numba")

    def njit(*args, **kwargs):
        if args and callable(args[0]):
            return args[0]
        return lambda f: f

    m.njit = njit
    m.prange = range
    m.set_num_threads = lambda n: None
    return m


def _pyfftw_stub():
    m = types.ModuleType("pyfftw")

    class FFTW:
        def __init__(self, inp, out, direction="FFTW_FORWARD", axes=(0, 1, 2), threads=1):
            self.inp, self.out, self.direction, self.axes = inp, out, direction, tuple(axes)

        def __call__(self):
            if self.direction == "FFTW_FORWARD":
                r = np.fft.fftn(self.inp, axes=self.axes)
            else:
                r = np.fft.ifftn(self.inp, axes=self.axes)
            self.out[...] = r
            return self.out

    m.FFTW = FFTW
    return m


class SeededUniform:
    """Stand-in for the stdlib ``random`` module inside zeldovich.py: ``uniform(a, b)``
    returns consecutive draws of ``Generator(PCG64(seed)).uniform(-2, 2, 3*Np)``."""

    def __init__(self, seed, count):
        self._v = np.random.Generator(np.random.PCG64(seed)).uniform(-2.0, 2.0, count)
        self._i = 0

    def uniform(self, a, b):
        assert a == -2.0 and b == 2.0
        v = float(self._v[self._i])
        self._i += 1
        return v


def load(overrides: dict):
    """Import the reference modules with ``overrides`` applied to configure_me.

    Returns a namespace object with the imported modules as attributes.
    """
    if not REF_SRC or not os.path.isdir(REF_SRC):
        raise RuntimeError("set PM_REFERENCE_SRC to the reference's src/ directory")
    for name in REF_MODULES + ["numba", "pyfftw"]:
        sys.modules.pop(name, None)
    tmp = tempfile.mkdtemp(prefix="pmref_")
    for fn in os.listdir(REF_SRC):
        if fn.endswith(".py"):
            with open(os.path.join(REF_SRC, fn)) as f:
                text = f.read().replace("'cfloat'", "'complex128'")
            with open(os.path.join(tmp, fn), "w") as f:
                f.write(text)
    sys.modules["numba"] = _numba_stub()
    sys.modules["pyfftw"] = _pyfftw_stub()
    cm = types.ModuleType("configure_me")
    with open(os.path.join(tmp, "configure_me.py")) as f:
        exec(compile(f.read(), "configure_me.py", "exec"), cm.__dict__)
    for k, v in overrides.items():
        setattr(cm, k, v)
    sys.modules["configure_me"] = cm
    sys.path.insert(0, tmp)
    try:
        ns = types.SimpleNamespace()
        for name in REF_MODULES[1:]:
            setattr(ns, name, importlib.import_module(name))
        ns.configure_me = cm
    finally:
        sys.path.remove(tmp)
        shutil.rmtree(tmp, ignore_errors=True)
    return ns
