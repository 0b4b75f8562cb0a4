"""Python face of a pm_ctx: the reference's per-step functions on device tensors.

Every method takes and returns torch CUDA tensors (float32, C-contiguous) in the
reference's layouts -- positions/velocities (3, Np), grids (N, N, N) indexed [z, y, x].
Work is enqueued on the current torch stream.  There is no CPU path: a missing library
or a tensor that is not on a CUDA device raises.
"""
from __future__ import annotations

import ctypes

import torch

from . import _lib
from .config import Config


def _stream_ptr():
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


def _ptr(t):
    return ctypes.c_void_p(t.data_ptr()) if t is not None else None


def _need(t: torch.Tensor, name: str, shape=None, dtype=torch.float32):
    if not isinstance(t, torch.Tensor) or t.device.type != "cuda":
        raise TypeError(f"{name} must be a CUDA tensor")
    if t.dtype != dtype:
        raise TypeError(f"{name} must be {dtype}, got {t.dtype}")
    if not t.is_contiguous():
        raise ValueError(f"{name} must be contiguous")
    if shape is not None and tuple(t.shape) != tuple(shape):
        raise ValueError(f"{name} must have shape {tuple(shape)}, got {tuple(t.shape)}")
    return t


class PMContext:
    """One simulation geometry (N_CELLS) and cosmology on one GPU."""

    def __init__(self, cfg: Config, device: int = 0):
        self.cfg = cfg
        self.n = cfg.n_cells
        self.device = device
        self._lib = _lib.load()
        if not self._lib.pm_supported_n(self.n):
            raise ValueError(f"N_CELLS={self.n} is not supported (2^a 3^b, 16..1024)")
        torch.cuda.init()
        with torch.cuda.device(device):
            h = ctypes.c_void_p()
            rc = self._lib.pm_ctx_create(ctypes.byref(cfg.c_struct()), device, ctypes.byref(h))
            if rc != 0:
                raise _lib.PMError(rc, "pm_ctx_create failed")
        self._h = h

    def close(self):
        if getattr(self, "_h", None):
            self._lib.pm_ctx_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # -------------------------------------------------------------------------------
    def _check(self, rc: int):
        if rc != 0:
            msg = self._lib.pm_last_error(self._h).decode(errors="replace")
            raise _lib.PMError(rc, msg)

    def check_device(self):
        """Synchronise and raise if a kernel flagged a bad particle (NaN, off-grid)."""
        bits = ctypes.c_int(0)
        rc = self._lib.pm_check_device(self._h, _stream_ptr(), ctypes.byref(bits))
        if rc != 0:
            what = [v for k, v in _lib.DEVICE_BITS.items() if bits.value & k]
            raise _lib.PMError(rc, "device check failed: " + "; ".join(what))

    def grid(self) -> torch.Tensor:
        return torch.empty((self.n,) * 3, dtype=torch.float32, device=f"cuda:{self.device}")

    # ---- reference functions --------------------------------------------------------
    def density(self, positions: torch.Tensor, mass: float, out: torch.Tensor | None = None) -> torch.Tensor:
        """density.py:7-48."""
        _need(positions, "positions")
        np_ = positions.shape[1]
        _need(positions, "positions", (3, np_))
        rho = out if out is not None else self.grid()
        _need(rho, "rho", (self.n,) * 3)
        self._check(self._lib.pm_density(self._h, _ptr(positions), np_, float(mass), _ptr(rho), _stream_ptr()))
        return rho

    def fourier_grid(self) -> torch.Tensor:
        """fourier_utils.py:5-16 (k = 0 entry is 0)."""
        g = self.grid()
        self._check(self._lib.pm_fourier_grid(self._h, _ptr(g), _stream_ptr()))
        return g

    def potential(self, density: torch.Tensor, fgrid: torch.Tensor | None, a: float,
                  out: torch.Tensor | None = None) -> torch.Tensor:
        """potential.py:7-29.  fgrid=None evaluates the reference Green function in-kernel."""
        _need(density, "density", (self.n,) * 3)
        if fgrid is not None:
            _need(fgrid, "fgrid", (self.n,) * 3)
        phi = out if out is not None else self.grid()
        self._check(self._lib.pm_potential(self._h, _ptr(density), _ptr(fgrid), float(a), _ptr(phi),
                                           _stream_ptr()))
        return phi

    def project(self, density: torch.Tensor, n_slices: int) -> torch.Tensor:
        """plot_helper.py:65-72: sum of the first n_slices planes, float64 (N, N)."""
        _need(density, "density", (self.n,) * 3)
        out = torch.empty((self.n, self.n), dtype=torch.float64, device=density.device)
        self._check(self._lib.pm_project(self._h, _ptr(density), int(n_slices), _ptr(out), _stream_ptr()))
        return out

    def power_spectrum(self, density: torch.Tensor, box_size: float | None = None, nbins: int = 0):
        """Shell-averaged P(k) of a density grid: (k [h/Mpc], P [(Mpc/h)^3], modes) as numpy
        float64 arrays of nbins - 1 shells (nbins = 0: N/2 + 1).  Same estimator as the
        oracle's power_spectrum; no counterpart in the reference."""
        import numpy as np
        _need(density, "density", (self.n,) * 3)
        nb = (self.n // 2 + 1 if nbins <= 0 else nbins) - 1
        k, p, m = (np.zeros(max(nb, 0), dtype=np.float64) for _ in range(3))
        box = float(self.cfg.box_size if box_size is None else box_size)
        self._check(self._lib.pm_power_spectrum(self._h, _ptr(density), box, int(nbins), k.ctypes.data,
                                                p.ctypes.data, m.ctypes.data, _stream_ptr()))
        return k, p, m

    def integrate(self, positions, velocities, a_val, f_a1, da, potentials):
        """integrate.py:15-97 (in place)."""
        _need(positions, "positions")
        np_ = positions.shape[1]
        _need(positions, "positions", (3, np_))
        _need(velocities, "velocities", (3, np_))
        _need(potentials, "potentials", (self.n,) * 3)
        self._check(self._lib.pm_integrate(self._h, _ptr(positions), _ptr(velocities), np_, float(a_val),
                                           float(f_a1), float(da), _ptr(potentials), _stream_ptr()))
        return positions, velocities

    def advance_time(self, density, positions, velocities, fgrid, a, da):
        """integrate.py:9-13 (in place)."""
        _need(density, "density", (self.n,) * 3)
        _need(positions, "positions")
        np_ = positions.shape[1]
        _need(velocities, "velocities", (3, np_))
        if fgrid is not None:
            _need(fgrid, "fgrid", (self.n,) * 3)
        self._check(self._lib.pm_advance_time(self._h, _ptr(density), _ptr(positions), _ptr(velocities), np_,
                                              _ptr(fgrid), float(a), float(da), _stream_ptr()))
        return positions, velocities

    def step(self, positions, velocities, mass, a, da, rho_out: torch.Tensor | None = None):
        """pmesh.py:60-61: density then advance_time with the built-in Green function."""
        _need(positions, "positions")
        np_ = positions.shape[1]
        _need(velocities, "velocities", (3, np_))
        if rho_out is not None:
            _need(rho_out, "rho_out", (self.n,) * 3)
        self._check(self._lib.pm_step(self._h, _ptr(positions), _ptr(velocities), np_, float(mass), float(a),
                                      float(da), _ptr(rho_out), _stream_ptr()))
        return positions, velocities

    def step_host(self, positions, velocities, mass, a, da):
        """pm_step on host (numpy or pinned torch CPU) arrays, updated in place; synchronous."""
        np_ = positions.shape[1]
        pp = ctypes.c_void_p(positions.data_ptr() if isinstance(positions, torch.Tensor)
                             else positions.ctypes.data)
        vp = ctypes.c_void_p(velocities.data_ptr() if isinstance(velocities, torch.Tensor)
                             else velocities.ctypes.data)
        self._check(self._lib.pm_step_host(self._h, pp, vp, np_, float(mass), float(a), float(da),
                                           _stream_ptr()))
        return positions, velocities

    def sort_keys(self, positions):
        """Cell keys of the deposit ordering, their stable sort and the permutation."""
        _need(positions, "positions")
        np_ = positions.shape[1]
        dev = positions.device
        keys = torch.empty(np_, dtype=torch.int32, device=dev)
        skeys = torch.empty(np_, dtype=torch.int32, device=dev)
        perm = torch.empty(np_, dtype=torch.int32, device=dev)
        self._check(self._lib.pm_sort_keys(self._h, _ptr(positions), np_, _ptr(keys), _ptr(skeys), _ptr(perm),
                                           _stream_ptr()))
        return keys, skeys, perm
