"""Initial conditions on the GPU (pm_ics_*): src/gaussian_random_field.py:9-123 and
src/zeldovich.py:10-100 with the same random streams as the host path (pmgpu/ics.py).

The host draws only the accepted uniform pairs of the rejection loop (numpy RandomState,
the reference's stream); Box-Muller, the power spectrum, the five transforms and the
Zel'dovich step run on the device.  Results are float32 CUDA tensors.
"""
from __future__ import annotations

import ctypes

import numpy as np
import torch

from . import _lib
from .config import Config
from .ics import jitter_state, uniform_pairs


class DeviceICs:
    """Scratch and tables for one N_PARTS on one GPU; reusable across seeds and boxes."""

    def __init__(self, n_parts: int, device: int = 0):
        self._lib = _lib.load()
        self.n = n_parts
        self.device = device
        torch.cuda.init()
        h = ctypes.c_void_p()
        with torch.cuda.device(device):
            rc = self._lib.pm_ics_create(n_parts, device, ctypes.byref(h))
        if rc != 0:
            raise _lib.PMError(rc, f"pm_ics_create failed for N_PARTS={n_parts} (supported: 2^a 3^b, 16..1024)")
        self._h = h

    def close(self):
        if getattr(self, "_h", None):
            self._lib.pm_ics_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @staticmethod
    def params(cfg: Config) -> "_lib.PMICParamsC":
        (sh, sl), (ih, il) = jitter_state(cfg.random_seed)
        p = _lib.PMICParamsC()
        p.power = float(cfg.power)
        p.lcdm_transfer = 1 if cfg.lcdm_transfer_function else 0
        p.jitter_state[0], p.jitter_state[1] = sh, sl
        p.jitter_inc[0], p.jitter_inc[1] = ih, il
        return p

    def generate(self, cfg: Config, uv=None, want_grf: bool = False, stream=None):
        """(positions, velocities[, grf]) on the device for cfg (N_PARTS must match).
        uv: the accepted uniform pairs (numpy or CUDA tensors); drawn here when None."""
        if cfg.n_parts != self.n:
            raise ValueError(f"this object is for N_PARTS={self.n}, the configuration has {cfg.n_parts}")
        if uv is None:
            uv = uniform_pairs(cfg.n_parts, cfg.random_seed)
        dev = torch.device("cuda", self.device)
        u, v = (torch.as_tensor(np.asarray(a, dtype=np.float32) if not isinstance(a, torch.Tensor) else a)
                .to(dev, torch.float32).contiguous() for a in uv)
        npart = self.n ** 3
        if u.numel() != npart or v.numel() != npart:
            raise ValueError(f"uniform pairs must hold {npart} entries each")
        pos = torch.empty((3, npart), dtype=torch.float32, device=dev)
        vel = torch.empty((3, npart), dtype=torch.float32, device=dev)
        grf = torch.empty((self.n,) * 3, dtype=torch.float32, device=dev) if want_grf else None
        with torch.cuda.device(self.device):
            st = stream if stream is not None else torch.cuda.current_stream(self.device)
            rc = self._lib.pm_ics_generate(self._h, ctypes.byref(cfg.c_struct()), ctypes.byref(self.params(cfg)),
                                           ctypes.c_void_p(u.data_ptr()), ctypes.c_void_p(v.data_ptr()),
                                           ctypes.c_void_p(pos.data_ptr()), ctypes.c_void_p(vel.data_ptr()),
                                           ctypes.c_void_p(grf.data_ptr()) if grf is not None else None,
                                           ctypes.c_void_p(st.cuda_stream))
        if rc != 0:
            raise _lib.PMError(rc, self._lib.pm_ics_last_error(self._h).decode(errors="replace"))
        return (pos, vel, grf) if want_grf else (pos, vel)


def device_initial_conditions(cfg: Config, device: int = 0):
    """GRF + Zel'dovich on the GPU: (positions, velocities) CUDA tensors (3, N_PARTS^3)."""
    g = DeviceICs(cfg.n_parts, device)
    try:
        return g.generate(cfg)
    finally:
        g.close()
