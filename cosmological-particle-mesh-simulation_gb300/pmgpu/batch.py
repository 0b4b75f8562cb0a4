"""Resident batch engine: many simulations advancing together on one GPU."""
from __future__ import annotations

import ctypes

import numpy as np
import torch

from . import _lib
from .config import Config


class Batch:
    """Wraps pm_batch_*.  Simulations are admitted from absolute (3, N_PARTS^3) float32
    positions / velocities (numpy on the host or CUDA tensors) and advance together."""

    def __init__(self, device: int = 0, mem_cap_bytes: int = 0, graphs: bool = True, autotune: bool = True):
        self._lib = _lib.load()
        self.device = device
        torch.cuda.init()
        h = ctypes.c_void_p()
        with torch.cuda.device(device):
            rc = self._lib.pm_batch_create(device, int(mem_cap_bytes), ctypes.byref(h))
        if rc != 0:
            raise _lib.PMError(rc, "pm_batch_create failed")
        self._h = h
        self.cfgs: dict[int, Config] = {}
        if not graphs:
            self._lib.pm_batch_set_graphs(self._h, 0)
        if not autotune:
            self._lib.pm_batch_set_autotune(self._h, 0)

    def close(self):
        if getattr(self, "_h", None):
            self._lib.pm_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, rc):
        if rc != 0:
            raise _lib.PMError(rc, self._lib.pm_batch_last_error(self._h).decode(errors="replace"))

    @staticmethod
    def footprint(cfg: Config) -> int:
        return int(_lib.load().pm_sim_footprint(ctypes.byref(cfg.c_struct())))

    def admits(self, cfg: Config) -> bool:
        """Whether add(cfg, ...) would pass the memory cap now."""
        return bool(self._lib.pm_batch_admits(self._h, ctypes.byref(cfg.c_struct())))

    def add(self, cfg: Config, positions, velocities) -> int:
        on_dev = isinstance(positions, torch.Tensor) and positions.is_cuda
        if on_dev:
            positions = positions.contiguous()
            velocities = velocities.contiguous()
            pp, vp = positions.data_ptr(), velocities.data_ptr()
        else:
            positions = np.ascontiguousarray(positions, dtype=np.float32)
            velocities = np.ascontiguousarray(velocities, dtype=np.float32)
            pp, vp = positions.ctypes.data, velocities.ctypes.data
        sid = ctypes.c_int(0)
        self._check(self._lib.pm_batch_add(self._h, ctypes.byref(cfg.c_struct()), ctypes.c_void_p(pp),
                                           ctypes.c_void_p(vp), 1 if on_dev else 0, ctypes.byref(sid)))
        self.cfgs[sid.value] = cfg
        return sid.value

    def step(self, nsteps: int = 1):
        stream = torch.cuda.current_stream().cuda_stream
        self._check(self._lib.pm_batch_step(self._h, int(nsteps), ctypes.c_void_p(stream)))

    def mark(self):
        """A CUDA event recorded after the work enqueued so far (on the current stream)."""
        ev = torch.cuda.Event()
        ev.record()
        return ev

    def active(self, sid: int) -> bool:
        r = self._lib.pm_batch_active(self._h, sid)
        if r < 0:
            raise KeyError(sid)
        return r == 1

    def get(self, sid: int, device: bool = False):
        cfg = self.cfgs[sid]
        npart = cfg.np_total
        a = ctypes.c_double(0)
        done = ctypes.c_int(0)
        stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
        if device:
            pos = torch.empty((3, npart), dtype=torch.float32, device=f"cuda:{self.device}")
            vel = torch.empty_like(pos)
            self._check(self._lib.pm_batch_get(self._h, sid, ctypes.c_void_p(pos.data_ptr()),
                                               ctypes.c_void_p(vel.data_ptr()), 1, ctypes.byref(a),
                                               ctypes.byref(done), stream))
        else:
            pos = np.empty((3, npart), dtype=np.float32)
            vel = np.empty_like(pos)
            self._check(self._lib.pm_batch_get(self._h, sid, ctypes.c_void_p(pos.ctypes.data),
                                               ctypes.c_void_p(vel.ctypes.data), 0, ctypes.byref(a),
                                               ctypes.byref(done), stream))
        return pos, vel, a.value, done.value

    def density(self, sid: int, out=None):
        """CIC density (N_CELLS^3 float32 CUDA tensor) of a resident simulation's current state."""
        n = self.cfgs[sid].n_cells
        if out is None:
            out = torch.empty((n, n, n), dtype=torch.float32, device=f"cuda:{self.device}")
        stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
        self._check(self._lib.pm_batch_density(self._h, sid, ctypes.c_void_p(out.data_ptr()), stream))
        return out

    def state(self, sid: int):
        a = ctypes.c_double(0)
        done = ctypes.c_int(0)
        self._check(self._lib.pm_batch_get(self._h, sid, None, None, 0, ctypes.byref(a), ctypes.byref(done),
                                           None))
        return a.value, done.value

    def remove(self, sid: int):
        self._check(self._lib.pm_batch_remove(self._h, sid))
        self.cfgs.pop(sid, None)

    def profile(self, nsteps: int) -> dict:
        """Run up to nsteps steps with CUDA events between phases; mean ms per phase."""
        arr = (ctypes.c_float * len(_lib.PROFILE_PHASES))()
        stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
        self._check(self._lib.pm_batch_profile(self._h, int(nsteps), arr, len(arr), stream))
        return dict(zip(_lib.PROFILE_PHASES, [float(x) for x in arr]))

    def set_autotune(self, enable: bool):
        self._check(self._lib.pm_batch_set_autotune(self._h, 1 if enable else 0))

    def schedule(self) -> list:
        """The current plan's launch schedule per grid size (tuned or default) and the kick's."""
        arr = (ctypes.c_int * 256)()
        k = self._lib.pm_batch_schedule(self._h, arr, 256)
        if k < 0:
            raise _lib.PMError(k, "pm_batch_schedule failed")
        modes = {0: "fused, dense tiles first", 1: "fused, index order", 2: "separate deposit + x R2C"}
        out = []
        for i in range(0, k, 4):
            n, a, c, d = arr[i:i + 4]
            if n == 0:
                out.append({"kick_ctas_per_sm": a, "tuned": bool(c)})
            else:
                out.append({"n_cells": n, "deposit": modes.get(a, a), "deposit_ctas_per_sm": c, "x_ctas_per_sm": d})
        return out

    def host_seconds(self) -> dict:
        """Host time spent so far in admissions, planning, graph capture, retirements and tuning,
        and the time planning waited for enqueued steps (``plan_wait``, not in ``plan``)."""
        arr = (ctypes.c_double * 6)()
        self._check(self._lib.pm_batch_host_seconds(self._h, arr, 6))
        return dict(zip(("admit", "plan", "capture", "retire", "tune", "plan_wait"),
                        [round(float(x), 4) for x in arr]))

    def launches_per_step(self) -> int:
        return int(self._lib.pm_batch_launches_per_step(self._h))

    def check_device(self):
        bits = ctypes.c_int(0)
        stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
        rc = self._lib.pm_batch_check(self._h, stream, ctypes.byref(bits))
        if rc != 0:
            what = [v for k, v in _lib.DEVICE_BITS.items() if bits.value & k]
            raise _lib.PMError(rc, "device check failed: " + "; ".join(what))
