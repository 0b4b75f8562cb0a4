"""Implementation behind the drop-in modules (density.py, potential.py, integrate.py,
fourier_utils.py) that carry the reference's module and function names.

Sizes and cosmology are read from the ``configure_me`` module found on ``sys.path``,
as in the reference.  Arguments may be numpy arrays (copied to the GPU and back; the
results are numpy, and advance_time/integrate update the caller's arrays in place like
the reference does) or CUDA tensors (no copies, results are tensors).
"""
from __future__ import annotations

import numpy as np
import torch

from .config import Config
from .context import PMContext

_ctx: PMContext | None = None
_ctx_key = None


def config() -> Config:
    import configure_me  # the caller's configuration module, as in the reference
    return Config.from_module(configure_me)


def context() -> PMContext:
    """The PMContext of the current configure_me (rebuilt when it changes)."""
    global _ctx, _ctx_key
    cfg = config()
    key = (cfg.n_cells, cfg.n_parts, cfg.omega_m0, cfg.omega_lambda0, cfg.omega_k0, cfg.h0, cfg.fix_cosmo_f)
    if _ctx is None or _ctx_key != key:
        _ctx = PMContext(cfg)
        _ctx_key = key
    return _ctx


class GreenTable(np.ndarray):
    """The array fourier_grid() returns: the reference's table (read-only).  potential()
    recognises it and evaluates the same Green function in-kernel instead of reading it."""

    _pm_builtin = True


def _dev(a):
    if isinstance(a, torch.Tensor) and a.is_cuda:
        return a, False
    return torch.from_numpy(np.ascontiguousarray(np.asarray(a), dtype=np.float32)).cuda(), True


def density(positions, mass):
    """density.py:7-48."""
    p, host = _dev(positions)
    rho = context().density(p, mass)
    return rho.cpu().numpy() if host else rho


def fourier_grid():
    """fourier_utils.py:5-16 (k = 0 entry 0)."""
    g = context().fourier_grid().cpu().numpy().view(GreenTable)
    g.flags.writeable = False
    return g


def _green(fgrid):
    if fgrid is None or getattr(fgrid, "_pm_builtin", False):
        return None
    return _dev(fgrid)[0]


def potential(density, fgrid, a):
    """potential.py:7-29."""
    d, host = _dev(density)
    phi = context().potential(d, _green(fgrid), a)
    return phi.cpu().numpy() if host else phi


def _write_back(dst, src):
    if isinstance(dst, np.ndarray):
        dst[...] = src.cpu().numpy()


def integrate(positions, velocities, a_val, f_a1, da, potentials):
    """integrate.py:15-97, in place."""
    p, hp = _dev(positions)
    v, hv = _dev(velocities)
    phi, _ = _dev(potentials)
    context().integrate(p, v, a_val, f_a1, da, phi)
    if hp:
        _write_back(positions, p)
    if hv:
        _write_back(velocities, v)
    return positions, velocities


def advance_time(density, positions, velocities, fgrid, a, da):
    """integrate.py:9-13, in place."""
    d, _ = _dev(density)
    p, hp = _dev(positions)
    v, hv = _dev(velocities)
    ctx = context()
    g = _green(fgrid)
    ctx.advance_time(d, p, v, g, a, da)
    if hp:
        _write_back(positions, p)
    if hv:
        _write_back(velocities, v)
    return positions, velocities
