"""Drop-in for plot_helper.py: the slab projection (plot_helper.py:65-72) on the GPU.

project(rho, n_slices) sums the first n_slices planes of the density grid in float64, in
plane order, as the reference's loop does (the result is bit-identical).  The plotting
functions (plot_step, plot_grf, plot_projection: matplotlib figures) are not part of the
engine.
"""
import numpy as np
import torch

_ctx = {}


def _context(n):
    from pmgpu.config import Config
    from pmgpu.context import PMContext
    if n not in _ctx:
        _ctx[n] = PMContext(Config(n_cells=n, n_parts=max(1, n // 2)))
    return _ctx[n]


def project(rho, n_slices):
    n = rho.shape[0]
    ctx = _context(n)
    on_host = not isinstance(rho, torch.Tensor)
    r = torch.from_numpy(np.ascontiguousarray(rho, dtype=np.float32)).cuda() if on_host else rho
    out = ctx.project(r, int(n_slices))
    return out.cpu().numpy() if on_host else out
