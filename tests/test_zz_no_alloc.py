"""pm_density_noalloc: the deposit for callers that cannot allocate device memory (hosts
whose device memory a pool or an arena has carved up, latency-critical loops that cannot take
an allocation's synchronisation, plugin hosts that supply every buffer).  It keeps its
scratch in a static device array of the library; called through the C ABI it must give the
density of pm_density (the existing entry point) and of the float64 oracle within the
parity tolerance (1e-5 relative L2), call after call, and allocate nothing once its first
call has set it up.

Kept in a file that pytest collects last, and written to pass alone in a fresh process."""
import ctypes
import gc

import numpy as np
import pytest

from conftest import rel_l2
from oracle import pm_oracle as O

pytestmark = pytest.mark.gpu

MAX_PARTICLES = 1 << 18
MAX_N = 128


def call_noalloc(lib, torch, pos, n, mass, out):
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    return lib.pm_density_noalloc(ctypes.c_void_p(pos.data_ptr()), pos.shape[1], n, mass,
                                  ctypes.c_void_p(out.data_ptr()), stream)


def test_noalloc_density_matches_pm_density(cuda):
    torch = cuda
    from pmgpu import _lib, ics
    from pmgpu.config import Config
    from pmgpu.context import PMContext
    lib = _lib.load()
    cases = [Config(n_parts=64, n_cells=128, box_size=200.0, random_seed=2),   # the maximum size
             Config(n_parts=32, n_cells=96, box_size=120.0, random_seed=9)]    # a different grid
    inputs, contexts = [], []
    for cfg in cases:
        pos, _ = ics.initial_conditions(cfg)
        p = torch.from_numpy(pos).cuda()
        ctx = PMContext(cfg)
        contexts.append(ctx)  # kept alive: freeing them would change the free-memory reading below
        ref = ctx.density(p, cfg.mass)
        out = torch.full_like(ref, -1.0)
        inputs.append((cfg, p, ref, out, pos))
    torch.cuda.synchronize()
    for cfg, p, ref, out, pos in inputs:  # two calls in a row, the second on other sizes
        assert call_noalloc(lib, torch, p, cfg.n_cells, cfg.mass, out) == 0
        torch.cuda.synchronize()
        o, r = out.cpu().numpy(), ref.cpu().numpy()
        assert rel_l2(o, r) < 1e-5
        assert np.array_equal(o, r)  # same deterministic kernels
        assert rel_l2(o, O.density(pos, cfg.mass, cfg.n_cells)) < 1e-5
    # once set up, further calls allocate nothing (and rewrite their outputs)
    for cfg, p, ref, out, pos in inputs:
        out.fill_(-1.0)
    gc.collect()
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    for cfg, p, ref, out, pos in inputs:
        assert call_noalloc(lib, torch, p, cfg.n_cells, cfg.mass, out) == 0
    torch.cuda.synchronize()
    assert torch.cuda.mem_get_info()[0] == free0
    for cfg, p, ref, out, pos in inputs:
        assert np.array_equal(out.cpu().numpy(), ref.cpu().numpy())


def test_noalloc_rejects_oversize(cuda):
    torch = cuda
    from pmgpu import _lib
    lib = _lib.load()
    pos = torch.rand((3, MAX_PARTICLES + 1), device="cuda") * 64
    out = torch.empty((MAX_N,) * 3, device="cuda")
    assert call_noalloc(lib, torch, pos, 64, 1.0, out) == _lib.PM_ERR_ARG
    small = pos[:, :1000].contiguous()
    big = torch.empty((256,) * 3, device="cuda")
    assert call_noalloc(lib, torch, small, 256, 1.0, big) == _lib.PM_ERR_ARG
