"""Host checks of the arithmetic identities the fused deposit relies on to stay bit-identical
when its code is reorganised (csrc/pm_deposit.cuh).  float32 numpy arithmetic rounds every
operation as the GPU's FP32 pipe does without contraction (the products below have no adds)."""
import numpy as np
import pytest

NRUN = 7


def cic_weights_scaled(fx, fy, fz, q):
    """cic_weights then times q (the order of integrate.py:44-51), float32."""
    f32 = np.float32
    tx, ty, tz = f32(1) - fx, f32(1) - fy, f32(1) - fz
    w = [tx * ty * tz, fx * ty * tz, tx * fy * tz, tx * ty * fz,
         fx * fy * tz, fx * ty * fz, tx * fy * fz, fx * fy * fz]
    return [wk * q for wk in w]


def prescaled_weights(fx, fy, fz, q):
    """quantised_weights: the x factor scaled by q first."""
    f32 = np.float32
    tx, xf = (f32(1) - fx) * q, fx * q
    ty, tz = f32(1) - fy, f32(1) - fz
    return [tx * ty * tz, xf * ty * tz, tx * fy * tz, tx * ty * fz,
            xf * fy * tz, xf * ty * fz, tx * fy * fz, xf * fy * fz]


@pytest.mark.parametrize("s", [0, 1, 12, 20, 23, 26])
def test_power_of_two_prescale_matches_scaled_weights(s):
    """Scaling by q = 2^s is exact, so (a q) b c == ((a b) c) q bit for bit."""
    rng = np.random.default_rng(s)
    n = 200_000
    f = rng.random((3, n), dtype=np.float32)
    # offsets as the engine makes them: exact zeros and values near 1 included
    f[:, :1000] = 0
    f[:, 1000:2000] = np.nextafter(np.float32(1), np.float32(0))
    q = np.float32(2.0 ** s)
    a = cic_weights_scaled(f[0], f[1], f[2], q)
    b = prescaled_weights(f[0], f[1], f[2], q)
    for k in range(8):
        assert a[k].dtype == np.float32 and b[k].dtype == np.float32
        assert np.array_equal(a[k].view(np.uint32), b[k].view(np.uint32)), k


def slot_search(off, begin, f):
    """RunTable::slot (binary search over the run offsets), without the permutation."""
    r = 0
    if off[4] <= f:
        r = 4
    if off[r + 2] <= f:
        r += 2
    if r + 1 < NRUN and off[r + 1] <= f:
        r += 1
    return (begin[r] + (f - off[r])) & 0xFFFFFFFF


def slot_select(off, begin, f):
    """RunRegs::slot (last run starting at or before f, by selects), without the permutation."""
    delta = [(begin[r] - off[r]) & 0xFFFFFFFF for r in range(NRUN)]
    d = delta[0]
    for r in range(1, NRUN):
        if f >= off[r]:
            d = delta[r]
    return (f + d) & 0xFFFFFFFF


def test_run_lookup_by_selects_matches_search():
    """Both lookups give every source entry of a tile the same place, empty runs included."""
    rng = np.random.default_rng(7)
    for trial in range(300):
        cnt = rng.integers(0, 40, NRUN)
        cnt[rng.random(NRUN) < 0.3] = 0  # empty runs
        off = [0] + list(np.cumsum(cnt))
        begin = [int(b) for b in rng.integers(0, 1 << 31, NRUN)]
        total = off[NRUN]
        for f in range(total):
            assert slot_search(off, begin, f) == slot_select(off, begin, f), (trial, f)
