"""Resident batch engine: displacement storage, sorted state, CUDA graphs, many sims.

A simulation stepped inside the batch must match the same simulation stepped by the
drop-in path (absolute positions) within float32 rounding growth, and a simulation
must give the same result alone and inside a mix of others (bit-identical: every
simulation's arithmetic is independent of its neighbours in the batch)."""
import numpy as np
import pytest

from conftest import golden_config, load_golden, periodic_maxdiff, rel_l2
from oracle import pm_oracle as O

pytestmark = pytest.mark.gpu


def small_cfg(n_parts, seed, box=100.0, steps=50):
    from pmgpu.config import Config
    return Config(n_parts=n_parts, n_cells=2 * n_parts, box_size=box, random_seed=seed, steps=steps)


def test_batch_matches_reference_fixture(cuda):
    from pmgpu.batch import Batch
    f, c = load_golden("n16_g32")
    cfg = golden_config(c)
    b = Batch()
    sid = b.add(cfg, f["pos0"], f["vel0"])
    for s in range(c["steps"]):
        b.step(1)
        pos, vel, a, done = b.get(sid)
        b.check_device()
        assert done == s + 1
        assert a == pytest.approx(f["a"][s + 1], rel=1e-14)
        assert rel_l2(vel, f[f"vel{s + 1}"]) < 1e-4
        assert periodic_maxdiff(pos, f[f"pos{s + 1}"], cfg.n_cells) < 1e-3


def test_batch_vs_dropin_many_steps(cuda):
    torch = cuda
    from pmgpu.batch import Batch
    from pmgpu.context import PMContext
    from pmgpu import ics
    cfg = small_cfg(32, 3, box=150.0, steps=100)
    pos, vel = ics.initial_conditions(cfg)
    b = Batch()
    sid = b.add(cfg, pos, vel)
    b.step(20)
    bp, bv, a, done = b.get(sid)
    b.check_device()
    ctx = PMContext(cfg)
    p, v = torch.from_numpy(pos).cuda(), torch.from_numpy(vel).cuda()
    aa = cfg.a_init
    for _ in range(20):
        ctx.step(p, v, cfg.mass, aa, cfg.da)
        aa += cfg.da
    ctx.check_device()
    assert done == 20 and a == pytest.approx(aa, rel=1e-14)
    # displacement storage is more precise than absolute float32 positions: small drift
    assert periodic_maxdiff(bp, p.cpu().numpy(), cfg.n_cells) < 5e-3
    assert rel_l2(bv, v.cpu().numpy()) < 1e-3


def test_alone_equals_in_mix(cuda):
    from pmgpu.batch import Batch
    from pmgpu import ics
    cfgs = [small_cfg(16, 1), small_cfg(24, 2, box=200.0), small_cfg(32, 3), small_cfg(16, 4, box=60.0),
            small_cfg(12, 5, box=80.0)]
    ics_ = [ics.initial_conditions(c) for c in cfgs]
    alone = []
    for c, (p, v) in zip(cfgs, ics_):
        b = Batch()
        sid = b.add(c, p, v)
        b.step(7)
        alone.append(b.get(sid)[:2])
        b.close()
    b = Batch()
    ids = [b.add(c, p, v) for c, (p, v) in zip(cfgs, ics_)]
    b.step(7)
    b.check_device()
    for sid, (pa, va) in zip(ids, alone):
        pm, vm, _, _ = b.get(sid)
        assert np.array_equal(pa, pm)
        assert np.array_equal(va, vm)


def test_graphs_equal_direct_launches(cuda):
    from pmgpu.batch import Batch
    from pmgpu import ics
    c = small_cfg(32, 9)
    p, v = ics.initial_conditions(c)
    out = []
    for graphs in (True, False):
        b = Batch(graphs=graphs)
        sid = b.add(c, p, v)
        b.step(5)
        out.append(b.get(sid)[:2])
    assert np.array_equal(out[0][0], out[1][0]) and np.array_equal(out[0][1], out[1][1])


def test_retire_and_admission(cuda):
    from pmgpu.batch import Batch
    from pmgpu import PMError
    from pmgpu import ics
    c1 = small_cfg(16, 1, steps=5)   # 4 loop steps (pmesh.py:56)
    c2 = small_cfg(16, 2, steps=12)
    b = Batch(mem_cap_bytes=Batch.footprint(c1) + Batch.footprint(c2) + 1024)
    s1 = b.add(c1, *ics.initial_conditions(c1))
    s2 = b.add(c2, *ics.initial_conditions(c2))
    with pytest.raises(PMError):
        b.add(small_cfg(16, 3), *ics.initial_conditions(small_cfg(16, 3)))
    b.step(100)
    cuda.cuda.synchronize()  # active() reports a simulation done once its last steps have run
    assert not b.active(s1) and not b.active(s2)
    assert b.state(s1)[1] == O.step_count(c1.a_init, c1.a_end, c1.steps)
    assert b.state(s2)[1] == O.step_count(c2.a_init, c2.a_end, c2.steps)
    b.remove(s1)
    b.remove(s2)
    s3 = b.add(small_cfg(16, 3), *ics.initial_conditions(small_cfg(16, 3)))
    assert b.active(s3)


def test_autotuned_schedules_give_identical_results(cuda):
    """The autotuner times its candidate schedules (deposit fused with dense tiles first or in
    index order, or separate; CTAs per SM of the deposit, the x passes and the kick) on the
    batch's own data between steps and keeps the fastest.  Every candidate, and the trials
    themselves, leave the results bit-identical: a tuned batch and an untuned one end in the
    same state."""
    from pmgpu.batch import Batch
    from pmgpu import ics
    cfgs = [small_cfg(32, 11, box=150.0), small_cfg(16, 12), small_cfg(24, 13, box=90.0)]
    ics_ = [ics.initial_conditions(c) for c in cfgs]
    out = {}
    for tune in (True, False):
        b = Batch(autotune=tune)
        ids = [b.add(c, p, v) for c, (p, v) in zip(cfgs, ics_)]
        b.step(6)
        b.check_device()
        sched = b.schedule()
        out[tune] = [b.get(i)[:2] for i in ids]
        b.close()
        sizes = sorted(e["n_cells"] for e in sched if "n_cells" in e)
        assert sizes == [32, 48, 64]
        kick = [e for e in sched if "kick_ctas_per_sm" in e]
        assert len(kick) == 1 and kick[0]["kick_ctas_per_sm"] in (4, 8, 16, 32)
        if tune:
            assert kick[0]["tuned"]
    for (p1, v1), (p2, v2) in zip(out[True], out[False]):
        assert np.array_equal(p1, p2) and np.array_equal(v1, v2)


def test_retired_simulation_leaves_without_disturbing_the_others(cuda):
    """A simulation that finishes leaves the batch without a copy of the others' state: its
    slots stay empty for one step (no keys, skipped by the sort) and the next kick writes the
    survivors back compactly.  The survivors' states are those of a batch without it, and a
    simulation admitted afterwards runs as it would alone."""
    from pmgpu.batch import Batch
    from pmgpu import ics
    short, long_, late = small_cfg(16, 21, steps=5), small_cfg(24, 22, steps=40), small_cfg(16, 23, steps=40)
    ic = {c.random_seed: ics.initial_conditions(c) for c in (short, long_, late)}
    b = Batch()
    s_short = b.add(short, *ic[21])
    s_long = b.add(long_, *ic[22])
    b.step(6)   # the short one runs its 4 steps and leaves
    s_late = b.add(late, *ic[23])
    b.step(9)
    b.check_device()
    cuda.cuda.synchronize()
    assert not b.active(s_short) and b.active(s_long) and b.active(s_late)
    got_long, got_late = b.get(s_long)[:2], b.get(s_late)[:2]
    assert b.state(s_short)[1] == O.step_count(short.a_init, short.a_end, short.steps)
    b.close()
    alone = Batch()
    a = alone.add(long_, *ic[22])
    alone.step(15)
    ref_long = alone.get(a)[:2]
    alone.close()
    alone = Batch()
    a = alone.add(late, *ic[23])
    alone.step(9)
    ref_late = alone.get(a)[:2]
    alone.close()
    for got, ref in ((got_long, ref_long), (got_late, ref_late)):
        assert np.array_equal(got[0], ref[0]) and np.array_equal(got[1], ref[1])
