"""The serving loop's host logic (pmgpu/serve.py) on CPU: admission in arrival order by memory
footprint, no overtaking, waiting for memory, finished simulations leaving at once, and the
latency summary.  The batch engine and the initial-conditions pool are replaced by fakes that
keep the same contract (admits / add / step / active / remove; submit -> done future)."""
import concurrent.futures as cf

import numpy as np
import pytest

from pmgpu import serve
from pmgpu.serve import Request, Server, summarize


def footprint(cfg):
    return cfg.n_parts ** 3  # "bytes": proportional to the particle count


class FakeBatch:
    def __init__(self, cap):
        self.cap, self.used, self.sims, self.next_id = cap, 0, {}, 0
        self.admit_log, self.max_used, self.steps = [], 0, 0

    def admits(self, cfg):
        return self.used + footprint(cfg) <= self.cap

    def add(self, cfg, positions, velocities):
        assert self.admits(cfg)
        sid = self.next_id
        self.next_id += 1
        self.sims[sid] = [cfg, cfg.steps]
        self.used += footprint(cfg)
        self.max_used = max(self.max_used, self.used)
        self.admit_log.append(cfg.random_seed)
        return sid

    def step(self, n):
        self.steps += n
        for s in self.sims.values():
            s[1] = max(0, s[1] - n)

    def active(self, sid):
        return self.sims[sid][1] > 0

    def get(self, sid, device=False):
        return None, None, 0.0, 0

    def remove(self, sid):
        self.used -= footprint(self.sims.pop(sid)[0])

    def check_device(self):
        pass


class SyncPool:
    """submit() runs at once; the initial conditions are stand-in arrays."""

    def submit(self, fn, r, pairs_only):
        f = cf.Future()
        f.set_result((r.rid, (np.zeros((3, 1), np.float32), np.zeros((3, 1), np.float32))))
        return f

    def shutdown(self, **kw):
        pass


def make_server(cap, steps_per_tick=4):
    s = object.__new__(Server)
    s.batch = FakeBatch(cap)
    s.device, s.device_ics, s._ics, s._ic_stream = 0, False, {}, None
    s.pk, s._ctx, s.cap, s.steps_per_tick = False, {}, cap, steps_per_tick
    s.pool, s.keep_results, s.outputs = SyncPool(), False, {}
    return s


@pytest.fixture(autouse=True)
def fake_footprint(monkeypatch):
    import pmgpu.batch
    monkeypatch.setattr(pmgpu.batch.Batch, "footprint", staticmethod(footprint))


def req(rid, n, steps, seed=None):
    return Request(rid, rid if seed is None else seed, n, 100.0, steps, 0.0)


def test_admission_respects_the_cap_and_arrival_order():
    s = make_server(cap=2 * 32 ** 3)
    stream = [req(i, 32, 8 + 4 * i) for i in range(5)]
    res = s.run(stream)
    assert sorted(r.rid for r in res) == list(range(5))
    assert s.batch.admit_log == [0, 1, 2, 3, 4]            # arrival order
    assert s.batch.max_used <= 2 * 32 ** 3                 # never over the cap
    assert all(r.completed >= r.admitted >= r.arrival for r in res)
    assert s.batch.sims == {} and s.batch.used == 0        # finished simulations left the batch


def test_no_overtaking_of_a_request_that_waits_for_memory():
    # a small request runs; the big one fits only alone, so the small ones behind it wait
    s = make_server(cap=48 ** 3)
    stream = [req(0, 16, 40), req(1, 48, 8), req(2, 16, 8), req(3, 16, 8)]
    res = s.run(stream)
    assert s.batch.admit_log == [0, 1, 2, 3]
    done = {r.rid: r for r in res}
    assert done[2].admitted >= done[1].admitted and done[3].admitted >= done[1].admitted
    assert s.batch.max_used <= 48 ** 3


def test_a_request_larger_than_the_cap_is_refused():
    s = make_server(cap=16 ** 3)
    with pytest.raises(RuntimeError, match="exceeds the memory cap"):
        s.run([req(0, 32, 4)])


def test_summary_of_results():
    s = make_server(cap=4 * 16 ** 3, steps_per_tick=2)
    res = s.run([req(i, 16, 6) for i in range(3)])
    out = summarize(res, wall=2.0)
    assert out["requests"] == 3
    assert out["particle_updates"] == sum(r.particle_updates for r in res)
    assert out["particle_updates_per_s"] == pytest.approx(out["particle_updates"] / 2.0)
    assert 0 <= out["p50_latency_s"] <= out["p99_latency_s"]


def test_poisson_stream_is_seeded_and_within_bounds():
    a = serve.poisson_stream(20.0, 5.0, seed=3)
    b = serve.poisson_stream(20.0, 5.0, seed=3)
    assert [(r.seed, r.n_parts, r.box, r.steps, r.arrival) for r in a] == \
           [(r.seed, r.n_parts, r.box, r.steps, r.arrival) for r in b]
    assert all(r.n_parts in (64, 96, 128, 192, 256) and 100.0 <= r.box <= 500.0 and 50 <= r.steps <= 500
               for r in a)
    assert all(0 < x.arrival < y.arrival < 5.0 for x, y in zip(a, a[1:]))
    assert 40 < len(a) < 160  # about rate x duration = 100
