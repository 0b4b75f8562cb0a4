"""Serving loop: simulation requests admitted by HBM footprint, stepped together.

A request is (seed, N_PARTS, box, steps) on a 2 N_PARTS grid.  Its initial conditions are
made on the host by a pool of worker processes as soon as it arrives; once they are ready
and its footprint fits under the memory cap, it joins the resident batch (continuous
batching: requests that arrive while others run are admitted as slots and memory free
up).  The batch advances all resident simulations together, a few steps per tick; a
finished simulation leaves the batch at once and its memory admits the next request.
Latency = completion time - arrival time (initial conditions, queueing and stepping).
"""
from __future__ import annotations

import concurrent.futures as cf
import dataclasses
import multiprocessing as mp
import time

import numpy as np

from ._lib import PM_ERR_ADMIT, PMError
from .config import Config, step_count


@dataclasses.dataclass
class Request:
    rid: int
    seed: int
    n_parts: int
    box: float
    steps: int
    arrival: float  # seconds from the start of the stream

    def config(self) -> Config:
        return Config(n_parts=self.n_parts, n_cells=2 * self.n_parts, box_size=self.box,
                      random_seed=self.seed, steps=self.steps)

    @property
    def particle_updates(self) -> int:
        c = self.config()
        return c.np_total * step_count(c.a_init, c.a_end, c.steps)


def poisson_stream(rate: float, duration: float, seed: int = 0, sizes=(64, 96, 128, 192, 256),
                   weights=(0.40, 0.25, 0.20, 0.10, 0.05), box=(100.0, 500.0), steps=(50, 500)):
    """Seeded request stream: Poisson arrivals at `rate`/s for `duration` s."""
    rng = np.random.default_rng(seed)
    t, out, rid = 0.0, [], 0
    while True:
        t += rng.exponential(1.0 / rate)
        if t >= duration:
            return out
        n = int(rng.choice(sizes, p=np.asarray(weights) / np.sum(weights)))
        out.append(Request(rid, int(rng.integers(0, 2 ** 31 - 1)), n, float(rng.uniform(*box)),
                           int(rng.integers(steps[0], steps[1] + 1)), t))
        rid += 1


def _make_ics(req: Request):
    from .ics import initial_conditions
    return req.rid, initial_conditions(req.config())


@dataclasses.dataclass
class Result:
    rid: int
    arrival: float
    admitted: float
    completed: float
    particle_updates: int

    @property
    def latency(self) -> float:
        return self.completed - self.arrival


class Server:
    """Runs a request stream against one GPU in real time."""

    def __init__(self, mem_cap_bytes: int, ic_workers: int = 8, steps_per_tick: int = 4, device: int = 0,
                 keep_results: bool = False):
        from .batch import Batch
        self.batch = Batch(device=device, mem_cap_bytes=mem_cap_bytes)
        self.cap = mem_cap_bytes
        self.steps_per_tick = steps_per_tick
        self.pool = cf.ProcessPoolExecutor(max_workers=ic_workers, mp_context=mp.get_context("spawn"))
        self.keep_results = keep_results
        self.outputs = {}

    def close(self):
        self.pool.shutdown(wait=False, cancel_futures=True)
        self.batch.close()

    def run(self, stream: list[Request], time_limit: float | None = None) -> list[Result]:
        from .batch import Batch
        t0 = time.perf_counter()
        now = lambda: time.perf_counter() - t0  # noqa: E731
        pending = sorted(stream, key=lambda r: r.arrival)
        futures = {}
        ready = {}        # rid -> (positions, velocities)
        queued = []       # arrived requests, in arrival order
        active = {}       # sim id -> (request, admitted time)
        results = []
        nxt = 0
        while nxt < len(pending) or queued or active:
            t = now()
            if time_limit is not None and t > time_limit:
                break
            while nxt < len(pending) and pending[nxt].arrival <= t:
                r = pending[nxt]
                futures[self.pool.submit(_make_ics, r)] = r
                queued.append(r)
                nxt += 1
            for fu in [f for f in futures if f.done()]:
                rid, ic = fu.result()
                ready[rid] = ic
                del futures[fu]
            # admit in arrival order while memory allows (no overtaking of a request that fits)
            while queued and queued[0].rid in ready:
                r = queued[0]
                fp = Batch.footprint(r.config())
                try:
                    sid = self.batch.add(r.config(), *ready[r.rid])
                except PMError as e:  # refused: over the memory cap -> wait for memory to free up
                    if e.code != PM_ERR_ADMIT:
                        raise
                    if fp > self.cap:
                        raise RuntimeError(f"request {r.rid} alone exceeds the memory cap") from e
                    break
                del ready[r.rid]
                queued.pop(0)
                active[sid] = (r, now())
            if active:
                self.batch.step(self.steps_per_tick)
                for sid in list(active):
                    if not self.batch.active(sid):
                        r, ta = active.pop(sid)
                        if self.keep_results:
                            self.outputs[r.rid] = self.batch.get(sid)[:2]
                        self.batch.remove(sid)
                        results.append(Result(r.rid, r.arrival, ta, now(), r.particle_updates))
            else:
                time.sleep(0.001)
        self.batch.check_device()
        return results


def summarize(results: list[Result], wall: float) -> dict:
    lat = np.array([r.latency for r in results]) if results else np.array([np.nan])
    pu = sum(r.particle_updates for r in results)
    return {"requests": len(results), "p50_latency_s": float(np.percentile(lat, 50)),
            "p99_latency_s": float(np.percentile(lat, 99)), "mean_latency_s": float(np.mean(lat)),
            "particle_updates": int(pu), "wall_s": wall, "particle_updates_per_s": pu / wall if wall > 0 else 0.0}
