"""Serving loop: simulation requests admitted by HBM footprint, stepped together.

A request is (seed, N_PARTS, box, steps) on a 2 N_PARTS grid.  As soon as it arrives a
pool of worker processes draws its random stream on the host: the accepted uniform pairs
of the reference's rejection loop (device_ics=True, the default; the Gaussian field and
Zel'dovich step then run on the GPU at admission, milliseconds) or the whole initial
conditions (device_ics=False).  Once they are ready and its footprint fits under the
memory cap, it joins the resident batch (continuous batching: requests that arrive while
others run are admitted as slots and memory free up).  The batch advances all resident
simulations together, a few steps per tick; the host enqueues at most `ahead` ticks beyond
what the device has finished, so that admissions wait little.  A finished simulation leaves
the batch at once (no copy of the others' state) and its memory admits the next request.
Latency = completion time - arrival time (initial conditions, queueing and stepping), with
completion observed when the simulation's final state is complete on the device.
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


def _draw(req: Request, pairs_only: bool):
    """Pool worker: the uniform pairs for device initial conditions, else the host ones."""
    if pairs_only:
        from .ics import uniform_pairs
        return req.rid, uniform_pairs(req.n_parts, req.seed)
    from .ics import initial_conditions
    return req.rid, initial_conditions(req.config())


def uses_device_ics(n_parts: int, device_ics: bool) -> bool:
    """Device initial conditions need an FFT size the engine supports; other sizes use the host."""
    from . import _lib
    return device_ics and bool(_lib.load().pm_supported_n(n_parts))


@dataclasses.dataclass
class Result:
    rid: int
    arrival: float
    admitted: float
    completed: float
    particle_updates: int
    pk: tuple | None = None  # (k, P(k), modes) of the final density (pk=True)

    @property
    def latency(self) -> float:
        return self.completed - self.arrival


class Server:
    """Runs a request stream against one GPU in real time."""

    def __init__(self, mem_cap_bytes: int, ic_workers: int = 8, steps_per_tick: int = 4, device: int = 0,
                 keep_results: bool = False, device_ics: bool = True, pk: bool = False, ahead: int = 2):
        import torch
        from .batch import Batch
        self.batch = Batch(device=device, mem_cap_bytes=mem_cap_bytes)
        self.device = device
        self.device_ics = device_ics
        self._ics = {}  # N_PARTS -> DeviceICs
        self._ic_stream = torch.cuda.Stream(device=device) if device_ics else None
        self.pk = pk
        self._ctx = {}  # N_CELLS -> PMContext (density + power spectrum of finished runs)
        self.cap = mem_cap_bytes
        self.steps_per_tick = steps_per_tick
        self.pool = cf.ProcessPoolExecutor(max_workers=ic_workers, mp_context=mp.get_context("spawn"))
        self.keep_results = keep_results
        self.outputs = {}
        self.ahead = max(1, ahead)

    def host_seconds(self) -> dict:
        """Host time the batch engine spent in admissions, planning, graph capture, retirements."""
        return self.batch.host_seconds()

    def close(self):
        self.pool.shutdown(wait=False, cancel_futures=True)
        for g in list(self._ics.values()) + list(self._ctx.values()):
            g.close()
        self._ics.clear()
        self._ctx.clear()
        self.batch.close()

    def _initial_state(self, r: Request, drawn):
        """Positions/velocities to admit: host arrays, or generated on the GPU from the pairs."""
        if not uses_device_ics(r.n_parts, self.device_ics):
            return drawn
        from .device_ics import DeviceICs
        g = self._ics.get(r.n_parts)
        if g is None:
            g = self._ics[r.n_parts] = DeviceICs(r.n_parts, self.device)
        return g.generate(r.config(), uv=drawn, stream=self._ic_stream)

    def _power_spectrum(self, r: Request, sid: int):
        """P(k) of a finished simulation's final density, on the GPU (pm_power_spectrum)."""
        from .context import PMContext
        cfg = r.config()
        ctx = self._ctx.get(cfg.n_cells)
        if ctx is None:
            ctx = self._ctx[cfg.n_cells] = PMContext(cfg, self.device)
        pos = self.batch.get(sid, device=True)[0]
        return ctx.power_spectrum(ctx.density(pos, cfg.mass), box_size=r.box)

    def run(self, stream: list[Request], time_limit: float | None = None) -> list[Result]:
        from .batch import Batch
        ticks = []  # events of the ticks enqueued and not yet known to be finished
        mark = getattr(self.batch, "mark", None)
        ahead = getattr(self, "ahead", 2)
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
                futures[self.pool.submit(_draw, r, uses_device_ics(r.n_parts, self.device_ics))] = r
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
                if self.cap and fp > self.cap:
                    raise RuntimeError(f"request {r.rid} alone exceeds the memory cap")
                if not self.batch.admits(r.config()):
                    break  # wait for memory to free up
                state = self._initial_state(r, ready[r.rid])
                try:
                    sid = self.batch.add(r.config(), *state)
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
                while len(ticks) >= ahead:  # bound the work enqueued beyond the device
                    ticks.pop(0).synchronize()
                self.batch.step(self.steps_per_tick)
                if mark is not None:
                    ticks.append(mark())
                for sid in list(active):
                    if not self.batch.active(sid):
                        r, ta = active.pop(sid)
                        if self.keep_results:
                            self.outputs[r.rid] = self.batch.get(sid)[:2]
                        pk = self._power_spectrum(r, sid) if self.pk else None
                        self.batch.remove(sid)
                        results.append(Result(r.rid, r.arrival, ta, now(), r.particle_updates, pk))
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
