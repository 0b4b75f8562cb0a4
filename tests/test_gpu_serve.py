"""Serving loop: requests admitted while others run (continuous batching under a memory
cap) must each give the same result as when run alone (bit-identical: a simulation's
arithmetic does not depend on its neighbours in the batch)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("device_ics", [False, True])
def test_served_results_equal_alone(cuda, device_ics):
    from pmgpu.batch import Batch
    from pmgpu.serve import Request, Server, summarize, uses_device_ics
    from pmgpu import ics
    from pmgpu.device_ics import DeviceICs
    stream = [Request(0, 11, 16, 100.0, 30, 0.0), Request(1, 12, 24, 200.0, 20, 0.0),
              Request(2, 13, 32, 150.0, 40, 0.05), Request(3, 14, 16, 80.0, 12, 0.1),
              Request(4, 15, 12, 120.0, 25, 0.15), Request(5, 16, 32, 300.0, 15, 0.2)]
    # a cap that holds about two of the larger requests: later ones wait for memory
    cap = 2 * Batch.footprint(stream[2].config()) + Batch.footprint(stream[0].config())
    srv = Server(mem_cap_bytes=cap, ic_workers=2, steps_per_tick=3, keep_results=True, device_ics=device_ics,
                 pk=device_ics)
    res = srv.run(stream)
    srv.close()
    assert sorted(r.rid for r in res) == list(range(len(stream)))
    s = summarize(res, max(r.completed for r in res))
    assert s["p99_latency_s"] >= s["p50_latency_s"] > 0
    for r in stream:
        b = Batch()
        if uses_device_ics(r.n_parts, device_ics):  # N_PARTS = 12 has no device transform: host
            state = DeviceICs(r.n_parts).generate(r.config())
        else:
            state = ics.initial_conditions(r.config())
        sid = b.add(r.config(), *state)
        b.step(1000)
        p, v, _, _ = b.get(sid)
        b.close()
        pm, vm = srv.outputs[r.rid]
        assert np.array_equal(p, pm) and np.array_equal(v, vm)
    if device_ics:  # every result carries the power spectrum of its final density
        from oracle import pm_oracle as O
        for out in res:
            r = stream[out.rid]
            k, pk, modes = out.pk
            pos = srv.outputs[out.rid][0]
            rho = O.density(pos, r.config().mass, r.config().n_cells)
            k2, pk2, m2 = O.power_spectrum(rho, r.box)
            assert np.array_equal(modes, m2) and np.abs(pk / pk2 - 1).max() < 1e-4
