"""bench.py's multi-rank path ("replicas only": each rank runs its own simulation) on CPU
ranks over gloo: the job time is the maximum over ranks, the throughput sums the replicas,
and the reference arm prints from rank 0 only."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as tmp  # noqa: E402


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, ws, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=ws)
    import bench
    t = bench.max_over_ranks(10.0 + 5.0 * rank, dist, "cpu")
    out[rank] = (t, bench.job_throughput(1000, 4, ws, t))
    dist.barrier()
    dist.destroy_process_group()


def test_max_over_ranks_and_job_throughput_with_two_gloo_ranks():
    ws, port = 2, _free_port()
    with tmp.Manager() as m:
        out = m.dict()
        tmp.spawn(_rank, args=(ws, port, out), nprocs=ws, join=True)
        res = dict(out)
    assert res[0] == res[1] == (15.0, 1000 * 4 * 2 / 15.0)


def test_single_rank_needs_no_process_group():
    import bench
    assert bench.max_over_ranks(3.5) == 3.5
    assert bench.job_throughput(10, 2, 1, 4.0) == 5.0


def test_reference_arm_prints_from_rank_zero_only(capsys):
    import argparse
    import bench
    args = argparse.Namespace(steps=1, cpu_steps=1, warmup=0, n_parts=8, n_cells=16, box=100.0)
    bench.run_reference(args, 2, 1)
    assert capsys.readouterr().out == ""


def test_reference_arm_line_contract(capsys):
    """Rank 0 of the reference arm prints one JSON line carrying the contract keys; it times
    the steps and warm-up asked for, its config has the GPU arm's keys, its e2e moves no
    host<->device bytes and its value is the CPU port's."""
    import argparse
    import json
    import bench
    args = argparse.Namespace(steps=2, cpu_steps=1, warmup=1, n_parts=8, n_cells=16, box=100.0)
    bench.run_reference(args, 1, 0)
    lines = [ln for ln in capsys.readouterr().out.splitlines() if ln.strip()]
    assert len(lines) == 1
    d = json.loads(lines[0])
    for key in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
                "scaling", "vs_baseline", "dtype", "data", "config", "cpu_baseline", "e2e"):
        assert key in d, key
    assert d["impl"] == "reference" and d["steps"] == 2 and d["warmup"] == 1 and d["value"] > 0
    cfg = bench.workload_config(3, 8, 16, 100.0)
    assert set(d["config"]) == set(bench.bench_config(cfg, 1, 0.0))
    assert d["metric"] == bench.METRIC and d["unit"] == bench.UNIT and d["higher_is_better"] is True
    assert d["e2e"] == {"value": d["value"], "unit": d["unit"], "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}
    assert (d["config"]["n_parts"], d["config"]["n_cells"], d["config"]["box_size"]) == (8, 16, 100.0)
    cb = d["cpu_baseline"]
    assert cb["value"] == d["value"] and cb["kind"] == "port" and cb["cores"] >= 1
