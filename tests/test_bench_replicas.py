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
