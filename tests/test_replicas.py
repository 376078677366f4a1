"""The multi-GPU path is replicas only: `bench.py --gpus N` runs one process
per GPU on its own copy of the workload, with no exchange on the data path;
the whole job takes as long as its slowest rank and its work is the rays of
all ranks. These tests run that aggregation on two CPU processes over gloo."""
import os
import socket
import sys

import multiprocessing as mp

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, port, seconds, units, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE="2",
                      LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    import torch.distributed as dist
    dist.init_process_group("gloo", rank=rank, world_size=2)
    import bench
    ws, r, local = bench.dist_env()
    value, t_max = bench.whole_job(seconds[rank], units, "cpu")
    dist.barrier()
    out.put((rank, ws, r, local, value, t_max))
    dist.destroy_process_group()


def test_whole_job_over_two_gloo_ranks():
    ctx = mp.get_context("spawn")
    out = ctx.Queue()
    port = _free_port()
    seconds = (0.5, 2.0)
    units = 4_194_304 * 20
    procs = [ctx.Process(target=_rank_main, args=(r, port, seconds, units, out)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=180)
    for p in procs:
        if p.is_alive():
            p.kill()
    assert all(p.exitcode == 0 for p in procs)
    res = sorted(out.get(timeout=10) for _ in range(2))
    for rank, (r, ws, r_env, local, value, t_max) in enumerate(res):
        assert (r, ws, r_env, local) == (rank, 2, rank, rank)
        assert t_max == 2.0  # the slowest rank's time on every rank
        assert value == pytest.approx(2 * units / 2.0 / 1e6)


def test_single_process_is_its_own_job():
    sys.path.insert(0, ROOT)
    import bench
    value, t = bench.whole_job(0.25, 1_000_000, "cpu")
    assert (value, t) == (4.0, 0.25)


def test_reference_arm_runs_on_rank_zero_only(monkeypatch, capsys):
    sys.path.insert(0, ROOT)
    import bench
    monkeypatch.setenv("RANK", "1")
    monkeypatch.setenv("WORLD_SIZE", "2")

    class Args:
        steps, warmup, gpus, no_reference_gpu = 1, 1, 2, True

    assert bench.run_reference(Args()) is None
    assert capsys.readouterr().out == ""
