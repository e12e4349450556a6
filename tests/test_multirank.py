"""The N > 1 path of bench.py (replicas, one process per GPU) on CPU with the
gloo backend, world size 2: max-over-ranks timing and the whole-job value.
The GPU path runs the same helpers over NCCL."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank_main(rank, world, port, out_dir):
    import torch.distributed as dist
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", init_method="env://", rank=rank, world_size=world)
    ms_local = 100.0 + 50.0 * rank                  # rank 1 is the slower one
    ms = bench.reduce_max(ms_local, world)
    value = bench.whole_job_value(4.0e11, ms, world)
    with open(os.path.join(out_dir, "r%d" % rank), "w") as f:
        f.write("%r %r" % (ms, value))
    dist.barrier()
    dist.destroy_process_group()


def test_two_rank_max_and_value(tmp_path):
    import torch.multiprocessing as mp
    world = 2
    mp.spawn(_rank_main, args=(world, _free_port(), str(tmp_path)), nprocs=world, join=True)
    got = [open(tmp_path / ("r%d" % r)).read().split() for r in range(world)]
    for ms, value in got:
        assert float(ms) == 150.0
        assert abs(float(value) - 4.0e11 * 2 / 0.150) < 1.0


def test_reference_arm_other_ranks_do_nothing(monkeypatch, capsys):
    import bench
    monkeypatch.setenv("RANK", "1")
    assert bench.run_reference(None, bench.WORKLOADS["plain"], [100]) == 0
    assert capsys.readouterr().out == ""
