"""Multi-rank logic of bench.py on CPU (gloo, world size 2): replicas are
reduced with the max of the ranks' times and the sum of their work, and the
reference arm runs on rank 0 only."""
import os
import socket
import sys
import types

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out):
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    import bench
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    mx, sm = bench.reduce_over_ranks(dist, "cpu", [1.5 + rank, 10.0 * rank], [rank + 1, 2, 7])
    out[rank] = (mx, sm)
    dist.barrier()
    dist.destroy_process_group()


def test_reduce_over_ranks_gloo():
    torch = pytest.importorskip("torch")
    mp = torch.multiprocessing.get_context("spawn")
    port = _free_port()
    with mp.Manager() as m:
        out = m.dict()
        procs = [mp.Process(target=_worker, args=(r, 2, port, out)) for r in range(2)]
        for p in procs:
            p.start()
        for p in procs:
            p.join(120)
            assert p.exitcode == 0
        for r in range(2):
            mx, sm = out[r]
            assert mx == [2.5, 10.0]
            assert sm == [3.0, 4.0, 14.0]


def test_reduce_single_rank_is_identity():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.reduce_over_ranks(None, "cpu", [1.0, 2.0], [3, 4]) == ([1.0, 2.0], [3, 4])


def test_reference_arm_runs_on_rank0_only(capsys):
    sys.path.insert(0, ROOT)
    import bench
    args = types.SimpleNamespace(steps=1, warmup=0, gpus=2)
    assert bench.run_reference(args, rank=1, world=2) is None
    assert capsys.readouterr().out == ""
