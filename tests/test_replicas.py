"""The multi-GPU path of bench.py is replicas (one independent field per GPU,
no data-path collective): the job's time is the slowest rank's and its value
all ranks' voxel-steps over that time. Checked with two gloo ranks on the CPU
(the GPU runs use the same functions over NCCL)."""
import os
import socket

import pytest
import torch.multiprocessing as mp


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    import sys

    import torch.distributed as dist
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    sys.path.insert(0, root)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    r, w, lr = bench.rank_info()
    t = bench.max_over_ranks(1.5 + rank, device="cpu")   # rank 1 is the slow one
    v = bench.job_value(1000.0, w, t)
    out.put((r, w, lr, t, v))
    dist.barrier()
    dist.destroy_process_group()


def test_two_replicas_take_the_slowest_rank():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [r[0] for r in res] == [0, 1] and all(r[1] == 2 for r in res)
    assert all(r[3] == pytest.approx(2.5) for r in res)            # max over ranks
    assert all(r[4] == pytest.approx(2 * 1000.0 / 2.5) for r in res)


def test_single_process_is_identity():
    import sys
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    import bench
    assert bench.max_over_ranks(3.25, device="cpu") == 3.25
    assert bench.job_value(10.0, 1, 2.0) == 5.0
