"""The replicas-only multi-process path on CPU with gloo, world size 2: each
rank times its own replica, the reported time is the slowest rank's, the
work is the sum over ranks."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.multiprocessing as mp  # noqa: E402


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, out):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    from sucrose_gb300 import ranks
    r, w, lr = ranks.rank_info()
    t = ranks.max_over_ranks(1.0 + r)        # rank 1 is slower
    units = ranks.sum_over_ranks(100 * (r + 1))
    seed = ranks.replica_seed(1003, r)
    dist.barrier()
    out[rank] = (t, units, seed, w)
    dist.destroy_process_group()


def test_gloo_two_ranks():
    ctx = mp.get_context("spawn")
    mgr = ctx.Manager()
    out = mgr.dict()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, out)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    assert out[0][0] == out[1][0] == 2.0
    assert out[0][1] == out[1][1] == 300.0
    assert out[0][2] != out[1][2]
    assert out[0][3] == 2
