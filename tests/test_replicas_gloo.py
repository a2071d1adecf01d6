"""The replica (N > 1) reduction on CPU: two gloo ranks, max over ranks."""
import os
import socket

import torch.multiprocessing as mp


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank(rank, world, port, q):
    import sys
    sys.path.insert(0, os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))),
                                    "open-3d-wallturbulence_gb300"))
    import torch.distributed as dist
    from owt.replicas import aggregate, barrier
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    barrier(device_sync=False)
    ms, rate = aggregate(100.0 * (rank + 1), steps_per_rank=10)
    q.put((rank, ms, rate))
    dist.destroy_process_group()


def test_replica_timing_is_max_over_ranks():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(60)
        assert p.exitcode == 0
    res = sorted(q.get() for _ in range(2))
    for rank, ms, rate in res:
        assert ms == 200.0                      # the slower rank
        assert abs(rate - 2 * 10 * 1e3 / 200.0) < 1e-9   # whole-job steps/s
