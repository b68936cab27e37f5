"""The replica logic bench.py uses for --gpus N (barrier, max over ranks),
run as two gloo ranks on the CPU."""
import os
import socket

import pytest
import torch
import torch.multiprocessing as mp


def _free_port():
    s = socket.socket()
    s.bind(('127.0.0.1', 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank(rank, world, port, q):
    os.environ.update(MASTER_ADDR='127.0.0.1', MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    import sys
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    import bench
    import torch.distributed as tdist
    tdist.init_process_group('gloo', rank=rank, world_size=world)
    tdist.barrier()
    # each rank "times" a different amount; everyone must see the maximum
    m = bench.max_over_ranks(torch, world, 10.0 + rank, device='cpu')
    q.put((rank, m))
    tdist.destroy_process_group()


def test_two_rank_max_over_ranks():
    world, port = 2, _free_port()
    ctx = mp.get_context('spawn')
    q = ctx.Queue()
    procs = [ctx.Process(target=_rank, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    out = dict(q.get(timeout=120) for _ in range(world))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert out == {0: 11.0, 1: 11.0}
