"""The N>1 path of bench.py on CPU: two gloo ranks shard one update, each
extracts its chunks (here with the CPU oracle standing in for the device), no
data-path exchange, and the job time is the max over ranks."""
import os
import socket

import numpy as np
import torch
import torch.distributed as dist
import torch.multiprocessing as mp


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _rank_main(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    from binarymeshfitting_gb300 import workloads
    from oracle import cpu
    _, rows = workloads.lod_update(n=24, seed=3)
    mine = workloads.shard(rows, rank, world)
    small = rows[mine].copy()
    small[:, 4] = np.minimum(small[:, 4], 17)  # keep the CPU work tiny
    total, counts = cpu.extract_batch(small[:, :5].astype(np.float32), 2, list(workloads.TERRAIN_PARAMS))
    t = torch.tensor([float(rank + 1)])
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    n = torch.tensor([float(len(mine))])
    dist.all_reduce(n)
    q.put((rank, mine.tolist(), total, float(t), float(n)))
    dist.destroy_process_group()


def test_two_rank_shard_and_max_time():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(60)
        assert p.exitcode == 0
    covered = sorted(res[0][1] + res[1][1])
    assert covered == list(range(24))
    assert res[0][3] == res[1][3] == 2.0  # max over ranks
    assert res[0][4] == 24.0
