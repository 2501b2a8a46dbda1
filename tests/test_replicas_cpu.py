"""The replicas path of the bench on the CPU (gloo backend, world size 2):
every rank takes its own shard of the workload, and the job's figure is the
slowest rank's time with the work of all ranks -- the cross-rank arithmetic
`bench.py` does under torchrun on GPUs, run here without a GPU."""
import os
import socket
import sys

import numpy as np

import oracle_lib as ol

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket(socket.AF_INET, socket.SOCK_STREAM) as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, q):
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    import bench
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    try:
        seconds, units = bench.reduce_over_ranks(1.5 + rank, 1000 * (rank + 1), "cpu")
        dist.barrier()
        q.put((rank, seconds, units))
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_report_the_slowest_time_and_all_work():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    try:
        res = sorted(q.get(timeout=180) for _ in range(2))
    finally:
        for p in procs:
            p.join(timeout=60)
            if p.is_alive():
                p.kill()
    assert [r[1] for r in res] == [2.5, 2.5]        # max over ranks of 1.5 s and 2.5 s
    assert [r[2] for r in res] == [3000.0, 3000.0]  # 1000 + 2000 units
    assert all(p.exitcode == 0 for p in procs)


def test_rank_shards_are_deterministic_and_distinct():
    sys.path.insert(0, ROOT)
    import bench
    import zeta_gb300 as z
    w = z.WORKLOADS["perft_batch"]

    def shard(rank):
        return ol.make_positions(bench.shard_seed(w["seed"], rank), 32, min_plies=w["min_plies"],
                                 max_plies=w["max_plies"], min_pieces=w["min_pieces"], min_depth=w["min_depth"],
                                 max_depth=w["max_depth"])

    a, a2, b = shard(0), shard(0), shard(1)
    assert np.array_equal(a[0], a2[0]) and np.array_equal(a[2], a2[2])
    assert not np.array_equal(a[0], b[0])
    assert bench.shard_seed(w["seed"], 0) == w["seed"]
