"""The N > 1 paths on CPU: two gloo ranks (127.0.0.1)."""
import os
import socket

import pytest

from conftest import REPO


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out):
    import sys
    import torch.distributed as dist
    sys.path.insert(0, REPO)
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    from pyqg_gb300.ensemble import shard_members
    # rank 1 is slower: the job time is the max, the value sums both ranks
    local = [2.0, 3.0][rank]
    value, total = bench.replica_value(local, 1000, 3600.0, world)
    mine = shard_members(1024, rank, world)
    out.put((rank, value, total, mine[0], len(mine)))
    dist.barrier()
    dist.destroy_process_group()


def test_replicas_take_the_slowest_rank_and_sum_the_work():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    import sys
    sys.path.insert(0, REPO)
    import bench
    expect = 2 * bench.sim_yr_per_hr(1000, 3600.0, 3.0)
    for rank, value, total, first, count in res:
        assert total == 3.0
        assert abs(value - expect) < 1e-9 * expect
    assert res[0][3] == 0 and res[1][3] == res[0][4] and res[0][4] + res[1][4] == 1024


def test_shard_members_cover_without_overlap():
    from pyqg_gb300.ensemble import shard_members
    for n in (1, 7, 1024):
        for world in (1, 2, 3, 8):
            got = [i for r in range(world) for i in shard_members(n, r, world)]
            assert got == list(range(n))
    with pytest.raises(ValueError):
        shard_members(4, 2, 2)
