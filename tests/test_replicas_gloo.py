"""Multi-process layout on CPU (gloo, world size 2): rows of the pair triangle
sharded across ranks, each rank computing its rows with the oracle, edge lists
gathered; the union equals the single-process result. Also the part sharding
and the max-over-ranks timing reduction bench.py uses."""
import os
import socket

import numpy as np
import pytest


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, out):
    import torch.distributed as dist

    import oracle
    from visacd_gb300 import meshgen as mg, replicas

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    v, t = mg.displaced_blob(2, seed=4)
    cv, ct = mg.offset_cage(v, t, 0.03)
    r0, r1 = replicas.shard_rows(len(v), rank, world)
    _, e, st = oracle.visibility(v, t, cv, ct, use_bvh=True, rows=(r0, r1))
    allv = replicas.gather_edges(e)
    t_max = replicas.max_over_ranks(float(rank + 1))
    dist.barrier()
    if rank == 0:
        np.save(out, allv)
        with open(out + ".txt", "w") as f:
            f.write(f"{t_max}")
    dist.destroy_process_group()


def test_sharded_visibility_two_ranks(tmp_path):
    import torch.multiprocessing as mp

    import oracle
    from visacd_gb300 import meshgen as mg

    out = str(tmp_path / "edges.npy")
    mp.start_processes(_worker, args=(2, _free_port(), out), nprocs=2, join=True, start_method="spawn")
    got = np.load(out)
    v, t = mg.displaced_blob(2, seed=4)
    cv, ct = mg.offset_cage(v, t, 0.03)
    _, ref, _ = oracle.visibility(v, t, cv, ct, use_bvh=True)
    np.testing.assert_array_equal(got, ref)
    assert float(open(out + ".txt").read()) == 2.0


def test_shard_rows_balances_pairs():
    from visacd_gb300 import replicas

    n = 10242
    total = n * (n - 1) // 2
    for world in (2, 3, 8):
        spans = [replicas.shard_rows(n, r, world) for r in range(world)]
        assert spans[0][0] == 0 and spans[-1][1] == n
        assert all(spans[i][1] == spans[i + 1][0] for i in range(world - 1))
        w = replicas.row_weights(n)
        loads = [int(w[a:b].sum()) for a, b in spans]
        assert sum(loads) == total
        assert max(loads) - min(loads) <= 2 * n


def test_shard_parts_covers_all():
    from visacd_gb300 import replicas

    costs = np.random.default_rng(0).integers(1, 1000, size=37)
    got = sorted(sum((replicas.shard_parts(costs, r, 4) for r in range(4)), []))
    assert got == list(range(37))
