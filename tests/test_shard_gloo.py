"""The multi-rank path on CPU: two gloo ranks each step their shard of the
worlds (with the oracle standing in for the GPU) and the gathered state equals
a single-process run.  Worlds are independent, so sharding needs no
collective inside a step."""
import os
import socket

import numpy as np
import torch.multiprocessing as mp

from cubez_gb300 import scenes, shard


def test_partition_balanced_and_complete():
    s = scenes.mixed(num_worlds=301, seed=7)
    parts = shard.partition(s.counts, 4)
    allw = sorted(w for p in parts for w in p)
    assert allw == list(range(301))
    loads = [sum(int(s.counts[w]) ** 2 for w in p) for p in parts]
    assert max(loads) - min(loads) <= int(s.counts.max()) ** 2


def _free_port():
    with socket.socket() as sk:
        sk.bind(("127.0.0.1", 0))
        return sk.getsockname()[1]


def _rank(rank, ws, port, out_path):
    import torch.distributed as dist

    from oracle.oracle import OracleBatch
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=ws)
    scene = scenes.mixed(num_worlds=12, seed=8)
    mine = shard.partition(scene.counts, ws)[rank]
    ob = OracleBatch(scene.subset(mine))
    ob.step(30, 1.0 / 60.0)
    b = ob.bodies()
    full = shard.gather_bodies({"position": b["position"], "velocity": b["velocity"]}, mine, scene)
    if rank == 0:
        np.savez(out_path, **full)
    dist.barrier()
    dist.destroy_process_group()


def test_two_gloo_ranks_match_single_process(tmp_path):
    from oracle.oracle import OracleBatch
    out = str(tmp_path / "gathered.npz")
    ctx = mp.get_context("spawn")
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, out)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    got = np.load(out)
    scene = scenes.mixed(num_worlds=12, seed=8)
    ob = OracleBatch(scene)
    ob.step(30, 1.0 / 60.0)
    ref = ob.bodies()
    np.testing.assert_array_equal(got["position"], ref["position"])
    np.testing.assert_array_equal(got["velocity"], ref["velocity"])
