"""Multi-rank path of the batched sweep on CPU: two gloo ranks each run their
shard of the instances (the oracle's Newton steps stand in for a GPU per
rank) and rank 0 gathers the results, which must match a one-process run
instance for instance."""
import os
import socket

import numpy as np
import pytest

from tissuefolding_paperversion_gb300 import mesh, shard


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _instances():
    return [mesh.config_tiny(seed=400 + i, n=3 + (i % 3), n_layers=1 + (i % 2)) for i in range(7)]


def _run(t, steps=2):
    from oracle.oracle import Port

    p = Port(t)
    its = [p.step(t.dt, t.rates)["iters"] for _ in range(steps)]
    return {"pos": p.positions(), "iters": its}


def _rank_main(rank, world, port, out_path):
    import torch.distributed as dist

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        ts = _instances()
        mine = shard.shard_instances([t.n_elems for t in ts], world)[rank]
        res = {i: _run(ts[i]) for i in mine}
        merged = shard.gather_results(dist, rank, world, res)
        slowest = shard.max_over_ranks(dist, float(len(mine)))
        if rank == 0:
            np.savez(out_path, keys=np.array(sorted(merged)), slowest=slowest,
                     **{f"pos{k}": merged[k]["pos"] for k in merged},
                     **{f"it{k}": np.array(merged[k]["iters"]) for k in merged})
    finally:
        dist.destroy_process_group()


def test_shard_assignment_is_balanced_and_complete():
    sizes = [50, 10, 40, 30, 30, 5, 5, 20]
    parts = shard.shard_instances(sizes, 3)
    assert sorted(i for p in parts for i in p) == list(range(len(sizes)))
    loads = [sum(sizes[i] for i in p) for p in parts]
    assert max(loads) - min(loads) <= max(sizes)
    assert parts == shard.shard_instances(sizes, 3)          # deterministic
    assert shard.shard_instances(sizes, 1) == [list(range(len(sizes)))]
    with pytest.raises(ValueError):
        shard.shard_instances(sizes, 0)


def test_two_gloo_ranks_reproduce_one_process(tmp_path):
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp

    from oracle.oracle import build_port

    build_port()
    out = str(tmp_path / "gathered.npz")
    mp.start_processes(_rank_main, args=(2, _free_port(), out), nprocs=2, join=True, start_method="spawn")
    f = np.load(out)
    ts = _instances()
    assert list(f["keys"]) == list(range(len(ts)))
    parts = shard.shard_instances([t.n_elems for t in ts], 2)
    assert float(f["slowest"]) == max(len(p) for p in parts)
    for i, t in enumerate(ts):
        ref = _run(t)
        np.testing.assert_array_equal(f[f"pos{i}"], ref["pos"])
        assert list(f[f"it{i}"]) == ref["iters"]
