"""Body shards across ranks (multi-GPU path), exercised with two gloo ranks on the CPU.

Each rank cuts its own shard out of the same serialised scene; together the shards must cover every
body exactly once, keep every collider, reproduce each body's bytes unchanged and be balanced by
estimated cost. Timing is reduced as in bench.py (max over ranks).
"""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402
from scenes import build_scene  # noqa: E402


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank: int, world: int, port: int, scene: bytes, out_dir: str):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        from joltphysics_gb300.shard import body_costs, shard_scene

        sub, mine = shard_scene(scene, rank, world)
        costs = body_costs(scene)
        load = sum(costs[i] for i in mine)
        gathered = [None] * world
        dist.all_gather_object(gathered, (mine, load, len(sub)))
        t = torch.tensor([float(rank + 1)])
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        if rank == 0:
            import pickle

            with open(os.path.join(out_dir, "result.pkl"), "wb") as f:
                pickle.dump({"gathered": gathered, "max": float(t.item()), "sub0": sub}, f)
    finally:
        dist.destroy_process_group()


def test_two_rank_shards_cover_and_balance(jsb, tmp_path):
    import pickle
    import struct

    from jsb_testlib import parse_scene

    scene = build_scene("uneven_batch", n_cloth=40, n_cube=12, steps=2, seed=6)
    mp.start_processes(_rank_main, args=(2, _free_port(), scene, str(tmp_path)), nprocs=2, join=True,
                       start_method="spawn")
    res = pickle.load(open(tmp_path / "result.pkl", "rb"))
    shards = [g[0] for g in res["gathered"]]
    loads = [g[1] for g in res["gathered"]]
    assert sorted(shards[0] + shards[1]) == list(range(52))
    assert not set(shards[0]) & set(shards[1])
    assert max(loads) <= 1.1 * min(loads)
    assert res["max"] == 2.0
    full, _ = parse_scene(scene)
    part, _ = parse_scene(res["sub0"])
    assert len(part.bodies) == len(shards[0]) and len(part.colliders) == len(full.colliders)
    for i, body in zip(shards[0], part.bodies):
        assert body.blob == full.bodies[i].blob and body.position == full.bodies[i].position
    assert struct.unpack_from("<I", res["sub0"], 8)[0] == len(shards[0])


def test_single_rank_takes_everything(jsb):
    from joltphysics_gb300.shard import assign_shards

    assert assign_shards([3.0, 1.0, 2.0], 1) == [[0, 1, 2]]
    assert assign_shards([5.0, 4.0, 3.0, 3.0], 2) == [[0, 3], [1, 2]]
    with pytest.raises(ValueError):
        assign_shards([1.0], 0)
