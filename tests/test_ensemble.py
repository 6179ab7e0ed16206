"""Independent chains over several ranks (kylin_v_gb300.ensemble): the split
is complete, deterministic and balanced, and results gathered from two gloo
ranks on the CPU come back whole and in chain order.  The per-rank work is a
stand-in function here (the GPU runner is exercised by the batched tests)."""
import json
import os
import socket

import pytest

import kvtest_util as U

U.load_package()
from kylin_v_gb300 import ensemble as E  # noqa: E402


def _fake_run(chains, idx):
    return {i: {"chain": c, "value": 0.5 * i} for c, i in zip(chains, idx)}


def test_shard_complete_deterministic_balanced():
    costs = [E.chain_cost(3 * L, D) for L, D in [(48, 256), (23, 32), (36, 128), (47, 128), (32, 256), (8, 64),
                                                  (20, 32), (39, 128), (27, 32), (17, 32), (21, 256)]]
    for world in (1, 2, 3, 4):
        parts = E.shard(costs, world)
        assert sorted(i for p in parts for i in p) == list(range(len(costs)))
        assert parts == E.shard(costs, world)
        if world > 1:
            loads = [sum(costs[i] for i in p) for p in parts]
            assert max(loads) <= sum(costs) / world + max(costs)
    assert E.shard([1.0, 2.0], 4)[2:] == [[], []]


def test_single_rank_gathers_everything():
    members = [f"c{i}" for i in range(5)]
    out = E.run_ensemble(members, [1.0] * 5, _fake_run)
    assert [o["chain"] for o in out] == members


def _worker(rank, world, port, path, n):
    import torch.distributed as dist

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        members = [f"chain{i}" for i in range(n)]
        costs = [float((7 * i) % 5 + 1) for i in range(n)]
        out = E.run_ensemble(members, costs, _fake_run, rank=rank, world=world)
        if rank == 0:
            with open(path, "w") as f:
                json.dump(out, f)
        else:
            assert out is None
        dist.barrier()
    finally:
        dist.destroy_process_group()


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


@pytest.mark.parametrize("n", [1, 5, 8])
def test_two_gloo_ranks_gather_in_chain_order(tmp_path, n):
    import torch.multiprocessing as mp

    path = str(tmp_path / "out.json")
    mp.spawn(_worker, args=(2, _free_port(), path, n), nprocs=2, join=True)
    with open(path) as f:
        out = json.load(f)
    assert [o["chain"] for o in out] == [f"chain{i}" for i in range(n)]
    assert [o["value"] for o in out] == [0.5 * i for i in range(n)]
