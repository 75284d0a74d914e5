"""Replicas and sharding of independent problems over ranks: the cost-based
schedule, and the control-plane collectives (max of per-rank times, gather of
per-rank results) on two gloo ranks on the CPU."""
import os
import socket

import pytest
import torch.multiprocessing as mp

from carcassonne_gb300.replicas import gather_to_root, max_over_ranks, problem_cost, shard_by_cost


def test_shard_by_cost_is_a_balanced_partition():
    from carcassonne_gb300 import batched
    specs = batched.sample_problems(32, 3)
    costs = [problem_cost(D, chi) for D, chi, _, _ in specs]
    for world in (1, 2, 3, 8):
        shards = shard_by_cost(costs, world)
        assert sorted(i for s in shards for i in s) == list(range(len(costs)))
        loads = [sum(costs[i] for i in s) for s in shards]
        # LPT bound: no rank exceeds the mean by more than the largest job
        assert max(loads) <= sum(costs) / world + max(costs)
    assert shard_by_cost(costs, 2) == shard_by_cost(list(costs), 2)  # deterministic


def test_shard_by_cost_rejects_empty_world():
    with pytest.raises(ValueError):
        shard_by_cost([1, 2], 0)


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank_main(rank, world, port, out_path):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        # rank r "measured" (r + 1) ms and 10 (r + 1) ms
        ms = max_over_ranks([1.0 + rank, 10.0 * (1 + rank)], dist)
        costs = [problem_cost(D, chi) for D, chi in [(6, 96), (2, 16), (5, 40), (4, 64), (3, 88)]]
        mine = shard_by_cost(costs, world)[rank]
        got = gather_to_root({"rank": rank, "problems": mine, "ms": ms}, dist, rank, world)
        if rank == 0:
            import json
            with open(out_path, "w") as f:
                json.dump(got, f)
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks(tmp_path):
    out = tmp_path / "gathered.json"
    mp.spawn(_rank_main, args=(2, _free_port(), str(out)), nprocs=2, join=True)
    import json
    got = json.loads(out.read_text())
    assert [g["rank"] for g in got] == [0, 1]
    assert all(g["ms"] == [2.0, 20.0] for g in got)           # the slowest rank's times everywhere
    assigned = sorted(i for g in got for i in g["problems"])
    assert assigned == list(range(5))                          # every problem on exactly one rank


def test_batched_problem_distribution():
    """The batched workload's problems (host side): D in {2..6}, chi in
    {16, 24, ..., 96} split into ket x bra factors whose product is chi, h in
    [2, 4), distinct seeds, reproducible from the workload seed."""
    from carcassonne_gb300 import batched
    specs = batched.sample_problems(256, 3)
    assert specs == batched.sample_problems(256, 3)
    assert {D for D, _, _, _ in specs} == {2, 3, 4, 5, 6}
    assert {chi for _, chi, _, _ in specs} <= set(range(16, 97, 8))
    assert all(2.0 <= h < 4.0 for _, _, h, _ in specs)
    assert len({s for _, _, _, s in specs}) == len(specs)
    for chi, (ck, cb) in batched.CHI_FACTORS.items():
        assert ck * cb == chi
    shards = shard_by_cost([problem_cost(D, chi) for D, chi, _, _ in specs], 8)
    assert sorted(i for s in shards for i in s) == list(range(256))


def test_problem_cost_ranks_like_costtracker():
    """problem_cost (the sharding key) against the CostTracker count of the
    actual operators (the oracle's, data/cost_tracker.py:17-22) for problems
    of the batched workload's structure: the same order, within 0.1 %."""
    import numpy as np
    from carcassonne_gb300 import batched, workloads
    from oracle import carc_oracle as orc
    from tests.tagrepr import parse_tag
    cases = [(2, 16), (3, 16), (2, 24), (4, 16), (3, 24), (2, 32)]
    exact, est = [], []
    for D, chi in cases:
        ck, cb = batched.CHI_FACTORS[chi]
        c, s, o = workloads.matvec_problem_arrays(D=D, c_ket=ck, c_bra=cb, seed=1,
                                                  op_arrays=workloads.ti_operator_arrays(h=3.0))
        oc = [{parse_tag(repr(t)): a for t, a in lst} for lst in c]
        osd = [{parse_tag(repr(t)): a for t, a in lst} for lst in s]
        oo = {parse_tag(repr(t)): a for t, a in o}
        H, _, _ = orc.expectation_and_normalization_multipliers(oc, osd, oo)
        exact.append(H.cost_of_multiply * 8)
        est.append(problem_cost(D, chi, nvec=8))
    assert list(np.argsort(exact)) == list(np.argsort(est))
    assert all(abs(a - b) <= 1e-3 * a for a, b in zip(exact, est))


def _host_solve(sub):
    """A host stand-in for the GPU batch solve: a deterministic function of
    each problem's spec, and a "time" proportional to the shard's cost."""
    from carcassonne_gb300 import batched
    return dict(energy=[-(D * 10.0 + c + h) for D, c, h, _ in sub], iterations=[D + c for D, c, _, _ in sub],
                seconds=sum(batched.pencil_cost(s) for s in sub) * 1e-12)


def _sharded_rank_main(rank, world, port, out_path):
    import json
    import torch.distributed as dist
    from carcassonne_gb300 import batched
    from carcassonne_gb300.replicas import run_sharded
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        specs = batched.sample_pencils(40, 3)   # problem generation, identical on every rank
        got = run_sharded(specs, batched.pencil_cost, _host_solve, dist, rank, world)
        if rank == 0:
            with open(out_path, "w") as f:
                json.dump(got, f)
        else:
            assert got is None
    finally:
        dist.destroy_process_group()


def test_sharded_batch_on_two_gloo_ranks(tmp_path):
    """The host side of the sharded batched-solve path (bench.py under
    torchrun): problem generation, the cost-based shard, per-rank solves, the
    max-over-ranks time and the gather of every problem's result to rank 0 in
    the original order, equal to one rank solving everything."""
    import json
    from carcassonne_gb300 import batched
    from carcassonne_gb300.replicas import run_sharded
    out = tmp_path / "sharded.json"
    mp.spawn(_sharded_rank_main, args=(2, _free_port(), str(out)), nprocs=2, join=True)
    got = json.loads(out.read_text())
    specs = batched.sample_pencils(40, 3)
    serial = run_sharded(specs, batched.pencil_cost, _host_solve)
    assert got["problems"] == 40 and got["ranks"] == 2
    assert got["energy"] == serial["energy"] and got["iterations"] == serial["iterations"]
    loads = [r["cost"] for r in got["per_rank"]]
    assert sum(r["problems"] for r in got["per_rank"]) == 40
    assert max(loads) <= sum(loads) / 2 + max(batched.pencil_cost(s) for s in specs)
    assert got["seconds"] == max(r["seconds"] for r in got["per_rank"])
    assert got["seconds"] < serial["seconds"]
