"""Multi-rank slice sharding on CPU ranks (gloo, world size 2): each rank contracts its
own contiguous slice range (with the CPU oracle standing in for the device) and the
ranks combine residues and SAT bits with one all-reduce each."""

from __future__ import annotations

import os
import socket

import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

from tensorsat_gb300.sharding import allreduce_or, allreduce_residues, combine_counts, slice_ranges


def test_slice_ranges_partition_and_align():
    for ns, world, group in [(1, 2, 1), (16, 2, 4), (1024, 3, 8), (7, 4, 2), (64, 8, 16)]:
        rs = slice_ranges(ns, world, group)
        assert len(rs) == world
        covered = [s for b, e in rs for s in range(b, e)]
        assert covered == list(range(ns))
        for b, e in rs:
            assert b % group == 0 or b == ns
    with pytest.raises(ValueError):
        slice_ranges(8, 0)
    with pytest.raises(ValueError):
        slice_ranges(8, 2, 3)
    assert combine_counts([5, 7]) == 12
    assert combine_counts([5, 7], [7]) == 5


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank: int, world: int, port: int, q) -> None:
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        from oracle import finrel_oracle as orc
        from tensorsat_gb300 import planner
        from tensorsat_gb300.contractions.gpu import PRIMES_31
        from tensorsat_gb300.lib.sat import CNFInstance

        cnf = CNFInstance.random(3, 16, 66, rng=9)
        wires = [tuple(dict.fromkeys(abs(l) - 1 for l in c)) for c in cnf.clauses]
        net = planner.Network(wires, {w: 2 for w in range(16)}, ())
        tree, sliced = planner.optimize(net, target_bits=5, trials=1, seed=0)
        sliced = tuple(sorted(sliced))
        ns = 1 << len(sliced)
        b, e = slice_ranges(ns, world, 2)[rank]
        part = 0
        for sid in range(b, e):
            fixed = {w: (sid >> j) & 1 for j, w in enumerate(sliced)}
            part += orc.cnf_count_by_tree(16, cnf.clauses, tree.steps, fixed=fixed)
        primes = PRIMES_31[:3]
        res = torch.tensor([[part % p] for p in primes], dtype=torch.int64)
        total = allreduce_residues(res, primes)
        bit = allreduce_or(torch.tensor([1 if part else 0]))
        if rank == 0:
            q.put((int(total[0, 0]), int(bit[0]), orc.brute_force_count(16, cnf.clauses)))
    finally:
        dist.destroy_process_group()


def test_two_rank_sharded_count_gloo():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=240)
    for p in procs:
        assert p.exitcode == 0
    total, bit, exp = q.get(timeout=10)
    assert total == exp % 2147483647
    assert bit == int(exp > 0)
