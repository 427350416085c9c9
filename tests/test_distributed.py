"""Multi-rank slice sharding on CPU ranks (gloo, world size 2): each rank contracts its
own contiguous slice range (with the CPU oracle standing in for the device) and the
ranks combine residues and SAT bits with one all-reduce each."""

from __future__ import annotations

import os

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


def _worker(rank: int, world: int, store_file: str, q) -> None:
    # a file rendezvous: no TCP port to race for with other processes on the host
    dist.init_process_group("gloo", init_method=f"file://{store_file}", rank=rank,
                            world_size=world)
    try:
        import numpy as np

        from oracle import finrel_oracle as orc
        from tensorsat_gb300 import _native
        from tensorsat_gb300.contractions.gpu import GpuContraction
        from tensorsat_gb300.lang.cuda_rel import CudaRel
        from tensorsat_gb300.lib.sat import CNFInstance

        cnf = CNFInstance.random(3, 16, 66, rng=9)
        d = cnf.clause_diagram()
        c = GpuContraction(CudaRel, d.wiring, target_bits=5, trials=1)
        steps, sliced = list(c.tree.steps), list(c.sliced_wires)
        shares = []

        def host_root(self, diagram, ring, primes, slice_range, group, cache_leaves,
                      workspace=None):
            # the device run of one rank's share, replaced by the oracle's contraction of
            # the same slices along the same tree
            shares.append(tuple(slice_range))
            total = 0
            for sid in range(*slice_range):
                fixed = {w: (sid >> j) & 1 for j, w in enumerate(sliced)}
                total += orc.cnf_count_by_tree(16, cnf.clauses, steps, "count", fixed=fixed)
            if ring == _native.TSG_RING_MODP:
                return np.array([[total % p] for p in primes], dtype=np.uint32)
            if ring == _native.TSG_RING_U64:
                return np.array([total % (1 << 64)], dtype=np.uint64)
            return np.array([1 if total else 0], dtype=np.uint8)

        GpuContraction._ring_root = host_root
        pg = dist.group.WORLD
        n_modp = c.count(d, ring="modp", num_primes=3, group=2, process_group=pg)
        n_u64 = c.count(d, ring="u64", group=2, process_group=pg)
        bit = bool(c.contract(d, group=2, process_group=pg))
        half = c.count(d, ring="modp", num_primes=2, group=2,
                       slice_range=(0, c.num_slices // 2), process_group=pg)
        q.put((rank, n_modp, n_u64, bit, half, shares, c.num_slices,
               orc.brute_force_count(16, cnf.clauses)))
    finally:
        dist.destroy_process_group()


def test_two_rank_sharded_count_gloo(tmp_path):
    """GpuContraction.count / .contract with a process group on two gloo CPU ranks: each
    rank runs only its own contiguous, group-aligned share of the slices, and one
    all-reduce per ring combines the shares into the exact count (mod primes with CRT,
    mod 2^64) and the SAT bit on every rank. The device run of a share is replaced by the
    oracle's contraction of the same slices (the GPU tests cover the device run)."""
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    store = str(tmp_path / "rendezvous")
    procs = [ctx.Process(target=_worker, args=(r, 2, store, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=240)
    for p in procs:
        assert p.exitcode == 0
    got = sorted(q.get(timeout=10) for _ in range(2))
    ns, exp = got[0][6], got[0][7]
    assert exp > 0
    for rank, n_modp, n_u64, bit, half, shares, _, _ in got:
        assert n_modp == n_u64 == exp
        assert bit is True
        assert 0 <= half <= exp
    assert got[0][4] == got[1][4]
    # the two ranks' shares of each call tile the slices with no overlap
    for call in range(4):
        a, b = got[0][5][call], got[1][5][call]
        assert a[0] == 0 and a[1] == b[0] and a[0] % 2 == 0 and b[0] % 2 == 0
    assert got[1][5][0][1] == ns and got[1][5][3][1] == ns // 2
