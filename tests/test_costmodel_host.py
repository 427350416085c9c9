"""Host parts of the learned cost model: candidate trees, tree graphs and batches (no
GPU needed)."""

from __future__ import annotations

import numpy as np
import torch

from tensorsat_gb300 import costmodel
from tensorsat_gb300.contractions.gpu import PRIMES_31, GpuContraction, plan_tree
from tensorsat_gb300.lang.cuda_rel import CudaRel
from tensorsat_gb300.lib.sat import CNFInstance


def test_candidates_graphs_and_batches():
    cnf = CNFInstance.random(3, 24, 100, rng=3)
    w = cnf.clause_diagram().wiring
    cands = costmodel.candidate_trees(w, 4)
    assert 2 <= len(cands) <= 4
    assert len({tuple(t.steps) for t, _ in cands}) == len(cands)
    # the first candidate is the planner's usual choice
    tree, sl = plan_tree(w, target_bits=26, trials=8, seed=0)
    assert tuple(cands[0][0].steps) == tuple(tree.steps) and cands[0][1] == sl
    graphs = []
    for t, s in cands:
        c = GpuContraction(CudaRel, w, tree=t, sliced=s)
        g = costmodel.tree_graph(c, 1, PRIMES_31[:3])
        L = t.num_leaves
        assert g["x"].shape == (L + len(t.steps), costmodel.FEATURES)
        assert all(g["children"][L + i] == t.steps[i] for i in range(len(t.steps)))
        assert np.all(g["x"][:L, 0] == 1) and np.all(g["x"][L:, 1] == 1)
        graphs.append(g)
    b = costmodel.make_batch(graphs, torch.device("cpu"))
    n = sum(g["x"].shape[0] for g in graphs)
    assert b.nodes == n and b.x.shape[0] % 128 == 0 and b.graphs == len(graphs)
    cstart, child, parent = b.cstart.numpy(), b.child.numpy(), b.parent.numpy()
    # every child edge appears once and points back to its parent
    for v in range(n):
        for e in range(cstart[v], cstart[v + 1]):
            assert parent[child[e]] == v
    assert int((parent >= 0).sum()) == cstart[-1] == sum(2 * (len(g["x"]) - 1) // 2 for g in graphs)


def test_candidate_settings_split_and_merge():
    """64 settings (the fixed list first), split over workers and merged back without
    repeats: the merged list is the single-worker list, planner's choice first."""
    st = costmodel.candidate_settings(64)
    assert len(st) == 64 and st[:len(costmodel.CANDIDATE_SETTINGS)] == costmodel.CANDIDATE_SETTINGS
    assert len({s[3] for s in st}) == 64
    w = CNFInstance.random(3, 20, 85, rng=5).clause_diagram().wiring
    whole = costmodel.candidate_trees(w, 12)
    parts = [costmodel.candidate_trees(w, 12, settings=costmodel.candidate_settings(12)[p::3])
             for p in range(3)]
    merged = costmodel.distinct([x[k] for k in range(4) for x in parts if k < len(x)])
    key = lambda ts: [(tuple(t.steps), s) for t, s in ts]
    assert key(merged)[0] == key(whole)[0]
    assert sorted(key(merged)) == sorted(key(whole))


def test_cnf_candidates_in_spawned_workers():
    """cnf_candidates splits each instance's planner settings over spawned workers and
    merges them back: the same candidate set as one process, the planner's usual choice
    first."""
    import multiprocessing as mp

    cnf = CNFInstance.random(3, 18, 76, rng=4)
    whole = costmodel.candidate_trees(cnf.clause_diagram().wiring, 6)
    with mp.get_context("spawn").Pool(2) as pool:
        got = costmodel.cnf_candidates(pool, [cnf], 6, parts=3)[0]
    key = lambda ts: [(tuple(t.steps), tuple(s)) for t, s in ts]
    assert key(got)[0] == key(whole)[0]
    assert sorted(key(got)) == sorted(key(whole))
