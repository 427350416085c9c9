"""Planner checks on the CPU: trees are well formed, slicing meets its target, and the
integer arrays handed to the native executor compute exact counts (numpy emulation of the
executor's index semantics against brute force)."""

from __future__ import annotations

import random

import numpy as np
import pytest

from oracle import finrel_oracle as orc
from plan_emulator import emulate_all
from tensorsat_gb300 import planner
from tensorsat_gb300.contractions.gpu import GpuContraction, _prepare
from tensorsat_gb300.lang.cuda_rel import CudaRel
from tensorsat_gb300.lib.sat import CNFInstance


def _leaves(diagram, contraction):
    lw = contraction._leaves
    arrays = []
    for slot, syn in zip(lw.slot_of_leaf, lw.synthetic):
        arrays.append(syn if syn is not None else diagram.blocks[slot].numpy())
    return arrays


def _check_tree(tree, net):
    L = tree.num_leaves
    live = set(range(L))
    out = set(net.out_wires)
    for s, (a, b) in enumerate(tree.steps):
        assert a in live and b in live
        live -= {a, b}
        res = tree.node_wires[L + s]
        assert res <= tree.node_wires[a] | tree.node_wires[b]
        live.add(L + s)
    assert live == {tree.root}
    assert tree.node_wires[tree.root] == out


@pytest.mark.parametrize("n,m,seed", [(12, 50, 0), (16, 68, 1), (20, 85, 2)])
def test_trees_well_formed_and_sliced_to_target(n, m, seed):
    cnf = CNFInstance.random(3, n, m, rng=seed)
    for d in ((cnf.inputs(None) >> cnf.diagram()).flatten(), cnf.clause_diagram()):
        net = planner.Network([tuple(ws) for ws in d.wiring.slot_wires_list],
                              {w: 2 for w in range(d.wiring.num_wires)}, ())
        tree, sl = planner.optimize(net, target_bits=6, trials=2, seed=seed)
        _check_tree(tree, net)
        assert tree.cost(sl)[1] <= 6
        replay = list(range(tree.num_leaves))
        for s, (i, j) in enumerate(tree.linear_path()):
            a, b = replay[i], replay[j]
            assert (a, b) == tree.steps[s]
            for x in sorted((i, j), reverse=True):
                replay.pop(x)
            replay.append(tree.num_leaves + s)


@pytest.mark.parametrize("n,m,seed,target", [(10, 42, 0, None), (12, 50, 1, 4), (14, 60, 2, 6),
                                             (12, 40, 3, 3)])
def test_emulated_native_plan_counts(n, m, seed, target):
    cnf = CNFInstance.random(3, n, m, rng=seed)
    exp = orc.brute_force_count(n, cnf.clauses)
    for d in ((cnf.inputs(None) >> cnf.diagram()).flatten(), cnf.clause_diagram()):
        c = GpuContraction(CudaRel, d.wiring, target_bits=target, trials=1, seed=seed)
        arrs = c.sliced_plan.native_arrays()
        leaves = _leaves(d, c)
        total = emulate_all(arrs, leaves, "count")
        assert int(total[0]) * c.discard_factor == exp
        sat = emulate_all(arrs, leaves, "or_and")
        assert int(sat[0]) == int(exp > 0)


def test_emulated_open_outputs_match_oracle():
    cnf = CNFInstance.random(3, 8, 20, rng=4)
    d = cnf.diagram()  # variables are open inputs
    c = GpuContraction(CudaRel, d.wiring, target_bits=3, trials=1)
    arrs = c.sliced_plan.native_arrays()
    got = emulate_all(arrs, _leaves(d, c), "or_and").reshape((2,) * 8)
    exp = np.zeros((2,) * 8, dtype=np.uint8)
    for idx in np.ndindex(*exp.shape):
        exp[idx] = all(any((idx[abs(l) - 1] == 1) == (l > 0) for l in cl) for cl in cnf.clauses)
    np.testing.assert_array_equal(got, exp)


def test_prepare_handles_dangling_and_repeated_wires():
    from tensorsat_gb300.diagrams import Wiring
    from tensorsat_gb300.lib.bincirc import bit

    w = Wiring(wire_types=(bit,) * 4, slot_wires_list=[(0, 0, 1)], out_wires=(1, 2))
    lw = _prepare(w)
    assert lw.leaf_wires[0] == (0, 1)
    assert 0 in lw.diag_slots
    assert (2,) in lw.leaf_wires  # dangling out wire -> all-ones leaf
    assert lw.discard_factor == 2  # wire 3 is connected to nothing
    assert lw.out_unique == (1, 2)


def test_slicing_never_touches_output_wires():
    cnf = CNFInstance.random(3, 12, 40, rng=0)
    d = cnf.clause_diagram("_" * 4 + "?" * 8)
    c = GpuContraction(CudaRel, d.wiring, target_bits=5, trials=1)
    assert not set(c.sliced_wires) & set(d.wiring.out_wires)


def _primal_degeneracy(num_vars: int, clauses) -> int:
    """Degeneracy of the primal graph (variables adjacent when they share a clause): the
    largest minimum degree met while repeatedly deleting a minimum-degree vertex. It is a
    lower bound on the graph's treewidth."""
    adj = {v: set() for v in range(num_vars)}
    for c in clauses:
        vs = {abs(l) - 1 for l in c}
        for v in vs:
            adj[v] |= vs - {v}
    deg = 0
    while adj:
        v = min(adj, key=lambda x: len(adj[x]))
        deg = max(deg, len(adj[v]))
        for u in adj.pop(v):
            adj[u].discard(v)
    return deg


def test_5sat_n100_m2100_admits_no_tree_under_the_2_30_cap():
    """Uniform random 5-SAT with n=100, m=2100, sliced over 8 wires, cannot keep every
    intermediate at 2^30 entries or fewer, whatever the tree.

    The wire sets of a tree's steps (both operands' wires together) are the bags of a tree
    decomposition of the primal graph, so some step spans at least treewidth + 1 wires,
    and one of its two operands carries at least half of them. Slicing 8 wires deletes 8
    vertices, which lowers the treewidth by at most 8. The treewidth is at least the
    degeneracy, 94 here, so some operand of every sliced tree has at least
    ceil((94 - 8 + 1) / 2) = 44 > 30 wires."""
    cnf = CNFInstance.random(5, 100, 2100, rng=0)
    deg = _primal_degeneracy(100, cnf.clauses)
    assert deg >= 94
    assert -(-(deg - 8 + 1) // 2) > 30
    d = cnf.clause_diagram()
    net = planner.Network([tuple(ws) for ws in d.wiring.slot_wires_list],
                          {w: 2 for w in range(d.wiring.num_wires)}, ())
    tree, _ = planner.optimize(net, target_bits=None, trials=1, seed=0, reconf=0)
    assert tree.cost(frozenset())[1] >= deg  # min-fill: 97 wires at the peak


def test_5sat_largest_instance_under_the_cap_plans_to_256_slices():
    """At clause ratio 21, n=39 (m=819) is where the planner's 5-SAT trees reach the 2^30
    cap with 8 sliced wires (256 slices); every launch of that plan passes the host
    bounds checks in every ring."""
    from tensorsat_gb300 import _native
    from tensorsat_gb300.contractions.gpu import PRIMES_31

    cnf = CNFInstance.random(5, 39, 819, rng=0)
    c = GpuContraction(CudaRel, cnf.clause_diagram().wiring, target_bits=30, trials=2)
    assert c.num_slices == 256 and c.stats()["peak_bits"] == 30
    npl = c.native_plan()
    for ring, primes in [(_native.TSG_RING_OR_AND, ()), (_native.TSG_RING_U64, ()),
                         (_native.TSG_RING_MODP, PRIMES_31[:3])]:
        npl.validate(ring, primes, 0, c.num_slices, 2)
    assert npl.workspace_bytes(_native.TSG_RING_MODP, 3, 2) < 80 * 2**30


@pytest.mark.parametrize("n,m,seed,target", [(12, 200, 0, 6), (14, 294, 1, 6), (16, 336, 2, 8)])
def test_emulated_5sat_sliced_plan_counts(n, m, seed, target):
    cnf = CNFInstance.random(5, n, m, rng=seed)
    exp = orc.brute_force_count(n, cnf.clauses)
    d = cnf.clause_diagram()
    c = GpuContraction(CudaRel, d.wiring, target_bits=target, trials=1, seed=seed)
    assert c.num_slices > 1
    arrs = c.sliced_plan.native_arrays()
    leaves = _leaves(d, c)
    assert int(emulate_all(arrs, leaves, "count")[0]) * c.discard_factor == exp
    assert int(emulate_all(arrs, leaves, "or_and")[0]) == int(exp > 0)


def test_native_subset_dp_equals_python_restatement():
    """tsg_plan_subset_dp against the pure-Python dynamic program: random subtrees with
    1-3 words of wires, with and without a cap, must give the same cost, splits and kept
    wires (bit for bit)."""
    import random

    from plan_dp_reference import subset_dp_reference

    rng = random.Random(0)
    for trial in range(60):
        n = rng.randint(1, 9)
        nw = rng.choice([5, 20, 63, 64, 65, 130])
        bits = [sum(1 << w for w in rng.sample(range(nw), rng.randint(0, min(nw, 12))))
                for _ in range(n)]
        keep = sum(1 << w for w in range(nw) if rng.random() < 0.2)
        live = sum(1 << w for w in range(nw) if rng.random() < 0.9)
        max_bits = rng.choice([None, 4, 8, 12])
        got_best, got_split, got_kept = planner.subset_dp(n, nw, bits, keep, live, max_bits)
        best, split, kept = subset_dp_reference(n, bits, keep, live, max_bits)
        assert got_best == best, trial
        assert [int(x) for x in got_split] == split, trial
        words = got_kept.shape[1]
        assert [sum(int(k) << (64 * w) for w, k in enumerate(row)) for row in got_kept] == kept
        assert words == max(1, (nw + 63) // 64)


@pytest.mark.parametrize("k,n,m,seed,target,trials", [(3, 30, 128, 0, 14, 2), (3, 36, 150, 3, 16, 2),
                                                     (5, 20, 420, 0, 12, 1),
                                                     (3, 60, 256, 0, 26, 2)])
def test_plans_with_native_dp_equal_python_dp_plans(monkeypatch, k, n, m, seed, target, trials):
    """Whole plans (reconfiguration before and after slicing) are the same trees and
    sliced wires whichever implementation of the subset DP runs."""
    from plan_dp_reference import subset_dp_reference

    cnf = CNFInstance.random(k, n, m, rng=seed)
    d = cnf.clause_diagram()
    net = planner.Network([tuple(ws) for ws in d.wiring.slot_wires_list],
                          {w: 2 for w in range(d.wiring.num_wires)}, ())
    native = planner.optimize(net, target_bits=target, trials=trials, seed=seed)

    def python_dp(n_, num_wires, bits, keep, live, max_bits):
        best, split, kept = subset_dp_reference(n_, bits, keep, live, max_bits)
        words = [[(v >> (64 * w)) & (2**64 - 1) for w in range(max(1, -(-v.bit_length() // 64)))]
                 for v in kept]
        return best, np.array(split, dtype=np.uint64), words

    monkeypatch.setattr(planner, "subset_dp", python_dp)
    reference = planner.optimize(net, target_bits=target, trials=trials, seed=seed)
    assert native[0].steps == reference[0].steps
    assert native[0].node_wires == reference[0].node_wires
    assert native[1] == reference[1]


def test_plans_round_trip_through_json(tmp_path):
    cnf = CNFInstance.random(3, 16, 68, rng=1)
    d = cnf.clause_diagram()
    c = GpuContraction(CudaRel, d.wiring, target_bits=6, trials=1)
    path = tmp_path / "plan.json"
    c.save_plan(path)
    again = GpuContraction.from_plan(CudaRel, d.wiring, path)
    assert again.tree.steps == c.tree.steps and again.tree.node_wires == c.tree.node_wires
    assert again.sliced_wires == c.sliced_wires
    for k, v in c.sliced_plan.native_arrays().items():
        np.testing.assert_array_equal(again.sliced_plan.native_arrays()[k], v)
    other = CNFInstance.random(3, 16, 68, rng=2).clause_diagram()
    with pytest.raises(ValueError):
        GpuContraction.from_plan(CudaRel, other.wiring, path)
    with pytest.raises(ValueError):
        planner.plan_from_dict({"format": "something else"})
    bad = c.plan_dict()
    bad["steps"][0] = [0, 0]
    with pytest.raises(ValueError):
        planner.plan_from_dict(bad)


def test_checkpointed_count_resumes_after_an_interruption(tmp_path, monkeypatch):
    """count_checkpointed records each finished chunk; after a failure mid-run a second
    call counts only the chunks still missing, and the total is the sum over all slices.
    The per-chunk GPU count is replaced by a host function of the slice range here (the
    real one, GpuContraction.count with slice_range, is covered by the GPU tests)."""
    cnf = CNFInstance.random(3, 20, 85, rng=2)
    d = cnf.clause_diagram()
    c = GpuContraction(CudaRel, d.wiring, target_bits=8, trials=1)
    ns = c.num_slices
    assert ns >= 8
    calls = []

    def fake_count(self, diagram, *, ring, num_primes, group, slice_range):
        assert slice_range[0] % group == 0
        calls.append(slice_range)
        if len(calls) == 3 and fail["on"]:
            raise RuntimeError("interrupted")
        return sum(range(*slice_range)) + 1

    fail = {"on": True}
    monkeypatch.setattr(GpuContraction, "count", fake_count)
    path = tmp_path / "count.json"
    with pytest.raises(RuntimeError):
        c.count_checkpointed(d, path, chunk_slices=ns // 8, group=64)
    assert len(calls) == 3
    fail["on"] = False
    calls.clear()
    total = c.count_checkpointed(d, path, chunk_slices=ns // 8, group=64)
    assert len(calls) == 8 - 2  # the two finished chunks are not recounted
    assert total == sum(range(ns)) + 8
    calls.clear()
    assert c.count_checkpointed(d, path, chunk_slices=ns // 8, group=64) == total
    assert calls == []
    with pytest.raises(ValueError):  # other arguments, same file
        c.count_checkpointed(d, path, chunk_slices=ns // 4, group=64)


def test_checkpointed_count_rejects_other_leaves(tmp_path, monkeypatch):
    """A checkpoint records a digest of the leaf tensors: resuming it with a diagram of the
    same wiring but another clause tensor (one literal's sign flipped) raises ValueError
    instead of adding chunk counts of another instance."""
    cnf = CNFInstance.random(3, 20, 85, rng=2)
    flipped = [list(c) for c in cnf.clauses]
    flipped[0][0] = -flipped[0][0]
    other = CNFInstance(cnf.num_vars, flipped)
    d, d2 = cnf.clause_diagram(), other.clause_diagram()
    assert d2.wiring == d.wiring
    c = GpuContraction(CudaRel, d.wiring, target_bits=8, trials=1)
    assert c.leaf_digest(d) != c.leaf_digest(d2)
    assert c.leaf_digest(d) == c.leaf_digest(cnf.clause_diagram())

    def fake_count(self, diagram, *, ring, num_primes, group, slice_range):
        if calls and fail["on"]:
            raise RuntimeError("interrupted")
        calls.append(slice_range)
        return 1

    calls: list = []
    fail = {"on": True}
    monkeypatch.setattr(GpuContraction, "count", fake_count)
    path = tmp_path / "count.json"
    with pytest.raises(RuntimeError):
        c.count_checkpointed(d, path, chunk_slices=c.num_slices // 4, group=64)
    assert len(calls) == 1
    fail["on"] = False
    with pytest.raises(ValueError, match="other leaf tensors"):
        c.count_checkpointed(d2, path, chunk_slices=c.num_slices // 4, group=64)
    assert c.count_checkpointed(d, path, chunk_slices=c.num_slices // 4, group=64) == 4


def test_checkpointed_count_argument_errors(tmp_path):
    cnf = CNFInstance.random(3, 12, 50, rng=0)
    closed = cnf.clause_diagram()
    c = GpuContraction(CudaRel, closed.wiring, target_bits=4, trials=1)
    with pytest.raises(ValueError):
        c.count_checkpointed(closed, tmp_path / "a.json", chunk_slices=0, group=1)
    opened = cnf.clause_diagram("_" + "?" * 11)
    o = GpuContraction(CudaRel, opened.wiring, target_bits=4, trials=1)
    with pytest.raises(ValueError):
        o.count_checkpointed(opened, tmp_path / "b.json", chunk_slices=4, group=1)
    (tmp_path / "c.json").write_text('{"format": "something else"}')
    with pytest.raises(ValueError):
        c.count_checkpointed(closed, tmp_path / "c.json", chunk_slices=4, group=1)


def test_vectorised_slicing_matches_the_set_based_restatement():
    """planner.slice_tree / unslice evaluate all candidate wires of a round at once; they
    pick exactly the wires the one-cost-per-candidate restatement picks (same sums in the
    same order), on min-fill trees of random 3-, 4- and 5-SAT networks at several caps."""
    from plan_dp_reference import slice_tree_reference, unslice_reference

    from tensorsat_gb300.contractions.gpu import _network, _prepare

    cases = [(3, 30, 128, 1), (3, 44, 187, 2), (3, 60, 256, 0), (4, 26, 250, 3), (5, 22, 300, 4)]
    for k, n, m, seed in cases:
        net = _network(_prepare(CNFInstance.random(k, n, m, rng=seed).clause_diagram().wiring))
        rng = random.Random(seed)
        tree = planner.build_tree(net, planner.minfill_order(net, rng,
                                                             planner.simplify_order(net)))
        forbid = frozenset(net.out_wires)
        peak = tree.cost(frozenset())[1]
        for cap in (peak - 1, peak - 4, max(6, peak - 10), 22):
            if cap >= peak or cap < 1:
                continue
            try:
                want = slice_tree_reference(tree, cap, forbid)
            except ValueError:
                continue
            got = planner.slice_tree(tree, cap, forbid)
            assert got == want, (k, n, seed, cap)
            assert planner.unslice(tree, got, cap + 2) == unslice_reference(tree, got, cap + 2)
