"""Batched runs of many networks (tsg_batch_run, BatchContraction).

CPU tests call the C ABI without a GPU: the shared workspace is the largest per-instance
workspace, and a batch with one bad instance is rejected by the host checks before
anything is launched. GPU tests compare a ragged batch of random 3-SAT instances (uneven
variable and clause counts, several of them sliced) with brute force and with per-instance
contractions, and replays of a captured CUDA graph with the uncaptured run. Counts and SAT
bits are integers: the tolerance is equality.
"""

from __future__ import annotations

import ctypes

import numpy as np
import pytest
import torch

from oracle import finrel_oracle as orc
from tensorsat_gb300 import _native
from tensorsat_gb300.contractions.batch import BatchContraction
from tensorsat_gb300.contractions.gpu import PRIMES_31, GpuContraction, plan_tree
from tensorsat_gb300.lang.cuda_rel import CudaRel
from tensorsat_gb300.lib.sat import CNFInstance


def ragged_instances(count: int, n_lo: int, n_hi: int, seed: int = 0) -> list[CNFInstance]:
    """Random 3-SAT instances with n uniform in [n_lo, n_hi] and clause ratio uniform in
    [3.5, 5.0], one generator per instance (seeded by its index)."""
    out = []
    for i in range(count):
        g = np.random.default_rng(seed * 100_003 + i)
        n = int(g.integers(n_lo, n_hi + 1))
        m = round(float(g.uniform(3.5, 5.0)) * n)
        out.append(CNFInstance.random(3, n, m, rng=g))
    return out


def _plans(instances, target_bits):
    return [GpuContraction(CudaRel, cnf.clause_diagram().wiring, target_bits=target_bits,
                           trials=1).native_plan() for cnf in instances]


def test_batch_workspace_is_the_largest_instance_workspace():
    plans = _plans(ragged_instances(6, 10, 20), target_bits=8)
    lib = _native.lib()
    groups = [1, 2, 4, 1, 2, 1]
    out = ctypes.c_int64()
    handles = (ctypes.c_void_p * len(plans))(*[p.handle.value for p in plans])
    for ring, planes in [(_native.TSG_RING_OR_AND, 1), (_native.TSG_RING_MODP, 3),
                         (_native.TSG_RING_U64, 1)]:
        _native.check(lib.tsg_batch_workspace_bytes(len(plans), handles, ring, planes,
                                                    _native.i64_array(groups), ctypes.byref(out)))
        assert out.value == max(p.workspace_bytes(ring, planes, g) for p, g in zip(plans, groups))


def test_lane_workspace_holds_every_lane_region():
    """Lanes: each lane's region holds the largest workspace of the instances assigned to
    it, so the total lies between the largest single workspace (one lane) and the sum of
    all (one instance per lane); lane counts beyond the instances change nothing and
    lanes outside 1..32 are rejected."""
    plans = _plans(ragged_instances(6, 10, 20), target_bits=8)
    lib = _native.lib()
    groups = [1, 2, 4, 1, 2, 1]
    handles = (ctypes.c_void_p * len(plans))(*[p.handle.value for p in plans])
    ring, planes = _native.TSG_RING_MODP, 3
    each = [p.workspace_bytes(ring, planes, g) for p, g in zip(plans, groups)]
    align = lambda x: (x + 255) // 256 * 256
    sizes = {}
    for lanes in (1, 2, 3, 6, 32):
        out = ctypes.c_int64()
        _native.check(lib.tsg_batch_lanes_workspace_bytes(
            len(plans), handles, ring, planes, _native.i64_array(groups), lanes,
            ctypes.byref(out)))
        sizes[lanes] = out.value
    assert sizes[1] == align(max(each))
    assert sizes[6] == sizes[32] == sum(align(x) for x in each)
    assert sizes[1] <= sizes[2] <= sizes[6] and sizes[1] <= sizes[3] <= sizes[6]
    out = ctypes.c_int64()
    for bad in (0, 33):
        assert lib.tsg_batch_lanes_workspace_bytes(
            len(plans), handles, ring, planes, _native.i64_array(groups), bad,
            ctypes.byref(out)) == _native.TSG_ERR_INVALID_ARGUMENT


def test_packed_workspace_regions():
    """Packed batches: a lane's region holds its largest instance (level-order placement
    for instances run in one group of all their slices, step order otherwise), so one lane
    needs the largest single-instance requirement and one lane per instance the sum; bad
    lane counts and group sizes are rejected on the host."""
    plans = _plans(ragged_instances(6, 10, 20), target_bits=8)
    lib = _native.lib()
    full = [1 << p.num_sliced for p in plans]
    groups = [full[0], max(1, full[1] // 2), full[2], full[3], full[4], full[5]]
    handles = (ctypes.c_void_p * len(plans))(*[p.handle.value for p in plans])
    ring, planes = _native.TSG_RING_MODP, 3

    def size(hs, gs, lanes):
        out = ctypes.c_int64()
        _native.check(lib.tsg_batch_packed_workspace_bytes(
            len(gs), hs, ring, planes, _native.i64_array(gs), lanes, ctypes.byref(out)))
        return out.value

    each = [size((ctypes.c_void_p * 1)(p.handle.value), [g], 1) for p, g in zip(plans, groups)]
    assert all(e % 256 == 0 and e >= 256 for e in each)
    assert size(handles, groups, 1) == max(each)
    assert size(handles, groups, 6) == size(handles, groups, 32) == sum(each)
    # the step-order placement for the instance run in several groups
    assert each[1] == (plans[1].workspace_bytes(ring, planes, groups[1]) + 255) // 256 * 256
    out = ctypes.c_int64()
    for bad in (0, 33):
        assert lib.tsg_batch_packed_workspace_bytes(
            len(plans), handles, ring, planes, _native.i64_array(groups), bad,
            ctypes.byref(out)) == _native.TSG_ERR_INVALID_ARGUMENT
    assert lib.tsg_batch_packed_workspace_bytes(
        len(plans), handles, ring, planes, _native.i64_array([3] + groups[1:]), 2,
        ctypes.byref(out)) == _native.TSG_ERR_INVALID_ARGUMENT


def test_packed_batch_rejects_a_bad_instance_before_launching():
    plans = _plans(ragged_instances(4, 10, 16, seed=1), target_bits=6)
    lib = _native.lib()
    n = len(plans)
    handles = (ctypes.c_void_p * n)(*[p.handle.value for p in plans])
    fake = (ctypes.c_void_p * n)(*([256] * n))
    launches = ctypes.c_int64(5)
    st = lib.tsg_batch_run_packed(n, handles, _native.TSG_RING_OR_AND, 0, None, fake,
                                  _native.i64_array([1, 1, 3, 1]), 2, None, 0, fake, None,
                                  ctypes.byref(launches))
    assert st == _native.TSG_ERR_INVALID_ARGUMENT and launches.value == 0
    assert lib.tsg_batch_run_packed(n, handles, _native.TSG_RING_OR_AND, 0, None, fake,
                                    _native.i64_array([1] * n), 0, None, 0, fake, None,
                                    None) == _native.TSG_ERR_INVALID_ARGUMENT


def test_batch_rejects_a_bad_instance_before_launching():
    """Instance 2 has a group size that is not a power of two: the call fails in the host
    checks (the pointers are never dereferenced, so placeholders suffice)."""
    plans = _plans(ragged_instances(4, 10, 16, seed=1), target_bits=6)
    lib = _native.lib()
    n = len(plans)
    handles = (ctypes.c_void_p * n)(*[p.handle.value for p in plans])
    fake = (ctypes.c_void_p * n)(*([256] * n))
    groups = _native.i64_array([1, 1, 3, 1])
    st = lib.tsg_batch_run(n, handles, _native.TSG_RING_OR_AND, 0, None, fake, groups, None, 0,
                           fake, None)
    assert st == _native.TSG_ERR_INVALID_ARGUMENT
    assert "instance 2" in lib.tsg_last_error().decode()
    assert lib.tsg_batch_run(-1, None, 0, 0, None, None, None, None, 0, None, None) \
        == _native.TSG_ERR_INVALID_ARGUMENT


def test_batch_accepts_trees_planned_elsewhere():
    """plan_tree gives the tree GpuContraction would plan, so trees planned in worker
    processes can be handed to a batch."""
    instances = ragged_instances(4, 10, 16, seed=5)
    diagrams = [cnf.clause_diagram() for cnf in instances]
    trees = [plan_tree(d.wiring, target_bits=6, trials=1) for d in diagrams]
    planned = BatchContraction(CudaRel, diagrams, target_bits=6, trials=1)
    given = BatchContraction(CudaRel, diagrams, trees=trees)
    for a, b in zip(planned.contractions, given.contractions):
        assert a.tree.steps == b.tree.steps and a.sliced_wires == b.sliced_wires
    assert plan_tree(diagrams[0].wiring, target_bits=None, trials=1)[1] == ()
    with pytest.raises(ValueError):
        BatchContraction(CudaRel, diagrams, trees=trees[:-1])


@pytest.mark.gpu
def test_ragged_batch_counts_and_sat_bits_match_brute_force(cuda):
    instances = ragged_instances(12, 12, 22, seed=2)
    diagrams = [cnf.clause_diagram() for cnf in instances]
    batch = BatchContraction(CudaRel, diagrams, target_bits=9, trials=1)
    assert any(c.num_slices > 1 for c in batch.contractions)
    expected = [orc.brute_force_count(cnf.num_vars, cnf.clauses) for cnf in instances]
    assert batch.count() == expected
    assert batch.count(num_primes=3) == expected
    bits = [bool(box) for box in batch.contract()]
    assert bits == [e > 0 for e in expected]
    # the same as contracting each network on its own
    for c, d, e in zip(batch.contractions, diagrams, expected):
        assert c.count(d, ring="modp", num_primes=2) == e


@pytest.mark.gpu
def test_packed_batch_equals_lanes_and_the_checkers(cuda):
    """Packed runs (small steps of a tree level across instances in shared launches) give
    the per-step runs' results bit for bit in every ring, with fewer launches: small
    sliced instances (one group of all slices, or several groups), and unsliced n = 28-32
    instances whose large steps run as their own launches between the packed ones."""
    small = ragged_instances(10, 12, 20, seed=7)
    large = ragged_instances(4, 28, 32, seed=8)
    instances = small + large
    diagrams = [cnf.clause_diagram() for cnf in instances]
    trees = [plan_tree(d.wiring, target_bits=9 if i < len(small) else None, trials=1)
             for i, d in enumerate(diagrams)]
    packed = BatchContraction(CudaRel, diagrams, trees=trees, lanes=3)
    lanes = BatchContraction(CudaRel, diagrams, trees=trees, lanes=3, packed=False)
    assert any(c.num_slices > 1 for c in packed.contractions)
    groups = [c.num_slices for c in packed.contractions]
    j = next(i for i, c in enumerate(packed.contractions) if c.num_slices >= 4)
    groups[j] = packed.contractions[j].num_slices // 4  # this one runs in four groups
    primes = PRIMES_31[:3]
    for ring, pr in ((_native.TSG_RING_MODP, primes), (_native.TSG_RING_U64, ()),
                     (_native.TSG_RING_OR_AND, ())):
        a = [r.cpu() for r in packed.run(ring, pr, groups=groups)]
        n_packed = packed.last_launches
        b = [r.cpu() for r in lanes.run(ring, pr, groups=groups)]
        assert all(torch.equal(x, y) for x, y in zip(a, b)), ring
        assert 0 < n_packed < lanes.last_launches
    expected = [orc.brute_force_count(c.num_vars, c.clauses) for c in small] + \
               [orc.dpll_count(c.num_vars, c.clauses)[0] for c in large]
    assert packed.count(num_primes=3, groups=groups) == expected
    assert [bool(x) for x in packed.contract(groups=groups)] == [e > 0 for e in expected]


@pytest.mark.gpu
@pytest.mark.parametrize("packed", [True, False])
def test_batch_graph_replay_matches_uncaptured_run(cuda, packed):
    instances = ragged_instances(8, 14, 24, seed=3)
    batch = BatchContraction(CudaRel, [cnf.clause_diagram() for cnf in instances],
                             target_bits=10, trials=1, packed=packed)
    primes = PRIMES_31[:3]
    direct = [r.clone() for r in batch.run(_native.TSG_RING_MODP, primes)]
    sat_direct = [r.clone() for r in batch.run(_native.TSG_RING_OR_AND)]
    g = batch.capture(_native.TSG_RING_MODP, primes)
    gs = batch.capture(_native.TSG_RING_OR_AND)
    for _ in range(2):
        for r in g.results + gs.results:
            r.fill_(7)  # replays must rewrite every result
        g.replay()
        gs.replay()
        torch.cuda.synchronize()
        for a, b in zip(g.results, direct):
            assert torch.equal(a, b)
        for a, b in zip(gs.results, sat_direct):
            assert torch.equal(a, b)
    GpuContraction.check_device()


@pytest.mark.gpu
def test_batch_serving_graphs_follow_loaded_leaves(cuda):
    """count/contract with graph=True capture one graph per ring on first use and replay
    it afterwards; load() copies the leaves of new diagrams with the same wirings into the
    captured pools. Here the inputs fix variable 1 to 1, then to 0, then to 1 again (a unit
    slot whose box changes while the wiring stays), and every replay must answer for the
    leaves loaded last."""
    instances = ragged_instances(6, 12, 18, seed=4)
    one = [cnf.clause_diagram("1" + "?" * (cnf.num_vars - 1)) for cnf in instances]
    zero = [cnf.clause_diagram("0" + "?" * (cnf.num_vars - 1)) for cnf in instances]
    exp1 = [orc.brute_force_count(c.num_vars, list(c.clauses) + [(1,)]) for c in instances]
    exp0 = [orc.brute_force_count(c.num_vars, list(c.clauses) + [(-1,)]) for c in instances]
    assert exp1 != exp0
    batch = BatchContraction(CudaRel, one, target_bits=8, trials=1)
    assert any(c.num_slices > 1 for c in batch.contractions)
    for diagrams, exp in ((one, exp1), (zero, exp0), (one, exp1)):
        assert batch.load(diagrams) > 0
        assert batch.count(num_primes=3, graph=True) == exp
        assert [bool(b) for b in batch.contract(graph=True)] == [e > 0 for e in exp]
    assert len(batch._graphs) == 2  # one capture per ring, replayed ever since
    with pytest.raises(ValueError):
        batch.load(one[:-1])


@pytest.mark.gpu
def test_batch_serve_pipelines_input_batches(cuda):
    """serve() yields, per input batch, the counts and SAT bits that load() + count() /
    contract() give, while it packs the next batch during the current one's replays; the
    batches alternate between inputs with variable 1 fixed to 1 and to 0."""
    instances = ragged_instances(6, 12, 18, seed=9)
    one = [cnf.clause_diagram("1" + "?" * (cnf.num_vars - 1)) for cnf in instances]
    zero = [cnf.clause_diagram("0" + "?" * (cnf.num_vars - 1)) for cnf in instances]
    exp1 = [orc.brute_force_count(c.num_vars, list(c.clauses) + [(1,)]) for c in instances]
    exp0 = [orc.brute_force_count(c.num_vars, list(c.clauses) + [(-1,)]) for c in instances]
    batch = BatchContraction(CudaRel, one, target_bits=8, trials=1)
    stream = [one, zero, one, zero, zero]
    want = [exp1, exp0, exp1, exp0, exp0]
    got = list(batch.serve(stream, num_primes=3))
    assert len(got) == len(stream)
    for (counts, boxes), exp in zip(got, want):
        assert counts == exp
        assert [bool(b) for b in boxes] == [e > 0 for e in exp]
    assert len(batch._graphs) == 2  # one capture per ring


def test_batch_prime_count_is_cached_while_leaves_shrink():
    """primes_needed() is computed once; a new input batch whose leaf entries are all at
    most the first ones keeps it (counts only shrink), any larger entry drops it."""
    instances = ragged_instances(3, 10, 14, seed=6)
    free = [cnf.clause_diagram() for cnf in instances]
    fixed = [cnf.clause_diagram("1" + "?" * (cnf.num_vars - 1)) for cnf in instances]
    batch = BatchContraction(CudaRel, free, target_bits=8, trials=1)
    need = batch.primes_needed()
    assert batch._need == need and batch._need_pool is not None
    parts = [c._host_pool(d) for c, d in zip(batch.contractions, fixed)]
    staged = np.concatenate([h for h, _ in parts])
    assert np.all(staged <= batch._need_pool)
    batch._keep_bound(staged, [dl for _, dl in parts])
    assert batch._need == need
    bigger = staged.copy()
    bigger[np.argmin(batch._need_pool)] = 1 if batch._need_pool.min() == 0 else 255
    batch._keep_bound(bigger, [])
    assert batch._need is None
    assert batch.primes_needed() == need


def test_ragged_plan_only_report_runs_on_the_host():
    """bench.py --workload ragged --plan-only plans a batch on the host cores and reports
    its algorithmic bytes per n without touching a GPU."""
    import json
    import subprocess
    import sys
    from pathlib import Path

    root = Path(__file__).resolve().parent.parent
    out = subprocess.run([sys.executable, str(root / "bench.py"), "--workload", "ragged",
                          "--instances", "6", "--n-range", "12", "16", "--plan-only"],
                         capture_output=True, text=True, timeout=600, check=True)
    line = json.loads(out.stdout.strip().splitlines()[-1])
    assert line["plan_only"] is True
    assert sum(b["instances"] for b in line["by_n"].values()) == 6
    assert line["total_bytes"] > 0 and line["peak_bits_max"] <= 26


def test_batch_load_checks_its_diagrams_before_any_device_work():
    instances = ragged_instances(3, 10, 14, seed=6)
    one = [cnf.clause_diagram("1" + "?" * (cnf.num_vars - 1)) for cnf in instances]
    batch = BatchContraction(CudaRel, one, target_bits=6, trials=1)
    with pytest.raises(ValueError):
        batch.load(one[:-1])  # wrong count
    with pytest.raises(ValueError):
        batch.load(list(reversed(one)))  # other wirings


def test_reference_arm_prints_its_line_on_the_host():
    """bench.py --impl reference times the oracle's restatement of the reference's numpy
    path on the host cores, loading the committed plan without the native library, and
    prints one JSON line with the reference arm's keys."""
    import json
    import subprocess
    import sys
    from pathlib import Path

    root = Path(__file__).resolve().parent.parent
    out = subprocess.run([sys.executable, str(root / "bench.py"), "--impl", "reference",
                          "--steps", "1", "--warmup", "0"],
                         capture_output=True, text=True, timeout=900, check=True)
    line = json.loads(out.stdout.strip().splitlines()[-1])
    assert line["impl"] == "reference" and line["value"] > 0
    assert line["cpu_baseline"]["kind"] == "port" and line["cpu_baseline"]["cores"] >= 1
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["e2e"]["value"] == line["value"]
    assert line["config"]["slices_per_instance"] == 8192
