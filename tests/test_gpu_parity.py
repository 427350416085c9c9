"""GPU parity tests: every result of the CUDA path is compared, bit for bit, with the
reference's own outputs (golden fixtures) or with the CPU oracle on the same inputs."""

from __future__ import annotations

import json
from pathlib import Path

import numpy as np
import pytest
import torch

from oracle import finrel_oracle as orc
from tensorsat_gb300 import _native
from tensorsat_gb300.contractions.gpu import PRIMES_31, GpuContraction
from tensorsat_gb300.contractions.simple import SimpleContraction
from tensorsat_gb300.lang.cuda_rel import CudaRel, FinSet
from tensorsat_gb300.lib import bincirc
from tensorsat_gb300.lib.sat import CNFInstance

pytestmark = pytest.mark.gpu
GOLDEN = Path(__file__).resolve().parent / "golden"


def _json(name):
    return json.loads((GOLDEN / name).read_text())


def test_native_library_is_the_compute_path(cuda):
    lib = _native.lib()
    assert lib.tsg_abi_version() == 1
    box = CudaRel._contract2(bincirc.or_, [0, 1, 2], bincirc.bit_1, [2], [0, 1])
    assert box.tensor.device.type == "cuda"
    assert box.numpy().tolist() == [[0, 1], [1, 1]]


def test_contract2_golden_vectors(cuda):
    cases = _json("contract2.json")
    arrays = np.load(GOLDEN / "contract2.npz")
    n = divergent = 0
    for c in cases:
        if c["kind"] != "contract2":
            continue
        i = c["id"]
        a, b = arrays[f"c{i}_lhs"], arrays[f"c{i}_rhs"]
        res = CudaRel._contract2(CudaRel(a), c["lhs_wires"], CudaRel(b), c["rhs_wires"],
                                 c["out_wires"]).numpy()
        ref = arrays[f"c{i}_out"]
        exact = orc.contract2_einsum_definition(a, c["lhs_wires"], b, c["rhs_wires"],
                                                c["out_wires"])
        if np.array_equal(ref, exact):
            np.testing.assert_array_equal(res.reshape(ref.shape), ref, err_msg=str(c))
            n += 1
        else:
            # upstream rewire_array transposes interleaved repeated wires; the kernel
            # follows the einsum definition (documented divergence)
            np.testing.assert_array_equal(res.reshape(exact.shape), exact, err_msg=str(c))
            divergent += 1
    assert n > 100 and divergent <= 10


def test_rewire_golden_vectors(cuda):
    cases = _json("contract2.json")
    arrays = np.load(GOLDEN / "contract2.npz")
    n = 0
    for c in cases:
        if c["kind"] != "rewire":
            continue
        i = c["id"]
        t = arrays[f"c{i}_in"]
        res = CudaRel(t)._rewire(c["out_ports"]).numpy()
        ref = arrays[f"c{i}_out"]
        ports = list(range(t.ndim))
        exact = orc.contract2_einsum_definition(t, ports, np.ones((), np.uint8), [],
                                                c["out_ports"])
        np.testing.assert_array_equal(res.reshape(exact.shape),
                                      ref if np.array_equal(ref, exact) else exact, err_msg=str(c))
        n += 1
    assert n > 30


def test_count_u64_per_step_matches_oracle(cuda):
    rng = np.random.default_rng(7)
    lib = _native.lib()
    for _ in range(40):
        lw = [int(x) for x in rng.integers(0, 5, size=int(rng.integers(1, 5)))]
        rw = [int(x) for x in rng.integers(0, 5, size=int(rng.integers(1, 5)))]
        dims = {w: int(rng.integers(1, 4)) for w in range(5)}
        present = sorted(set(lw) | set(rw))
        ow = [int(x) for x in rng.choice(present, size=int(rng.integers(0, len(present) + 1)),
                                         replace=False)]
        a = rng.integers(0, 50, size=[dims[w] for w in lw]).astype(np.uint64)
        b = rng.integers(0, 50, size=[dims[w] for w in rw]).astype(np.uint64)
        ta = torch.from_numpy(a.view(np.int64)).to(cuda)
        tb = torch.from_numpy(b.view(np.int64)).to(cuda)
        out = torch.empty([dims[w] for w in ow], dtype=torch.int64, device=cuda)
        st = lib.tsg_contract2_count_u64(
            ta.data_ptr(), len(lw), _native.i64_array(lw), _native.i64_array(a.shape),
            tb.data_ptr(), len(rw), _native.i64_array(rw), _native.i64_array(b.shape),
            len(ow), _native.i64_array(ow), out.data_ptr(), 0)
        _native.check(st)
        torch.cuda.synchronize()
        exp = orc.contract2_count(a, lw, b, rw, ow).astype(np.uint64)
        np.testing.assert_array_equal(out.cpu().numpy().view(np.uint64), exp)


def test_modp_per_step_matches_oracle(cuda):
    """tsg_contract2_modp: per plane, the residues of the exact einsum (the oracle's integer
    count of the same contraction) modulo each prime; 3 planes, repeated and summed wires,
    and sums long enough for the split-K form."""
    rng = np.random.default_rng(11)
    lib = _native.lib()
    primes = [2147483647, 2147483629, 2147483587]
    arr = (_native.c_uint32 * 3)(*primes)
    for case in range(40):
        if case >= 34:  # at most 2 outputs over 2^10 or more summed entries (split-K form)
            lw = [int(x) for x in rng.choice(12, size=10, replace=False)]
            rw = [int(x) for x in rng.choice(12, size=10, replace=False)]
            dims = {w: 2 for w in range(12)}
            ow = [int(x) for x in rng.choice(sorted(set(lw) | set(rw)),
                                             size=int(rng.integers(0, 2)), replace=False)]
        else:
            lw = [int(x) for x in rng.integers(0, 5, size=int(rng.integers(1, 5)))]
            rw = [int(x) for x in rng.integers(0, 5, size=int(rng.integers(1, 5)))]
            dims = {w: int(rng.integers(1, 4)) for w in range(5)}
            present = sorted(set(lw) | set(rw))
            ow = [int(x) for x in rng.choice(present, size=int(rng.integers(0, len(present) + 1)),
                                             replace=False)]
        a = rng.integers(0, 1 << 31, size=[3] + [dims[w] for w in lw], dtype=np.int64)
        b = rng.integers(0, 1 << 31, size=[3] + [dims[w] for w in rw], dtype=np.int64)
        for q, p in enumerate(primes):
            a[q] %= p
            b[q] %= p
        ta = torch.from_numpy(a.astype(np.uint32).view(np.int32)).to(cuda)
        tb = torch.from_numpy(b.astype(np.uint32).view(np.int32)).to(cuda)
        out = torch.empty([3] + [dims[w] for w in ow], dtype=torch.int32, device=cuda)
        _native.check(lib.tsg_contract2_modp(
            ta.data_ptr(), len(lw), _native.i64_array(lw), _native.i64_array(a.shape[1:]),
            tb.data_ptr(), len(rw), _native.i64_array(rw), _native.i64_array(b.shape[1:]),
            len(ow), _native.i64_array(ow), 3, arr, out.data_ptr(), 0))
        torch.cuda.synchronize()
        got = out.cpu().numpy().view(np.uint32)
        for q, p in enumerate(primes):
            exact = orc.contract2_count(a[q].astype(object), lw, b[q].astype(object), rw, ow)
            want = np.vectorize(lambda x: int(x) % p, otypes=[object])(np.asarray(exact, dtype=object))
            np.testing.assert_array_equal(got[q].astype(np.int64), want.astype(np.int64),
                                          err_msg=str((case, q, lw, rw, ow)))


def test_union_spider_scalar_stack(cuda):
    a = CudaRel(np.array([[0, 1], [0, 0]], dtype=np.uint8))
    b = CudaRel(np.array([[0, 0], [1, 0]], dtype=np.uint8))
    assert (a + b).numpy().tolist() == [[0, 1], [1, 0]]
    for dim, ports in [(2, 1), (2, 3), (3, 2), (1, 4)]:
        np.testing.assert_array_equal(CudaRel.spider(FinSet(dim), ports).numpy(),
                                      orc.spider(dim, ports))
    assert bool(CudaRel.scalar(True)) and not bool(CudaRel.scalar(False))
    st = CudaRel.stack([a, b], 1)
    np.testing.assert_array_equal(st.numpy(), np.stack([a.numpy(), b.numpy()], axis=1))
    assert a[1, :].numpy().tolist() == [0, 0]


def test_notebook_contract2_examples(cuda):
    kats = _json("notebook_kats.json")
    bit = bincirc.bit
    cnot = CudaRel.contract2(CudaRel.spider(bit, 3), [0, 2, 4], bincirc.xor_, [4, 1, 3],
                             [0, 1, 2, 3])
    assert sorted(map(list, cnot.to_set())) == kats["cnot"]
    assert cnot == CudaRel.from_callable((2, 2), (2, 2), lambda a, b: (a, a ^ b))
    func = CudaRel.contract2(bincirc.or_, [1, 2, 3], bincirc.and_, [0, 3, 4])
    assert sorted(map(list, func.to_set())) == kats["a_and_b_or_c"]
    f1 = CudaRel.contract2(bincirc.or_, [0, 2, 3], bincirc.or_, [1, 2, 4], [0, 1, 2, 3, 4])
    f2 = CudaRel.contract2(f1, [0, 1, 2, 3, 4], bincirc.and_, [3, 4, 5])
    assert sorted(map(list, f2.to_set())) == kats["a_or_c_and_b_or_c"]


@pytest.mark.parametrize("case", _json("kissat.json"), ids=lambda c: c["test"])
def test_kissat_known_answers(cuda, case):
    cnf = CNFInstance(case["num_vars"], [tuple(c) for c in case["clauses"]])
    diagram = (cnf.inputs(None) >> cnf.diagram()).flatten()
    contraction = GpuContraction(CudaRel, diagram.wiring, optimize="greedy", trials=2)
    sat = bool(contraction.contract(diagram))
    assert sat == case["expected"] == case["sat_reference"]
    assert contraction.count(diagram) == int(case["count"])


@pytest.mark.parametrize("seed", range(8))
def test_random_3sat_n20_sat_and_count(cuda, seed):
    cnf = CNFInstance.random(3, 20, 85, rng=seed)
    expected = orc.brute_force_count(20, cnf.clauses)
    bintree = (cnf.inputs(None) >> cnf.diagram()).flatten()
    clause = cnf.clause_diagram()
    for d in (bintree, clause):
        c = GpuContraction(CudaRel, d.wiring)
        assert bool(c.contract(d)) == (expected > 0)
        assert c.count(d, ring="u64") == expected
        assert c.count(d, ring="modp", num_primes=3) == expected
        assert c.count(d, ring="modp", num_primes=1) == expected % PRIMES_31[0]


@pytest.mark.parametrize("target_bits", [4, 6, 9])
def test_sliced_plans_all_groups(cuda, target_bits):
    cnf = CNFInstance.random(3, 18, 76, rng=11)
    expected = orc.brute_force_count(18, cnf.clauses)
    d = cnf.clause_diagram()
    c = GpuContraction(CudaRel, d.wiring, target_bits=target_bits, trials=2)
    assert c.num_slices > 1
    for group in sorted({1, 2, min(8, c.num_slices), c.num_slices}):
        assert c.count(d, ring="u64", group=group) == expected
        assert c.count(d, ring="modp", num_primes=2, group=group) == expected
        assert bool(c.contract(d, group=group)) == (expected > 0)


def test_slice_ranges_accumulate(cuda):
    cnf = CNFInstance.random(3, 18, 70, rng=5)
    expected = orc.brute_force_count(18, cnf.clauses)
    d = cnf.clause_diagram()
    c = GpuContraction(CudaRel, d.wiring, target_bits=6, trials=1)
    ns = c.num_slices
    res = None
    for b in range(0, ns, 2):
        res = c.run(d, _native.TSG_RING_U64, slice_range=(b, min(ns, b + 2)), group=2,
                    result=res, accumulate=res is not None)
    assert int(res.cpu().numpy().view(np.uint64)[0]) * c.discard_factor == expected
    # per-slice parity with the oracle
    sl = c.sliced_wires
    for sid in (0, ns - 1, ns // 3):
        r = c.run(d, _native.TSG_RING_U64, slice_range=(sid, sid + 1), group=1)
        fixed = {w: (sid >> j) & 1 for j, w in enumerate(sl)}
        exp = orc.cnf_count_by_tree(18, cnf.clauses, c.tree.steps, fixed=fixed)
        assert int(r.cpu().numpy().view(np.uint64)[0]) * c.discard_factor == exp


def test_open_outputs_solution_set(cuda):
    kats = _json("notebook_kats.json")
    cnf = CNFInstance.random(4, 10, 95, rng=0)
    d = cnf.diagram()
    c = GpuContraction(CudaRel, d.wiring)
    box = c.contract(d)
    assert sorted(map(list, box.to_set())) == kats["ksat4_n10_m95_rng0_solutions"]
    counts = c.count(d)
    assert counts.shape == (2,) * 10
    assert {tuple(i) for i in zip(*np.nonzero(counts.astype(np.int64)))} == box.to_set()


def test_assignment_search_reuses_one_plan(cuda):
    kats = _json("notebook_kats.json")
    cnf = CNFInstance.random(4, 20, 195, rng=1)
    d = cnf.diagram()
    plan_wiring = cnf.contraction_wiring()
    contraction = GpuContraction(CudaRel, plan_wiring)
    assert bool(contraction.contract((cnf.inputs(0) >> d).flatten())) in (True, False)
    trace = []
    for cand, _ in kats["ksat4_n20_m195_rng1_assignment_search"]["trace"]:
        diag = (cnf.inputs(cand) >> d).flatten()
        trace.append([cand, bool(contraction.contract(diag))])
    assert trace == kats["ksat4_n20_m195_rng1_assignment_search"]["trace"]


def test_temporary_variants_do_not_share_a_cached_pool(cuda):
    """One plan, leaf variants passed as unnamed temporaries in a loop: each freed
    diagram's id may be reused by the next one, so the leaf-pool cache must not match on
    ids. The SAT bits and counts of every variant equal brute force."""
    cnf = CNFInstance.random(3, 12, 40, rng=5)
    d = cnf.diagram()
    c = GpuContraction(CudaRel, cnf.contraction_wiring())
    specs = [f"{a:012b}" for a in range(0, 4096, 97)]
    want = [orc.brute_force_count(12, list(cnf.clauses) + [(i + 1,) if b == "1" else (-(i + 1),)
                                                       for i, b in enumerate(s)]) > 0
            for s in specs]
    assert any(want) and not all(want)
    got = [bool(c.contract((cnf.inputs(s) >> d).flatten())) for s in specs]
    assert got == want
    counts = [c.count((cnf.inputs(s) >> d).flatten()) for s in specs]
    assert counts == [int(w) for w in want]


def test_empty_clause_network_counts_zero(cuda):
    """A clause with no literal is a 0-port tensor holding 0: the network has no model.
    Its SAT bit and counts match the oracle's DPLL counter, in every ring."""
    for clauses in ([(1, 2), (), (-3,)], [(1,), ()], [(1,), (-1, 2), ()]):
        n = max([abs(l) for c in clauses for l in c] or [1])
        cnf = CNFInstance(n, clauses)
        d = cnf.clause_diagram()
        assert any(orc_shape == () for orc_shape in
                   (tuple(b.tensor.shape) for b in d.blocks))
        c = GpuContraction(CudaRel, d.wiring)
        assert orc.dpll_count(n, clauses)[0] == 0
        assert c.count(d, ring="u64") == 0
        assert c.count(d, ring="modp", num_primes=2) == 0
        assert bool(c.contract(d)) is False


def test_sharp_sat_example(cuda):
    kats = _json("notebook_kats.json")["sharp_sat_example"]
    cnf = CNFInstance(3, [tuple(c) for c in kats["clauses"]])
    d = (cnf.inputs(None) >> cnf.diagram()).flatten()
    c = GpuContraction(CudaRel, d.wiring)
    assert c.count(d) == kats["count"] == 6
    assert bool(c.contract(d)) == kats["sat"]


def test_simple_contraction_matches_oracle(cuda):
    # SimpleContraction keeps every wire until the root (as upstream): keep it small
    cnf = CNFInstance(3, [(1, -2), (2, 3), (-1, -3)])
    d = (cnf.inputs(None) >> cnf.diagram()).flatten()
    n = d.wiring.num_slots
    path = [(0, 1)] * (n - 1)
    box = SimpleContraction(CudaRel, d.wiring, path).contract(d)
    assert bool(box) == (orc.brute_force_count(3, cnf.clauses) > 0)
    three = CNFInstance(3, [(1, 2), (-1, 3)])
    inp = three.inputs("01?")
    sc = SimpleContraction(CudaRel, inp.wiring, [(0, 1), (0, 1)])
    assert sc.contract(inp).to_set() == {(0, 1, 0), (0, 1, 1)}


def test_autoray_einsum(cuda):
    from tensorsat_gb300 import _autoray

    res = _autoray.einsum("abd,dce->abce", bincirc.or_, bincirc.or_)
    exp = orc.contract2_or_and(bincirc.or_.numpy(), [0, 1, 2], bincirc.or_.numpy(), [2, 3, 4],
                               [0, 1, 3, 4])
    np.testing.assert_array_equal(res.numpy(), exp)
    un = _autoray.einsum("ab->a", bincirc.not_)
    assert un.numpy().tolist() == [1, 1]


@pytest.mark.parametrize("n,m,seed,target", [(40, 170, 0, 20), (36, 150, 3, 16)])
def test_sliced_count_properties(cuda, n, m, seed, target):
    """Size-independent checks where brute force is out of reach: the u64 count equals the
    3-prime CRT count, the SAT bit agrees with count > 0, a different tree and slicing give
    the same count, and single slices match the oracle."""
    cnf = CNFInstance.random(3, n, m, rng=seed)
    d = cnf.clause_diagram()
    c1 = GpuContraction(CudaRel, d.wiring, target_bits=target, trials=2, seed=0)
    c2 = GpuContraction(CudaRel, d.wiring, target_bits=target - 2, trials=2, seed=1)
    n1 = c1.count(d, ring="u64")
    assert n1 == c1.count(d, ring="modp", num_primes=3)
    assert n1 == c2.count(d, ring="modp", num_primes=3)
    assert bool(c1.contract(d)) == (n1 > 0) == bool(c2.contract(d))
    sl = c1.sliced_wires
    sid = c1.num_slices // 2
    r = c1.run(d, _native.TSG_RING_U64, slice_range=(sid, sid + 1), group=1)
    fixed = {w: (sid >> j) & 1 for j, w in enumerate(sl)}
    assert int(r.cpu().numpy().view(np.uint64)[0]) * c1.discard_factor == orc.cnf_count_by_tree(
        n, cnf.clauses, c1.tree.steps, fixed=fixed)


def test_timed_run_matches_plain_run(cuda):
    """tsg_plan_run_timed gives the results of tsg_plan_run (integers: equality) and one
    non-negative device time per tree step plus the root reductions."""
    cnf = CNFInstance.random(3, 30, 128, rng=4)
    d = cnf.clause_diagram()
    c = GpuContraction(CudaRel, d.wiring, target_bits=14, trials=2)
    npl = c.native_plan()
    ns = c.num_slices
    group = min(8, ns)
    pool = c.leaf_pool(d)
    stream = torch.cuda.current_stream().cuda_stream
    for ring, primes, nres, dt in [(_native.TSG_RING_MODP, PRIMES_31[:3], 3, torch.int32),
                                   (_native.TSG_RING_OR_AND, (), 1, torch.uint8)]:
        ws = torch.empty(npl.workspace_bytes(ring, max(1, len(primes)), group),
                         dtype=torch.uint8, device=cuda)
        plain = torch.zeros(nres, dtype=dt, device=cuda)
        timed = torch.zeros(nres, dtype=dt, device=cuda)
        npl.run(ring, primes, pool, 0, ns, group, ws, plain, False, stream)
        ms = npl.run_timed(ring, primes, pool, 0, ns, group, ws, timed, False, stream)
        torch.cuda.synchronize()
        assert torch.equal(plain, timed)
        assert len(ms) == len(c.tree.steps) + 1
        assert all(x >= 0 for x in ms) and sum(ms) > 0
