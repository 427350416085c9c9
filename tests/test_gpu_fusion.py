"""Fused steps on the GPU: a step whose large result is read once, as its consumer's reused
operand, is computed inside the consumer (asked for with TSG_STEP_FUSE step options, in the
tile and the streaming form). Fused and unfused runs give identical results, and both
equal the oracle's contraction of single slices along the same tree.

The leaves here are random {0,1} tensors on the wiring of CNF clause networks, so the
per-slice counts are large and varied (a CNF network's counts are mostly zero), and every
fused index map is exercised with non-trivial values.
"""

from __future__ import annotations

import numpy as np
import pytest

from oracle import finrel_oracle as orc
from tensorsat_gb300 import _native, autotune
from tensorsat_gb300.contractions.gpu import PRIMES_31, GpuContraction
from tensorsat_gb300.diagrams import Diagram
from tensorsat_gb300.lang.cuda_rel import CudaRel, leaf_array
from tensorsat_gb300.lib.sat import CNFInstance

pytestmark = pytest.mark.gpu

# (k, n, m, seed, target bits): instances whose trees fuse at least one step
CASES = [(3, 44, 187, 1, 22), (4, 30, 300, 1, 22), (5, 30, 630, 1, 22)]


@pytest.fixture
def lib():
    lib = _native.lib()
    yield lib
    lib.tsg_set_fusion(1)


RINGS = (_native.TSG_RING_MODP, _native.TSG_RING_U64, _native.TSG_RING_OR_AND)


def _fuse(c, on):
    """Asks for every fusion the structure allows (on) or clears the options (off)."""
    for r in RINGS:
        if on:
            autotune.fuse_all(c, r)
        else:
            autotune.set_options(c, r, None)


def _random_leaves(cnf, seed, density=0.99):
    """Random {0,1} leaves on the clause network's wiring, each entry 1 with probability
    ``density``: dense enough that hundreds of leaves still leave a large count."""
    d0 = cnf.clause_diagram()
    rng = np.random.default_rng(seed)
    arrays = [(rng.random(leaf_array(b).shape) < density).astype(np.uint8) for b in d0.blocks]
    return Diagram._new(d0.wiring, tuple(CudaRel(a) for a in arrays)), arrays


@pytest.mark.parametrize("k,n,m,seed,target", CASES)
def test_fused_equals_unfused_and_the_oracle(cuda, lib, k, n, m, seed, target):
    cnf = CNFInstance.random(k, n, m, rng=seed)
    d, arrays = _random_leaves(cnf, seed)
    c = GpuContraction(CudaRel, d.wiring, target_bits=target, trials=2, seed=0)
    npl = c.native_plan()
    primes = PRIMES_31[:3]
    ns = c.num_slices
    lib.tsg_set_fusion(1)
    _fuse(c, True)
    for ring, pr in ((_native.TSG_RING_MODP, primes), (_native.TSG_RING_U64, ())):
        fused = npl.fused_steps(ring, pr, 4, c.tree)
        assert fused, "no fused step"
        kinds = npl.describe(ring, pr, 4)
        for s, p in fused.items():
            assert kinds[s][0] == _native.TSG_KERNEL_FUSED
            assert kinds[p][0] == _native.TSG_KERNEL_NONE
    probe = [0, ns // 2 + 1, ns - 1]
    results = {}
    for on in (1, 0):
        _fuse(c, bool(on))
        results[on] = (
            c.count(d, ring="u64", group=4),
            c.count(d, ring="modp", num_primes=3, group=4),
            [c.count(d, ring="u64", group=1, slice_range=(s, s + 1)) for s in probe],
            [c.count(d, ring="modp", num_primes=2, group=1, slice_range=(s, s + 1))
             for s in probe],
        )
    assert results[1] == results[0]
    total_u64, total_modp, per_slice, per_slice_modp = results[1]
    assert total_u64 == total_modp > 0
    assert per_slice == per_slice_modp and all(x > 0 for x in per_slice)
    leaf_wires = [tuple(ws) for ws in d.wiring.slot_wires_list]
    for s, got in zip(probe[:2], per_slice[:2]):
        fixed = {w: (s >> j) & 1 for j, w in enumerate(c.sliced_wires)}
        want = orc.tree_contract(arrays, leaf_wires, (), c.tree.steps, "count", fixed=fixed)
        assert got == int(want), s


def test_fused_cnf_counts_equal_dpll(cuda, lib):
    """Exact model counts of satisfiable CNF networks whose trees fuse steps."""
    lib.tsg_set_fusion(1)
    for k, n, m, seed, target in [(3, 44, 187, 1, 22), (4, 30, 300, 1, 22), (3, 48, 204, 3, 22)]:
        cnf = CNFInstance.random(k, n, m, rng=seed)
        d = cnf.clause_diagram()
        c = GpuContraction(CudaRel, d.wiring, target_bits=target, trials=2, seed=0)
        _fuse(c, True)
        assert c.native_plan().fused_steps(_native.TSG_RING_MODP, PRIMES_31[:3], 16, c.tree)
        want = orc.dpll_count(n, cnf.clauses)[0]
        assert want > 0
        assert c.count(d, ring="modp", num_primes=3, group=16) == want
        assert c.count(d, ring="u64", group=16) == want
        assert bool(c.contract(d, group=16)) is True


def test_fused_or_and_bits_per_slice(cuda, lib):
    """The OR-AND ring fuses the same steps (packed words of 0/1 bytes): for every slice of
    a satisfiable instance, the fused SAT bit equals the unfused one and equals whether the
    slice's exact count is non-zero."""
    cnf = CNFInstance.random(3, 44, 187, rng=1)
    d = cnf.clause_diagram()
    c = GpuContraction(CudaRel, d.wiring, target_bits=22, trials=2, seed=0)
    lib.tsg_set_fusion(1)
    _fuse(c, True)
    assert c.native_plan().fused_steps(_native.TSG_RING_OR_AND, (), 1, c.tree)
    ns = c.num_slices
    counts = [c.count(d, ring="u64", group=1, slice_range=(s, s + 1)) for s in range(ns)]
    assert 0 < sum(1 for x in counts if x) < ns
    bits = {}
    for on in (1, 0):
        _fuse(c, bool(on))
        bits[on] = [bool(c.contract(d, group=1, slice_range=(s, s + 1))) for s in range(ns)]
    assert bits[1] == bits[0] == [x > 0 for x in counts]
