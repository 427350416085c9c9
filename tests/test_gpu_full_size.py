"""Parity at the benchmark's full size: uniform random 3-SAT n=60, m=256 (seed 0), the tree
the benchmark runs (intermediates capped at 2^26 entries, thousands of slices).

Brute force is out of reach at n=60. The whole-instance count is pinned by the oracle's
exact DPLL model counter (itself checked against brute force), and by size-independent
properties:
* the count modulo 2^64 (exact, since the count is below 2^60) equals the 3-prime CRT
  count;
* two half ranges of slices add up to the whole count;
* the SAT bit equals count > 0.
Single slices at both ends of the range are compared exactly with the CPU oracle's
contraction of the same slice along the same tree, which pins the kernels on the
2^26-entry intermediates themselves. Integers throughout: the tolerance is equality.
"""

from __future__ import annotations

import numpy as np
import pytest

from oracle import finrel_oracle as orc
from tensorsat_gb300 import _native
from tensorsat_gb300.contractions.gpu import GpuContraction
from tensorsat_gb300.lang.cuda_rel import CudaRel
from tensorsat_gb300.lib.sat import CNFInstance

pytestmark = pytest.mark.gpu

N, M = 60, 256


@pytest.fixture(scope="module")
def n60(cuda):
    cnf = CNFInstance.random(3, N, M, rng=0)
    d = cnf.clause_diagram()
    c = GpuContraction(CudaRel, d.wiring, target_bits=26, trials=8, seed=0)
    assert c.stats()["peak_bits"] == 26 and c.num_slices >= 4096
    return cnf, d, c


def test_n60_full_count_properties(n60):
    cnf, d, c = n60
    total_u64 = c.count(d, ring="u64")
    total_crt = c.count(d, ring="modp", num_primes=3)
    assert total_u64 == total_crt
    assert total_crt == orc.dpll_count(N, cnf.clauses)[0]
    half = c.num_slices // 2
    lo = c.count(d, ring="modp", num_primes=3, slice_range=(0, half))
    hi = c.count(d, ring="modp", num_primes=3, slice_range=(half, c.num_slices))
    assert lo + hi == total_crt
    assert bool(c.contract(d)) == (total_crt > 0)


@pytest.mark.parametrize("end", ["first", "last"])
def test_n60_single_slice_matches_oracle(n60, end):
    cnf, d, c = n60
    sid = 0 if end == "first" else c.num_slices - 1
    r = c.run(d, _native.TSG_RING_U64, slice_range=(sid, sid + 1), group=1)
    got = int(r.cpu().numpy().view(np.uint64)[0]) * c.discard_factor
    fixed = {w: (sid >> j) & 1 for j, w in enumerate(c.sliced_wires)}
    assert got == orc.cnf_count_by_tree(N, cnf.clauses, c.tree.steps, fixed=fixed)
    bit = c.run(d, _native.TSG_RING_OR_AND, slice_range=(sid, sid + 1), group=1)
    assert int(bit.cpu().numpy()[0]) == int(orc.cnf_count_by_tree(N, cnf.clauses, c.tree.steps,
                                                                   "or_and", fixed=fixed))


def test_n60_satisfiable_instance_slice_ranges_match_dpll(cuda):
    """The seed-0 instance above has no models, so its root counts are all zero. Seed 8
    (558 models) gives non-zero counts at the same size: each slice's exact count is the
    DPLL count with the slice's sliced variables fixed by unit clauses (their sum is the
    whole instance's count), and the GPU's counts and SAT bits over slice ranges of 512
    must equal those sums."""
    cnf = CNFInstance.random(3, N, M, rng=8)
    d = cnf.clause_diagram()
    c = GpuContraction(CudaRel, d.wiring, target_bits=26, trials=4, seed=0)
    assert c.stats()["peak_bits"] == 26 and c.num_slices >= 4096
    per_slice = []
    for sid in range(c.num_slices):
        units = [((w + 1) if (sid >> j) & 1 else -(w + 1),)
                 for j, w in enumerate(c.sliced_wires)]
        per_slice.append(orc.dpll_count(N, list(cnf.clauses) + units)[0])
    total = orc.dpll_count(N, cnf.clauses)[0]
    assert sum(per_slice) == total > 0
    width = 512
    sums = [sum(per_slice[a:a + width]) for a in range(0, c.num_slices, width)]
    busiest = max(range(len(sums)), key=lambda i: sums[i])
    empty = sums.index(0)
    for i in (busiest, empty):
        rng = (i * width, (i + 1) * width)
        assert c.count(d, ring="modp", num_primes=3, slice_range=rng, group=32) == sums[i]
        assert c.count(d, ring="u64", slice_range=rng, group=32) == sums[i]
        assert bool(c.contract(d, slice_range=rng, group=32)) == (sums[i] > 0)
