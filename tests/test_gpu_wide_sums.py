"""Tile-kernel steps that sum 5 or 6 wires (32 or 64 summed combinations, kept in the
kernel's offset tables). Count-ring sums with a leaf factor are reduced every 16 terms,
pairs of Montgomery products every 2. Checked on CNF networks (mod 3 primes with CRT,
mod 2^64 and the SAT bit against the oracle's DPLL count) and on random dense {0,1} leaves
of the same wiring (every intermediate residue is a full Montgomery residue, so the
reductions of 32-term sums with a leaf factor are exercised; mod 2^64 and mod 3 primes
against the oracle's exact contraction along the same tree). Integers: equality."""

from __future__ import annotations

import numpy as np
import pytest

from oracle import finrel_oracle as orc
from tensorsat_gb300 import _native
from tensorsat_gb300.contractions.gpu import PRIMES_31, GpuContraction
from tensorsat_gb300.diagrams import Diagram
from tensorsat_gb300.lang.cuda_rel import CudaRel, leaf_array
from tensorsat_gb300.lib.sat import CNFInstance

pytestmark = pytest.mark.gpu

# (k, n, m, seed): each tree has a step summing 5 wires on the tile kernel; the 5-SAT ones
# with a clause leaf as an operand of that step
CASES = [(5, 24, 400, 1), (5, 22, 300, 2), (3, 34, 140, 5), (4, 26, 250, 1)]


def _wide_tile_steps(c):
    t = c.tree
    L = t.num_leaves
    sl = set(c.sliced_wires)
    kinds = c.native_plan().describe(_native.TSG_RING_MODP, PRIMES_31[:3], 1)
    out = []
    for s, (a, b) in enumerate(t.steps):
        k = len(t.step_union(s) - t.node_wires[L + s] - sl)
        if k >= 5 and int(kinds[s][0]) == _native.TSG_KERNEL_TILE:
            out.append((s, k, a < L or b < L))
    return out


@pytest.mark.parametrize("k,n,m,seed", CASES)
def test_wide_sums_on_cnf_networks(cuda, k, n, m, seed):
    cnf = CNFInstance.random(k, n, m, rng=seed)
    d = cnf.clause_diagram()
    c = GpuContraction(CudaRel, d.wiring, target_bits=26, trials=1, seed=0)
    assert _wide_tile_steps(c)
    want = orc.dpll_count(n, cnf.clauses)[0]
    assert c.count(d, ring="modp", num_primes=3) == want
    assert c.count(d, ring="u64") == want % (1 << 64)
    assert bool(c.contract(d)) == (want > 0)


@pytest.mark.parametrize("k,n,m,seed", CASES[:2])
def test_wide_sums_with_leaf_factors_on_dense_leaves(cuda, k, n, m, seed):
    cnf = CNFInstance.random(k, n, m, rng=seed)
    d0 = cnf.clause_diagram()
    rng = np.random.default_rng(seed)
    arrays = [(rng.random(leaf_array(b).shape) < 0.995).astype(np.uint8) for b in d0.blocks]
    d = Diagram._new(d0.wiring, tuple(CudaRel(a) for a in arrays))
    c = GpuContraction(CudaRel, d.wiring, target_bits=26, trials=1, seed=0)
    wide = _wide_tile_steps(c)
    assert any(leaf for _, _, leaf in wide)
    leaf_wires = [tuple(ws) for ws in d.wiring.slot_wires_list]
    want = int(orc.tree_contract(arrays, leaf_wires, (), c.tree.steps, "count"))
    assert want > 1 << 16
    assert c.count(d, ring="modp", num_primes=3) == want % (PRIMES_31[0] * PRIMES_31[1] * PRIMES_31[2])
    assert c.count(d, ring="u64") == want % (1 << 64)
