"""Leaf variants of one plan in one launch sequence (``tsg_plan_run_variants``): the
reference's assignment-search idiom (one wiring, one unit-input diagram per candidate,
``notebooks/02-random-ksat.ipynb`` cells 35-36) with the variant index as an extra batch
axis of every launch. Each variant's SAT bit and count equal its own contraction and the
oracle."""

from __future__ import annotations

import json
from pathlib import Path

import numpy as np
import pytest

from oracle import finrel_oracle as orc
from tensorsat_gb300.contractions.gpu import GpuContraction
from tensorsat_gb300.diagrams import Diagram
from tensorsat_gb300.lang.cuda_rel import CudaRel, leaf_array
from tensorsat_gb300.lib.sat import CNFInstance

pytestmark = pytest.mark.gpu
GOLDEN = Path(__file__).resolve().parent / "golden"


def test_assignment_search_trace_in_one_launch_sequence(cuda):
    kats = json.loads((GOLDEN / "notebook_kats.json").read_text())
    trace = kats["ksat4_n20_m195_rng1_assignment_search"]["trace"]
    cnf = CNFInstance.random(4, 20, 195, rng=1)
    d = cnf.diagram()
    c = GpuContraction(CudaRel, cnf.contraction_wiring())
    diagrams = [(cnf.inputs(cand) >> d).flatten() for cand, _ in trace]
    bits = [bool(b) for b in c.contract_variants(diagrams)]
    assert [[cand, b] for (cand, _), b in zip(trace, bits)] == trace


def test_sliced_variants_count_like_single_runs(cuda):
    """Random leaf variants on a sliced plan (5 variants, padded to 8 inside): counts and
    bits equal one contraction per variant, and the oracle on one of them."""
    cnf = CNFInstance.random(3, 20, 85, rng=2)
    d0 = cnf.clause_diagram()
    c = GpuContraction(CudaRel, d0.wiring, target_bits=8, trials=1)
    assert c.num_slices >= 4
    rng = np.random.default_rng(11)
    variants, arrays = [], []
    for _ in range(5):
        arrs = [(rng.random(leaf_array(b).shape) < 0.9).astype(np.uint8) for b in d0.blocks]
        variants.append(Diagram._new(d0.wiring, tuple(CudaRel(a) for a in arrs)))
        arrays.append(arrs)
    counts = c.count_variants(variants, num_primes=2, group=2)
    single = [c.count(v, ring="modp", num_primes=2, group=2) for v in variants]
    assert counts == single and any(x > 0 for x in counts)
    bits = [bool(b) for b in c.contract_variants(variants, group=2)]
    assert bits == [x > 0 for x in counts]
    leaf_wires = [tuple(ws) for ws in d0.wiring.slot_wires_list]
    want = orc.tree_contract(arrays[3], leaf_wires, (), c.tree.steps, "count")
    assert counts[3] == int(want)
