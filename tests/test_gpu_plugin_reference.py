"""The reference-side binding on the GPU: upstream tensorsat code drives ``FinRelCuda``.

``tensorsat_gb300.plugin.make_finrel_cuda`` defines the box class a tensorsat maintainer
would add next to ``FinRel`` (``tensorsat/lang/fin_rel.py:162``). Here the unmodified
upstream package (``TENSORSAT_REFERENCE``, else the ``baseline/_ref`` install) calls it:

* every ``FinRel._contract2`` / ``FinRel._rewire`` golden vector goes through
  ``FinRelCuda._contract2`` / ``_rewire`` and is compared bit for bit with upstream
  ``FinRel`` on the same inputs (``tensorsat/lang/fin_rel.py:255-288,379-393``);
* ``_union``, ``_spider``, ``_scalar`` and ``_as_scalar`` against upstream ``FinRel``;
* the known-answer SAT cases of ``examples/test_sat_solver.py`` (golden ``kissat.json``):
  the upstream bintree diagrams, with their ``FinRel`` boxes moved to ``FinRelCuda``, are
  contracted by upstream ``SimpleContraction(FinRelCuda, wiring, path)``
  (``tensorsat/contractions/simple.py:251-292``) where its keep-every-wire bookkeeping
  stays small, and along a planned tree through the public ``Box.contract2``
  (``tensorsat/diagrams.py:811-866``) for every case; the bits equal upstream ``FinRel``
  on the same calls and the known answers.
"""

from __future__ import annotations

import json
import sys
from pathlib import Path

import numpy as np
import pytest

from tensorsat_gb300 import planner

pytestmark = pytest.mark.gpu
GOLDEN = Path(__file__).resolve().parent / "golden"


@pytest.fixture(scope="module")
def upstream():
    sys.path.insert(0, str(GOLDEN))
    import _ref_import

    if not _ref_import.available():
        pytest.skip("upstream tensorsat sources not found; tried "
                    + ", ".join(_ref_import.candidate_roots()))
    _ref_import.install()
    import tensorsat
    import tensorsat.contractions.simple
    import tensorsat.diagrams
    import tensorsat.lang.fin_rel
    import tensorsat.lib.sat

    return tensorsat


@pytest.fixture(scope="module")
def finrel_cuda(upstream, cuda):
    from tensorsat_gb300.plugin import make_finrel_cuda

    return make_finrel_cuda(upstream)


def _cases(kind):
    cases = json.loads((GOLDEN / "contract2.json").read_text())
    arrays = np.load(GOLDEN / "contract2.npz")
    return [c for c in cases if c["kind"] == kind], arrays


def _einsum_reference(a, aw, b, bw, ow):
    from oracle import finrel_oracle as orc

    return orc.contract2_einsum_definition(a, aw, b, bw, ow)


def test_contract2_vectors_through_finrel_cuda(upstream, finrel_cuda):
    FinRel = upstream.lang.fin_rel.FinRel
    cases, arrays = _cases("contract2")
    same = divergent = 0
    for c in cases:
        i = c["id"]
        a, b = arrays[f"c{i}_lhs"], arrays[f"c{i}_rhs"]
        lw, rw, ow = c["lhs_wires"], c["rhs_wires"], c["out_wires"]
        up = FinRel._contract2(FinRel._new(a.copy()), lw, FinRel._new(b.copy()), rw, ow).tensor
        got = finrel_cuda._contract2(finrel_cuda.from_array(a), lw,
                                     finrel_cuda.from_array(b), rw, ow)
        got = got.to_finrel().tensor
        np.testing.assert_array_equal(up, arrays[f"c{i}_out"], err_msg=str(c))
        exact = _einsum_reference(a, lw, b, rw, ow)
        if np.array_equal(up, exact):
            np.testing.assert_array_equal(got, up, err_msg=str(c))
            same += 1
        else:
            # upstream rewire_array transposes interleaved repeated wires; the kernel
            # follows the einsum definition (documented divergence)
            np.testing.assert_array_equal(got, exact, err_msg=str(c))
            divergent += 1
    assert same > 100 and divergent <= 10


def test_rewire_vectors_through_finrel_cuda(upstream, finrel_cuda):
    FinRel = upstream.lang.fin_rel.FinRel
    cases, arrays = _cases("rewire")
    n = 0
    for c in cases:
        i = c["id"]
        t = arrays[f"c{i}_in"]
        up = FinRel._new(t.copy())._rewire(c["out_ports"]).tensor
        got = finrel_cuda.from_array(t)._rewire(c["out_ports"]).to_finrel().tensor
        exact = _einsum_reference(t, list(range(t.ndim)), np.ones((), np.uint8), [],
                                  c["out_ports"])
        np.testing.assert_array_equal(got, up if np.array_equal(up, exact) else exact,
                                      err_msg=str(c))
        n += 1
    assert n > 30


def test_union_spider_scalar_against_finrel(upstream, finrel_cuda):
    FinRel = upstream.lang.fin_rel.FinRel
    FinSet = upstream.lang.fin_rel.FinSet
    rng = np.random.default_rng(3)
    for shape in [(), (2,), (2, 3), (3, 1, 2), (2, 2, 2, 2)]:
        a = rng.integers(0, 2, size=shape).astype(np.uint8)
        b = rng.integers(0, 2, size=shape).astype(np.uint8)
        up = (FinRel._new(a.copy()) + FinRel._new(b.copy())).tensor
        got = (finrel_cuda.from_array(a) + finrel_cuda.from_array(b)).to_finrel()
        np.testing.assert_array_equal(got.tensor, up)
    for dim, ports in [(1, 1), (2, 1), (2, 3), (3, 2), (4, 4)]:
        up = FinRel._spider(FinSet(dim), ports).tensor
        got = finrel_cuda._spider(FinSet(dim), ports).to_finrel().tensor
        np.testing.assert_array_equal(got, up)
    for v in (False, True):
        assert bool(finrel_cuda._scalar(v)) == bool(FinRel._scalar(v)) == v


def _upstream_network(upstream, clauses, num_vars):
    """The upstream SAT network of a clause list, built through the upstream DIMACS
    parser (``CNFInstance`` itself is not a final class upstream)."""
    sat = upstream.lib.sat
    lines = [f"p cnf {num_vars} {len(clauses)}"]
    lines += [" ".join(str(l) for l in c) + " 0" for c in clauses]
    cnf = sat.CNFInstance.from_dimacs("\n".join(lines))
    return (cnf.inputs(None) >> cnf.diagram()).flatten()


def _to_cuda(upstream, finrel_cuda, diagram):
    Diagram = upstream.diagrams.Diagram
    blocks = {i: finrel_cuda.from_finrel(b) for i, b in enumerate(diagram.blocks)}
    return Diagram(diagram.wiring, blocks)


def _tree_bit(box_class, boxes, slot_wires, out_wires, steps):
    """SAT bit along a tree through the public Box.contract2, with cotengra's
    bookkeeping: a wire is summed once no remaining tensor and no output needs it."""
    from collections import Counter

    nodes = {i: (b, tuple(ws)) for i, (b, ws) in enumerate(zip(boxes, slot_wires))}
    holders = Counter(w for _, ws in nodes.values() for w in set(ws))
    L = len(boxes)
    for s, (x, y) in enumerate(steps):
        (a, aw), (b, bw) = nodes.pop(x), nodes.pop(y)
        for w in set(aw) | set(bw):
            holders[w] -= (w in aw) + (w in bw)
        keep = tuple(w for w in dict.fromkeys(aw + bw) if holders[w] > 0 or w in out_wires)
        res = box_class.contract2(a, aw, b, bw, keep)
        for w in keep:
            holders[w] += 1
        nodes[L + s] = (res, keep)
    (res, _), = nodes.values()
    return bool(res)


def test_kissat_cases_through_upstream_drivers(upstream, finrel_cuda):
    FinRel = upstream.lang.fin_rel.FinRel
    SimpleContraction = upstream.contractions.simple.SimpleContraction
    cases = json.loads((GOLDEN / "kissat.json").read_text())
    simple = 0
    for case in cases:
        clauses = case["clauses"]
        n = max(abs(l) for c in clauses for l in c)
        d = _upstream_network(upstream, clauses, n)
        dc = _to_cuda(upstream, finrel_cuda, d)
        w = d.wiring
        expected = bool(case["expected"])
        # upstream SimpleContraction keeps every wire of a subtree until the root: only
        # networks with few wires stay small under it
        if w.num_wires <= 22 and w.num_slots >= 2:
            path = [(0, 1)] * (w.num_slots - 1)
            got = SimpleContraction(finrel_cuda, w, path).contract(dc)
            up = SimpleContraction(FinRel, w, path).contract(d)
            assert bool(got) == bool(up) == expected, case
            simple += 1
        net = planner.Network([tuple(ws) for ws in w.slot_wires_list],
                              {x: 2 for x in range(w.num_wires)}, tuple(w.out_wires))
        tree, _ = planner.optimize(net, target_bits=None, trials=1, seed=0)
        got = _tree_bit(finrel_cuda, list(dc.blocks), w.slot_wires_list, w.out_wires,
                        tree.steps)
        up = _tree_bit(FinRel, list(d.blocks), w.slot_wires_list, w.out_wires, tree.steps)
        assert got == up == expected, case
    assert simple >= 10
