"""Generates the golden fixtures of tests/golden from the upstream tensorsat sources.

Run in a container that holds the upstream checkout, named by ``TENSORSAT_REFERENCE``
(the example files it reads lie outside the installed package):

    TENSORSAT_REFERENCE=/root/reference python tests/golden/make_golden.py

Everything here is computed by the upstream code itself, imported through
``_ref_import`` (no upstream file is modified or copied):

* ``kissat.json``: the 41 active known-answer tests of ``examples/test_sat_solver.py``:
  expected bit (parsed from the test file), clauses from the upstream DIMACS parser, the
  SAT bit computed by upstream ``FinRel._contract2`` along a contraction tree, and the
  model count (brute force for n <= 30, else the exact-integer tree contraction).
* ``dimacs.json``: the 6 parser tests of ``examples/test_dimacs_parser.py`` (DIMACS text
  and the clauses the upstream parser returns).
* ``random_instances.json``: ``CNFInstance.random`` clauses for the benchmark configs'
  generators (numpy Generator streams pin the instance identity).
* ``wirings.json``: flattened wirings (slot wires, out wires, box names) of upstream
  diagrams: ``inputs(spec) >> diagram()`` and ``contraction_wiring()``.
* ``contract2.npz`` + ``contract2.json``: random ``FinRel._contract2`` and
  ``FinRel._rewire`` cases (repeated / discarded / permuted wires, dims 1-3).
* ``notebook_kats.json``: answers of the upstream notebooks' executable examples,
  recomputed by upstream code (CNOT and a&(b|c) by contract2, the 4-SAT solution set, the
  4-SAT SAT bit, the assignment-search trace, the #SAT example count).
"""

from __future__ import annotations

import json
import os
import re
import sys
import time
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
REPO = HERE.parent.parent
sys.path.insert(0, str(HERE))
sys.path.insert(0, str(REPO))

import _ref_import  # noqa: E402

_ref_import.install()

from tensorsat.lang.fin_rel import FinRel  # noqa: E402
from tensorsat.lib import bincirc as ref_bincirc  # noqa: E402
from tensorsat.lib.sat import CNFInstance  # noqa: E402

from oracle import finrel_oracle as orc  # noqa: E402
from tensorsat_gb300 import planner  # noqa: E402

REF = Path(_ref_import.REFERENCE_ROOT)


def ref_tree_contract(diagram, out_wires=(), seed=0):
    """Contracts a flat upstream diagram with upstream FinRel._contract2, one call per
    node of a tree from tensorsat_gb300.planner (cotengra-style wire bookkeeping)."""
    w = diagram.wiring
    leaf_wires = [tuple(ws) for ws in w.slot_wires_list]
    net = planner.Network(leaf_wires, {i: t.size for i, t in enumerate(w.wire_types)},
                          tuple(w.out_wires))
    tree, _ = planner.optimize(net, target_bits=None, trials=2, seed=seed)
    boxes = list(diagram.boxes)
    nodes = {i: (b, tuple(ws)) for i, (b, ws) in enumerate(zip(boxes, leaf_wires))}
    from collections import Counter
    holders = Counter(x for ws in leaf_wires for x in set(ws))
    outs = list(dict.fromkeys(w.out_wires))
    L = len(boxes)
    for s, (a, b) in enumerate(tree.steps):
        (ba, wa), (bb, wb) = nodes.pop(a), nodes.pop(b)
        for x in set(wa):
            holders[x] -= 1
        for x in set(wb):
            holders[x] -= 1
        keep = [x for x in dict.fromkeys(wa + wb) if holders[x] > 0 or x in outs]
        res = FinRel._contract2(ba, wa, bb, wb, keep)
        for x in keep:
            holders[x] += 1
        nodes[L + s] = (res, tuple(keep))
    (res, rw), = nodes.values()
    if outs:
        res = res._rewire([rw.index(x) for x in w.out_wires])
    return res, tree


def kissat_tests():
    text = (REF / "examples" / "test_sat_solver.py").read_text()
    cases = []
    pat = re.compile(
        r"^def (test_\w+)\(\) -> None:\n\s+is_sat: bool = check_sat_file\(\"(\w+)\"\)\n"
        r"\s+assert\((not )?is_sat\)", re.M)
    for m in pat.finditer(text):
        cases.append((m.group(1), m.group(2), m.group(3) is None))
    return cases


def make_kissat():
    out = []
    for test, fname, expected in kissat_tests():
        dimacs = (REF / "examples" / "kissat" / "cnf" / f"{fname}.cnf").read_text()
        cnf = CNFInstance.from_dimacs(dimacs)
        t0 = time.time()
        d = (cnf.inputs(None) >> cnf.diagram()).flatten()
        res, tree = ref_tree_contract(d)
        sat = bool(res)
        n = cnf.num_vars
        if n <= 30:
            count = orc.brute_force_count(n, cnf.clauses)
        else:
            count = orc.cnf_count_by_tree(n, cnf.clauses, _clause_tree(cnf).steps)
        assert (count > 0) == sat, (fname, count, sat)
        out.append({"test": test, "file": fname, "expected": expected, "num_vars": n,
                    "clauses": [list(c) for c in cnf.clauses], "sat_reference": sat,
                    "count": str(count), "count_pinned_by": "brute force" if n <= 30 else
                    "exact tree contraction"})
        print(f"kissat {fname}: n={n} sat={sat} count={count} ({time.time()-t0:.1f}s)",
              flush=True)
    return out


def _clause_tree(cnf):
    wires = [tuple(dict.fromkeys(abs(l) - 1 for l in c)) for c in cnf.clauses]
    net = planner.Network(wires, {w: 2 for w in range(cnf.num_vars)}, ())
    tree, _ = planner.optimize(net, target_bits=None, trials=2)
    return tree


def make_dimacs():
    text = (REF / "examples" / "test_dimacs_parser.py").read_text()
    files = re.findall(r'open\("examples/kissat/cnf/(\w+)\.cnf"\)', text)
    out = []
    for f in files:
        dimacs = (REF / "examples" / "kissat" / "cnf" / f"{f}.cnf").read_text()
        cnf = CNFInstance.from_dimacs(dimacs)
        out.append({"file": f, "dimacs": dimacs, "num_vars": cnf.num_vars,
                    "clauses": [list(c) for c in cnf.clauses]})
    return out


def make_random():
    out = []
    for k, n, m, seeds in [(3, 20, 85, range(8)), (3, 60, 256, range(4)), (4, 10, 95, [0]),
                           (4, 20, 195, [1]), (3, 30, 128, [0]), (5, 100, 2100, [0])]:
        for s in seeds:
            cnf = CNFInstance.random(k, n, m, rng=s)
            out.append({"k": k, "n": n, "m": m, "rng": s,
                        "clauses": [list(c) for c in cnf.clauses]})
    # ragged batch scheme: per-instance Generator seeded by the instance index
    for i in range(4):
        g = np.random.default_rng(i)
        n = int(g.integers(30, 81))
        m = round(float(g.uniform(3.5, 5.0)) * n)
        cnf = CNFInstance.random(3, n, m, rng=g)
        out.append({"k": 3, "n": n, "m": m, "ragged_index": i,
                    "clauses": [list(c) for c in cnf.clauses]})
    return out


def _wiring_json(d):
    w = d.wiring
    return {"slot_wires_list": [list(x) for x in w.slot_wires_list],
            "out_wires": list(w.out_wires), "num_wires": w.num_wires,
            "boxes": [b.name for b in d.boxes]}


def make_wirings():
    out = []
    cnf = CNFInstance.random(3, 20, 85, rng=0)
    out.append({"k": 3, "n": 20, "m": 85, "rng": 0, "inputs": None,
                **_wiring_json((cnf.inputs(None) >> cnf.diagram()).flatten())})
    small = CNFInstance.random(3, 6, 10, rng=1)
    for spec in ["01?10?", 5, None]:
        out.append({"k": 3, "n": 6, "m": 10, "rng": 1, "inputs": spec,
                    **_wiring_json((small.inputs(spec) >> small.diagram()).flatten())})
    out.append({"k": 3, "n": 6, "m": 10, "rng": 1, "inputs": "discard_unk",
                **_wiring_json((small.inputs(None, discard_unk=True) >> small.diagram()).flatten())})
    w = small.contraction_wiring()
    out.append({"k": 3, "n": 6, "m": 10, "rng": 1, "inputs": "contraction_wiring",
                "slot_wires_list": [list(x) for x in w.slot_wires_list],
                "out_wires": list(w.out_wires), "num_wires": w.num_wires, "boxes": None})
    k4 = CNFInstance.random(4, 5, 12, rng=3)
    out.append({"k": 4, "n": 5, "m": 12, "rng": 3, "inputs": "diagram",
                **_wiring_json(k4.diagram())})
    return out


def make_contract2(rng):
    arrays = {}
    cases = []
    for i in range(160):
        nw = int(rng.integers(1, 7))
        dims = {w: int(rng.integers(1, 4)) if rng.random() < 0.3 else 2 for w in range(nw)}
        lr = int(rng.integers(0, 5))
        rr = int(rng.integers(0, 5))
        lw = [int(x) for x in rng.integers(0, nw, size=lr)]
        rw = [int(x) for x in rng.integers(0, nw, size=rr)]
        present = sorted(set(lw) | set(rw))
        if present:
            k = int(rng.integers(0, len(present) + 2))
            ow = [int(x) for x in rng.choice(present, size=k, replace=True)]
        else:
            ow = []
        lhs = (rng.random([dims[w] for w in lw]) < 0.5).astype(np.uint8)
        rhs = (rng.random([dims[w] for w in rw]) < 0.5).astype(np.uint8)
        try:
            res = FinRel._contract2(FinRel._new(lhs), lw, FinRel._new(rhs), rw, ow).tensor
        except ValueError:
            # upstream rewire_array cannot broadcast when repeated output wires are
            # interleaved with others out of order; such cases have no upstream answer
            continue
        mine = orc.contract2_or_and(lhs, lw, rhs, rw, ow)
        assert np.array_equal(np.asarray(res), mine), i
        arrays[f"c{i}_lhs"] = lhs
        arrays[f"c{i}_rhs"] = rhs
        arrays[f"c{i}_out"] = np.asarray(res)
        cases.append({"id": i, "kind": "contract2", "lhs_wires": lw, "rhs_wires": rw,
                      "out_wires": ow})
    for i in range(160, 220):
        r = int(rng.integers(0, 5))
        shape = [int(rng.integers(1, 4)) for _ in range(r)]
        t = (rng.random(shape) < 0.5).astype(np.uint8)
        k = int(rng.integers(0, r + 2)) if r else 0
        ports = [int(x) for x in rng.integers(0, r, size=k)] if r else []
        try:
            res = FinRel._new(t)._rewire(ports).tensor
        except ValueError:
            continue
        assert np.array_equal(np.asarray(res), orc.rewire_or_and(t, ports)), i
        arrays[f"c{i}_in"] = t
        arrays[f"c{i}_out"] = np.asarray(res)
        cases.append({"id": i, "kind": "rewire", "out_ports": ports})
    return arrays, cases


def make_notebook_kats():
    bit = ref_bincirc.bit
    kats = {}
    cnot = FinRel.contract2(FinRel.spider(bit, 3), [0, 2, 4], ref_bincirc.xor_, [4, 1, 3],
                            [0, 1, 2, 3])
    assert cnot == FinRel.from_callable((2, 2), (2, 2), lambda a, b: (a, a ^ b))
    kats["cnot"] = sorted(map(list, cnot.to_set()))
    func = FinRel.contract2(ref_bincirc.or_, [1, 2, 3], ref_bincirc.and_, [0, 3, 4])
    kats["a_and_b_or_c"] = sorted(map(list, func.to_set()))
    _f = FinRel.contract2(ref_bincirc.or_, [0, 2, 3], ref_bincirc.or_, [1, 2, 4],
                          out_wires=[0, 1, 2, 3, 4])
    f2 = FinRel.contract2(_f, [0, 1, 2, 3, 4], ref_bincirc.and_, [3, 4, 5])
    kats["a_or_c_and_b_or_c"] = sorted(map(list, f2.to_set()))
    cnf = CNFInstance.random(4, 10, 95, rng=0)
    res, _ = ref_tree_contract(cnf.diagram())
    kats["ksat4_n10_m95_rng0_solutions"] = sorted(map(list, res.to_set()))
    cnf20 = CNFInstance.random(4, 20, 195, rng=1)
    d20 = cnf20.diagram()
    sat, _ = ref_tree_contract((cnf20.inputs(None) >> d20).flatten())
    kats["ksat4_n20_m195_rng1_sat"] = bool(sat)
    trace = []
    n = cnf20.num_vars
    assignment = ""
    for i in range(n):
        found = None
        for b in "01":
            cand = assignment[:i] + b + "?" * (n - i - 1)
            ok, _ = ref_tree_contract((cnf20.inputs(cand) >> d20).flatten())
            trace.append([cand, bool(ok)])
            if ok:
                found = b
                break
        if not found:
            assignment = ""
            break
        assignment += found
    kats["ksat4_n20_m195_rng1_assignment_search"] = {"trace": trace, "assignment": assignment}
    # ((a|b)|c) & ((~c|~b)|~a): the #SAT prototype's formula
    clauses = [(1, 2, 3), (-3, -2, -1)]
    small = CNFInstance._new(3, tuple(clauses))
    ok, _ = ref_tree_contract((small.inputs(None) >> small.diagram()).flatten())
    kats["sharp_sat_example"] = {"clauses": [list(c) for c in clauses],
                                 "count": orc.brute_force_count(3, clauses), "sat": bool(ok)}
    return kats


def main() -> None:
    rng = np.random.default_rng(20250213)
    (HERE / "kissat.json").write_text(json.dumps(make_kissat(), indent=0))
    (HERE / "dimacs.json").write_text(json.dumps(make_dimacs(), indent=1))
    (HERE / "random_instances.json").write_text(json.dumps(make_random()))
    (HERE / "wirings.json").write_text(json.dumps(make_wirings()))
    arrays, cases = make_contract2(rng)
    np.savez_compressed(HERE / "contract2.npz", **arrays)
    (HERE / "contract2.json").write_text(json.dumps(cases))
    (HERE / "notebook_kats.json").write_text(json.dumps(make_notebook_kats(), indent=1))
    print("golden fixtures written to", HERE)


if __name__ == "__main__":
    os.chdir(REPO)
    main()
