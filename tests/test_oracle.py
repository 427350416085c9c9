"""The oracle is pinned before it is trusted: against the reference's own outputs
(per-step vectors, known-answer SAT tests, notebook examples) and brute force."""

from __future__ import annotations

import json
from pathlib import Path

import numpy as np
import pytest

from oracle import finrel_oracle as orc
from tensorsat_gb300 import planner
from tensorsat_gb300.lib.sat import CNFInstance

GOLDEN = Path(__file__).resolve().parent / "golden"


def _json(name):
    return json.loads((GOLDEN / name).read_text())


def test_oracle_contract2_and_rewire_match_reference_vectors():
    cases = _json("contract2.json")
    arrays = np.load(GOLDEN / "contract2.npz")
    for c in cases:
        i = c["id"]
        if c["kind"] == "contract2":
            got = orc.contract2_or_and(arrays[f"c{i}_lhs"], c["lhs_wires"], arrays[f"c{i}_rhs"],
                                       c["rhs_wires"], c["out_wires"])
        else:
            got = orc.rewire_or_and(arrays[f"c{i}_in"], c["out_ports"])
        np.testing.assert_array_equal(got, arrays[f"c{i}_out"], err_msg=str(c))


def _clause_tree(num_vars, clauses, seed=0):
    wires = [tuple(dict.fromkeys(abs(l) - 1 for l in c)) for c in clauses]
    net = planner.Network(wires, {w: 2 for w in range(num_vars)}, ())
    tree, _ = planner.optimize(net, target_bits=None, trials=1, seed=seed)
    return tree


@pytest.mark.parametrize("case", _json("kissat.json"), ids=lambda c: c["test"])
def test_oracle_kissat_known_answers(case):
    n, clauses = case["num_vars"], [tuple(c) for c in case["clauses"]]
    tree = _clause_tree(n, clauses)
    sat = orc.cnf_count_by_tree(n, clauses, tree.steps, "or_and")
    assert bool(sat) == case["expected"] == case["sat_reference"]
    count = orc.cnf_count_by_tree(n, clauses, tree.steps)
    assert count == int(case["count"])
    if n <= 30:
        assert orc.brute_force_count(n, clauses) == count


def test_brute_force_counts_random_3sat_n20():
    counts = [orc.brute_force_count(20, CNFInstance.random(3, 20, 85, rng=s).clauses)
              for s in range(8)]
    assert counts == [0, 0, 4, 2, 0, 3, 8, 4]


def test_brute_force_edge_cases():
    assert orc.brute_force_count(0, []) == 1
    assert orc.brute_force_count(3, []) == 8
    assert orc.brute_force_count(1, [(1,), (-1,)]) == 0
    assert orc.brute_force_count(7, [(1, -1)]) == 128
    assert orc.brute_force_count(8, [(8,)]) == 128


def test_dpll_counter_matches_brute_force():
    cases = [(3, n, round(r * n), s) for n in (10, 14, 18, 22) for r in (1.5, 3.0, 4.3)
             for s in range(3)]
    cases += [(5, n, round(r * n), s) for n in (8, 14, 20, 24) for r in (5.0, 12.0, 21.0)
              for s in range(2)]
    cases += [(4, 16, 100, 0), (2, 20, 15, 1), (7, 22, 300, 0)]
    for k, n, m, s in cases:
        cnf = CNFInstance.random(k, n, m, rng=s)
        assert orc.dpll_count(n, cnf.clauses)[0] == orc.brute_force_count(n, cnf.clauses), \
            (k, n, m, s)


def test_dpll_counter_edge_cases():
    assert orc.dpll_count(0, [])[0] == 1
    assert orc.dpll_count(3, [])[0] == 8
    assert orc.dpll_count(100, [])[0] == 2**100  # beyond 64 bits
    with pytest.raises(RuntimeError):
        orc.dpll_count(128, [])
    assert orc.dpll_count(1, [(1,), (-1,)])[0] == 0
    assert orc.dpll_count(7, [(1, -1)])[0] == 128  # tautology
    assert orc.dpll_count(8, [(8,)])[0] == 128
    assert orc.dpll_count(4, [(2, 2, -3)])[0] == orc.brute_force_count(4, [(2, 2, -3)])
    assert orc.dpll_count(4, [()])[0] == 0  # the empty clause
    with pytest.raises(ValueError):
        orc.dpll_count(3, [(4,)])
    with pytest.raises(RuntimeError):
        orc.dpll_count(40, CNFInstance.random(3, 40, 60, rng=0).clauses, node_limit=3)


@pytest.mark.parametrize("case", _json("kissat.json"), ids=lambda c: c["test"])
def test_dpll_counter_kissat_known_answers(case):
    n, clauses = case["num_vars"], [tuple(c) for c in case["clauses"]]
    count = orc.dpll_count(n, clauses)[0]
    assert count == int(case["count"])
    assert (count > 0) == case["expected"]


def test_oracle_counts_are_tree_independent():
    cnf = CNFInstance.random(3, 16, 64, rng=3)
    exp = orc.brute_force_count(16, cnf.clauses)
    for seed in range(3):
        tree = _clause_tree(16, cnf.clauses, seed)
        assert orc.cnf_count_by_tree(16, cnf.clauses, tree.steps) == exp


def test_sharp_sat_notebook_example():
    kat = _json("notebook_kats.json")["sharp_sat_example"]
    assert orc.brute_force_count(3, kat["clauses"]) == kat["count"] == 6


def test_rewire_array_semantics():
    # like upstream rewire_array, kept ports must stay in input order (permutations go
    # through np.transpose in FinRel._rewire before this is reached)
    a = np.arange(6, dtype=np.uint64).reshape(2, 3)
    np.testing.assert_array_equal(orc.rewire_array(a, [0]), a.sum(axis=1))
    with pytest.raises(ValueError):
        orc.rewire_array(a, [1, 0])
    np.testing.assert_array_equal(orc.rewire_or_and(a.astype(np.uint8) % 2, [1, 0]),
                                  (a.T % 2).astype(np.uint8))
    d = orc.rewire_array(np.array([1, 2], dtype=np.uint64), [0, 0])
    np.testing.assert_array_equal(d, np.diag([1, 2]))
