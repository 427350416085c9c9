"""Host front end parity (no GPU): CNF generation, DIMACS parsing, diagrams and wirings
match the reference's own outputs recorded in tests/golden."""

from __future__ import annotations

import json
from pathlib import Path

import numpy as np
import pytest

from oracle import finrel_oracle as orc
from tensorsat_gb300.contractions.simple import SimpleContraction
from tensorsat_gb300.diagrams import Wiring
from tensorsat_gb300.lang.cuda_rel import CudaRel, FinSet
from tensorsat_gb300.lib import bincirc
from tensorsat_gb300.lib.sat import CNFInstance

GOLDEN = Path(__file__).resolve().parent / "golden"


def _json(name):
    return json.loads((GOLDEN / name).read_text())


@pytest.mark.parametrize("case", _json("random_instances.json"),
                         ids=lambda c: f"k{c['k']}n{c['n']}m{c['m']}")
def test_random_instances_match_reference_streams(case):
    if "ragged_index" in case:
        g = np.random.default_rng(case["ragged_index"])
        n = int(g.integers(30, 81))
        m = round(float(g.uniform(3.5, 5.0)) * n)
        assert (n, m) == (case["n"], case["m"])
        cnf = CNFInstance.random(3, n, m, rng=g)
    else:
        cnf = CNFInstance.random(case["k"], case["n"], case["m"], rng=case["rng"])
    assert [list(c) for c in cnf.clauses] == case["clauses"]


@pytest.mark.parametrize("case", _json("dimacs.json"), ids=lambda c: c["file"])
def test_dimacs_parser(case):
    cnf = CNFInstance.from_dimacs(case["dimacs"])
    assert cnf.num_vars == case["num_vars"]
    assert [list(c) for c in cnf.clauses] == case["clauses"]
    again = CNFInstance.from_dimacs(cnf.to_dimacs())
    assert again.clauses == cnf.clauses and again.num_vars == cnf.num_vars


def test_dimacs_errors():
    with pytest.raises(ValueError):
        CNFInstance.from_dimacs("p dnf 2 1\n1 2 0")
    with pytest.raises(ValueError):
        CNFInstance.from_dimacs("p cnf 2 2\n1 2 0")
    with pytest.raises(ValueError):
        CNFInstance.from_dimacs("p cnf 1 1\n1 2 0")


def test_random_argument_errors():
    for args in [(0, 5, 3), (4, 3, 3), (3, 5, 0), (1, 2, 5)]:
        with pytest.raises(ValueError):
            CNFInstance.random(*args, rng=0)


def _diagram_for(case):
    cnf = CNFInstance.random(case["k"], case["n"], case["m"], rng=case["rng"])
    spec = case["inputs"]
    if spec == "discard_unk":
        return (cnf.inputs(None, discard_unk=True) >> cnf.diagram()).flatten()
    if spec == "contraction_wiring":
        return cnf.contraction_wiring()
    if spec == "diagram":
        return cnf.diagram()
    return (cnf.inputs(spec) >> cnf.diagram()).flatten()


@pytest.mark.parametrize("case", _json("wirings.json"), ids=lambda c: str(c["inputs"]))
def test_flattened_wirings_match_reference(case):
    d = _diagram_for(case)
    w = d if isinstance(d, Wiring) else d.wiring
    assert [list(x) for x in w.slot_wires_list] == case["slot_wires_list"]
    assert list(w.out_wires) == case["out_wires"]
    assert w.num_wires == case["num_wires"]
    if case["boxes"] is not None:
        assert [b.name for b in d.boxes] == case["boxes"]


def test_inputs_validation():
    cnf = CNFInstance.random(3, 4, 3, rng=0)
    with pytest.raises(ValueError):
        cnf.inputs("01")
    with pytest.raises(ValueError):
        cnf.inputs("01x?")
    with pytest.raises(ValueError):
        cnf.inputs(-1)
    # '_' leaves the variable open: an input port, then the output port every wire gets
    d = cnf.inputs("01?_")
    assert d.wiring.num_slots == 3 and d.wiring.out_wires == (3, 0, 1, 2, 3)


def test_gate_tensors():
    assert bincirc.not_.numpy().tolist() == [[0, 1], [1, 0]]
    assert bincirc.or_.to_set() == {(a, b, a | b) for a in (0, 1) for b in (0, 1)}
    assert bincirc.bit_unk.numpy().tolist() == [1, 1]
    assert bincirc.bit_1.numpy().tolist() == [0, 1]
    assert bincirc.bit.size == 2 and FinSet(2) is bincirc.bit


def test_clause_diagram_tensors_match_oracle():
    cnf = CNFInstance(4, [(1, -2, 3), (-1, -1), (2, -2, 4)])
    d = cnf.clause_diagram("1??_")
    assert d.wiring.out_wires == (3,)
    for clause, ws, box in zip(cnf.clauses, d.wiring.slot_wires_list, d.boxes):
        t, vs = orc.clause_tensor(clause)
        assert tuple(ws) == vs
        np.testing.assert_array_equal(box.numpy(), t)
    assert d.boxes[-1] is bincirc.bit_1


def test_contract2_argument_validation_is_host_side():
    with pytest.raises(ValueError):
        CudaRel.contract2(bincirc.or_, [0, 1], bincirc.not_, [1, 2])
    with pytest.raises(ValueError):
        CudaRel.contract2(bincirc.or_, [0, 1, 2], bincirc.not_, [2, 3], [0, 7])
    with pytest.raises(ValueError):
        bincirc.or_.rewire([0, 5])
    with pytest.raises(ValueError):
        bool(bincirc.or_)


def test_simple_contraction_bookkeeping_matches_reference_restatement():
    cnf = CNFInstance.random(3, 5, 8, rng=0)
    d = (cnf.inputs(None) >> cnf.diagram()).flatten()
    n = d.wiring.num_slots
    rng = np.random.default_rng(0)
    path = [tuple(int(x) for x in rng.choice(n - i, size=2, replace=False)) for i in range(n - 1)]
    sc = SimpleContraction(CudaRel, d.wiring, path)
    exp = orc.simple_contract2_args(d.wiring.slot_wires_list, d.wiring.out_wires, path)
    assert [tuple(map(tuple, (a[1], a[3], a[4]))) for a in sc.contract2_args] == \
        [tuple(map(tuple, (e[1], e[3], e[4]))) for e in exp]
    with pytest.raises(ValueError):
        SimpleContraction(CudaRel, d.wiring, path[:-1])
    with pytest.raises(ValueError):
        SimpleContraction(CudaRel, d.wiring, [(n, 0)] + path[1:])


def test_contraction_validation():
    from tensorsat_gb300.contractions.gpu import GpuContraction

    cnf = CNFInstance.random(3, 6, 10, rng=1)
    d = (cnf.inputs(None) >> cnf.diagram()).flatten()
    c = GpuContraction(CudaRel, d.wiring)
    # the wiring does not depend on the input values (plan reuse across assignments)
    assert c.can_contract((cnf.inputs("0?1???") >> cnf.diagram()).flatten())
    other_cnf = CNFInstance.random(3, 6, 10, rng=2)
    assert not c.can_contract((other_cnf.inputs(None) >> other_cnf.diagram()).flatten())
    assert c.can_contract(d)
    nested = cnf.inputs(None) >> cnf.diagram()
    assert not c.can_contract(nested)
    assert len(c.path) == len(c.tree.steps)


def test_zero_dim_tensors_keep_their_shape():
    """0-d arrays stay 0-d in boxes (a scalar relation, or the clause tensor of an empty
    clause), so their port count matches the wiring."""
    import numpy as np

    from tensorsat_gb300.lang.cuda_rel import CudaRel, leaf_array
    from tensorsat_gb300.lib.sat import CNFInstance

    assert tuple(CudaRel(np.array(1, dtype=np.uint8)).tensor.shape) == ()
    d = CNFInstance(2, [(1, 2), ()]).clause_diagram()
    assert [leaf_array(b).shape for b in d.blocks] == [(2, 2), ()]
    assert d.wiring.slot_wires_list[1] == ()
