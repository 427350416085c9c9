"""CNF instances and the diagrams they compile to.

:class:`CNFInstance` keeps the API of ``tensorsat/lib/sat.py:40-275``:

* :meth:`CNFInstance.random` draws clauses with the same sequence of numpy ``Generator``
  calls as the reference (``sat.py:43-78``), so a seed names the same instance;
* :meth:`CNFInstance.from_dimacs` / :meth:`to_dimacs` parse and print DIMACS like
  ``sat.py:80-100,135-142``;
* :meth:`inputs`, :meth:`diagram` and :meth:`contraction_wiring` build the same diagrams,
  slot for slot and wire for wire, as ``sat.py:165-262`` (NOT per negative literal, a
  balanced OR tree per clause, ``bit_1`` on its output).

:meth:`CNFInstance.clause_diagram` is new: it compiles the instance straight into the
flat network of one ``2^k`` clause tensor per clause (zero only at the clause's single
falsifying assignment) over variable wires, which is what contracting the bintree
diagram's gates per clause produces, without the per-gate detour.
"""

from __future__ import annotations

import re
from collections.abc import Sequence
from math import comb
from typing import Literal, TypeAlias

import numpy as np

from ..diagrams import Diagram, DiagramBuilder, Wire, Wiring
from ..lang.cuda_rel import CudaRel
from .bincirc import bit, bit_0, bit_1, bit_unk, bits, not_, or_

Clause: TypeAlias = tuple[int, ...]
CNFDiagramMode: TypeAlias = Literal["bintree"]


class CNFInstance:
    """A SAT instance in CNF form."""

    __slots__ = ("_num_vars", "_clauses")

    @classmethod
    def random(cls, k: int, n: int, m: int, *, rng: int | np.random.Generator | None = None
               ) -> "CNFInstance":
        """Random ``k``-SAT instance with ``n`` variables and ``m`` distinct clauses: each
        clause takes ``k`` distinct variables and independent fair signs, and is stored
        sorted; duplicate clauses are redrawn."""
        if k <= 0:
            raise ValueError("Clause size 'k' must be positive.")
        if n < k:
            raise ValueError(f"Number of variables 'n' must be at least {k = }.")
        if m <= 0:
            raise ValueError("Number of clauses 'm' must be positive.")
        if m > comb(n, k) * 2**k:
            raise ValueError(f"Number of clauses 'm' cannot exceed {comb(n, k)*2**k = }")
        if not isinstance(rng, np.random.Generator):
            rng = np.random.default_rng(rng)
        clauses: list[Clause] = []
        seen: set[Clause] = set()
        while len(clauses) < m:
            variables = [int(v) for v in rng.choice(range(n), size=k, replace=False)]
            negated = [int(s) for s in rng.choice(range(2), size=k)]
            clause = tuple(sorted(-v - 1 if neg else v + 1 for v, neg in zip(variables, negated)))
            if clause not in seen:
                seen.add(clause)
                clauses.append(clause)
        return cls._new(n, tuple(clauses))

    @classmethod
    def from_dimacs(cls, dimacs: str) -> "CNFInstance":
        """Parses a DIMACS CNF string (comment lines start with 'c')."""
        lines = [
            s for line in dimacs.strip().split("\n") if (s := line.strip()) and not s.startswith("c")
        ]
        header = re.compile(r"p cnf ([0-9]+) ([0-9]+)").match(lines[0])
        if not header:
            raise ValueError("DIMACS code must start with 'p cnf <num vars> <num clauses>'.")
        num_vars, num_clauses = map(int, header.groups())
        clauses = tuple(tuple(map(int, line.split(" ")))[:-1] for line in lines[1:])
        if len(clauses) != num_clauses:
            raise ValueError("Number of clauses does not match the specified number.")
        if num_vars < max(abs(lit) for clause in clauses for lit in clause):
            raise ValueError("Clauses contain invalid variables.")
        return cls._new(num_vars, clauses)

    @classmethod
    def _new(cls, num_vars: int, clauses: tuple[Clause, ...]) -> "CNFInstance":
        self = object.__new__(cls)
        self._num_vars = num_vars
        self._clauses = clauses
        return self

    def __new__(cls, num_vars: int, clauses: Sequence[Sequence[int]]) -> "CNFInstance":
        if num_vars < max(abs(lit) for clause in clauses for lit in clause):
            raise ValueError("Clauses contain invalid variables.")
        return cls._new(num_vars, tuple(tuple(c) for c in clauses))

    @property
    def num_vars(self) -> int:
        return self._num_vars

    @property
    def clauses(self) -> tuple[Clause, ...]:
        return self._clauses

    def to_dimacs(self) -> str:
        lines = [f"p cnf {self._num_vars} {len(self._clauses)}"]
        lines.extend(f"{' '.join(map(str, c))} 0" for c in self._clauses)
        return "\n".join(lines)

    def _normalize_inputs(self, inputs: str | int | None) -> str:
        n = self._num_vars
        if isinstance(inputs, int):
            if inputs < 0:
                raise ValueError("Inputs must be specified by a non-negative number.")
            return f"{inputs:0>{n}b}"
        if inputs is None:
            return "?" * n
        if not all(b in "01?_" for b in inputs):
            raise ValueError("Input specification characters must be '0', '1', '?' or '_'.")
        if len(inputs) != n:
            raise ValueError(
                f"Expected input specification string to be {n} characters long,"
                f" found {len(inputs)} characters instead."
            )
        return inputs

    def inputs(self, inputs: str | int | None, /, *, discard_unk: bool = False) -> Diagram:
        """Diagram fixing each variable: '0' -> bit_0, '1' -> bit_1, '?' -> bit_unk (or a
        bare discarded wire when ``discard_unk``), '_' -> left open as an input."""
        spec = self._normalize_inputs(inputs)
        builder = DiagramBuilder()
        for i, b in enumerate(spec):
            if b == "0":
                (w,) = bit_0 @ builder
            elif b == "1":
                (w,) = bit_1 @ builder
            elif b == "?":
                if discard_unk:
                    w = builder.wiring.add_wire(bit)
                else:
                    (w,) = bit_unk @ builder
            else:
                w = builder.add_input(bit)
            assert w == i
        builder.add_outputs(builder.wiring.wires)
        return builder.diagram()

    def diagram(self, *, mode: CNFDiagramMode = "bintree") -> Diagram:
        if mode == "bintree":
            return self._build_diagram_bintree()
        raise NotImplementedError(f"Unknown diagram mode for CNFInstance: {mode!r}")

    def contraction_wiring(self, *, mode: CNFDiagramMode = "bintree") -> Wiring:
        """Wiring shared by ``inputs(x) >> diagram()`` for every input specification."""
        return (self.inputs(0) >> self.diagram(mode=mode)).flatten().wiring

    def _build_diagram_bintree(self) -> Diagram:
        builder = DiagramBuilder()
        builder.add_inputs(bits(self._num_vars))
        for clause in self._clauses:
            # literal wires: the variable itself, or a NOT gate's output
            layer: list[Wire] = []
            for lit in clause:
                if lit > 0:
                    layer.append(lit - 1)
                else:
                    layer.append((not_ @ builder[-lit - 1])[0])
            # balanced OR tree: pair neighbours; an odd leftover joins the last pair
            while len(layer) > 1:
                paired = [(or_ @ builder[layer[2 * i: 2 * i + 2]])[0] for i in range(len(layer) // 2)]
                if len(layer) % 2 == 1:
                    (paired[-1],) = or_ @ builder[paired[-1], layer[-1]]
                layer = paired
            bit_1 @ builder[layer[0]]
        return builder.diagram()

    def clause_diagram(self, inputs: str | int | None = None) -> Diagram:
        """Flat diagram with one clause tensor per clause over the variable wires.

        Wire ``i`` is variable ``i+1``. A clause over the distinct variables
        ``v_1..v_r`` (first-appearance order) is the ``2^r`` tensor that is 1 exactly at
        the assignments satisfying one of its literals. Inputs '0'/'1' add a ``bit_0`` /
        ``bit_1`` unit slot on the variable, '?' leaves the wire to be summed, '_' makes it
        an out wire. Variables in no clause stay as wires without slots (a factor 2 each
        in the model count).
        """
        spec = self._normalize_inputs(inputs)
        n = self._num_vars
        slot_wires: list[tuple[int, ...]] = []
        boxes: list[CudaRel] = []
        for clause in self._clauses:
            vs = list(dict.fromkeys(abs(l) - 1 for l in clause))
            r = len(vs)
            idx = np.indices((2,) * r).reshape(r, -1).T if r else np.zeros((1, 0), dtype=int)
            pos = {v: i for i, v in enumerate(vs)}
            sat = np.zeros(idx.shape[0], dtype=np.uint8)
            for lit in clause:
                col = idx[:, pos[abs(lit) - 1]]
                sat |= (col == (1 if lit > 0 else 0)).astype(np.uint8)
            slot_wires.append(tuple(vs))
            boxes.append(CudaRel._new(_host_u8(sat.reshape((2,) * r))))
        for i, b in enumerate(spec):
            if b == "0":
                slot_wires.append((i,))
                boxes.append(bit_0)
            elif b == "1":
                slot_wires.append((i,))
                boxes.append(bit_1)
        out = tuple(i for i, b in enumerate(spec) if b == "_")
        wiring = Wiring(wire_types=(bit,) * n, slot_wires_list=slot_wires, out_wires=out)
        return Diagram._new(wiring, tuple(boxes))

    def __repr__(self) -> str:
        attrs = [f"{self._num_vars} vars", f"{len(self._clauses)} clauses"]
        ks = {len(c) for c in self._clauses}
        if len(ks) == 1:
            attrs.append(f"k={ks.pop()}")
        else:
            attrs.append(f"k in [{min(ks)}..{max(ks)}]")
        return f"<CNFInstance: {', '.join(attrs)}>"


def _host_u8(a: np.ndarray):
    import torch

    return torch.from_numpy(np.require(a, dtype=np.uint8, requirements="C"))  # keeps 0-d arrays 0-d


__all__ = ["CNFInstance", "Clause", "CNFDiagramMode", "bit_unk"]
