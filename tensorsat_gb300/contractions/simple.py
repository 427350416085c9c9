"""Contractions along an explicit pop/append path (``tensorsat/contractions/simple.py``).

:class:`SimpleContraction` reproduces the reference's bookkeeping exactly
(``simple.py:231-291``): each step's result keeps ``lhs_only + common + rhs_only`` wires,
and a wire missing from the wiring's out wires is dropped only from the *last* step whose
result carries it. Every intermediate therefore keeps all the wires of its subtree until
the root, which makes this driver exponential in the network size; it exists for API
parity and small networks. :class:`~tensorsat_gb300.contractions.gpu.GpuContraction` is
the driver with per-step wire elimination and the tree executor.

Each step calls ``box_class._contract2``; with :class:`CudaRel` that is one device
contraction per step.
"""

from __future__ import annotations

from collections.abc import Sequence
from typing import TypeAlias

from ..diagrams import Box, Diagram, TensorLikeType, Wire, Wires, Wiring
from .abc import Contraction

ContractionPath: TypeAlias = tuple[tuple[int, int], ...]
Contract2Args: TypeAlias = tuple[int, Wires, int, Wires, Wires]


class SimpleContraction(Contraction):
    """A simple contraction based on an explicit contraction path."""

    def __init__(self, box_class: type, wiring: Wiring, path: Sequence[tuple[int, int]]) -> None:
        path = tuple(tuple(p) for p in path)
        super().__init__(box_class, wiring)
        if wiring.num_wires == 0:
            raise ValueError("Cannot define contraction for empty wiring.")
        for t in wiring.wire_types:
            if not isinstance(t, TensorLikeType):
                raise ValueError("Wiring must have tensor-like wire types.")
        n = wiring.num_slots
        if not path and n >= 2:
            raise ValueError("Contraction path can only be empty for number of wiring slots <= 1.")
        if len(path) >= n and n > 0:
            raise ValueError(
                "Path is too long for the given wiring:"
                f" there are {len(path)} contractions, but {n} slots to contract."
            )
        if n and len(path) != n - 1:
            raise ValueError(
                "Path does not fully contract the given wiring:"
                f" there are {len(path)} contractions, but {n} slots to contract."
            )
        for idx, (lhs, rhs) in enumerate(path):
            if not 0 <= lhs < n - idx:
                raise ValueError(f"Invalid lhs for contraction {(lhs, rhs) = } at {idx = }.")
            if not 0 <= rhs < n - idx:
                raise ValueError(f"Invalid rhs for contraction {(lhs, rhs) = } at {idx = }.")
        self._path = path
        self._init_args()

    def _init_args(self) -> None:
        wiring = self._wiring
        if self._path:
            args: list[tuple[int, Wires, int, Wires, list[Wire]]] = []
            wires_list = list(wiring.slot_wires_list)
            for lhs_idx, rhs_idx in self._path:
                lhs_wires = wires_list.pop(lhs_idx)
                rhs_wires = wires_list.pop(rhs_idx - int(lhs_idx < rhs_idx))
                common = set(lhs_wires) & set(rhs_wires)
                if common:
                    res = (
                        tuple(w for w in lhs_wires if w not in common)
                        + tuple(w for w in lhs_wires if w in common)
                        + tuple(w for w in rhs_wires if w not in common)
                    )
                else:
                    res = tuple(lhs_wires) + tuple(rhs_wires)
                wires_list.append(res)
                args.append((lhs_idx, lhs_wires, rhs_idx, rhs_wires, list(res)))
            final = args[-1][-1]
            for w in sorted(set(final) - set(wiring.out_wires)):
                for *_, res_list in reversed(args):
                    if w in res_list:
                        res_list.remove(w)
                        break
            self._args = tuple((a, aw, b, bw, tuple(r)) for a, aw, b, bw, r in args)
            self._box_out_wires = tuple(final)
        else:
            self._args = ()
            self._box_out_wires = () if wiring.num_slots == 0 else wiring.slot_wires_list[0]
        self._dangling = tuple(sorted(wiring.dangling_wires))

    @property
    def contract2_args(self) -> tuple[Contract2Args, ...]:
        """The arguments of every contract2 call of the contraction."""
        return self._args

    @property
    def path(self) -> ContractionPath:
        return self._path

    def contract(self, diagram: Diagram) -> Box:
        self.validate(diagram)
        cls = self._box_class
        wiring = self._wiring
        boxes = list(diagram.boxes)
        box = None
        if boxes:
            for lhs_idx, lhs_wires, rhs_idx, rhs_wires, res_wires in self._args:
                lhs = boxes.pop(lhs_idx)
                rhs = boxes.pop(rhs_idx - int(lhs_idx < rhs_idx))
                boxes.append(cls._contract2(lhs, lhs_wires, rhs, rhs_wires, res_wires))
            box = boxes[0]
        out_wires = wiring.out_wires
        box_out = self._box_out_wires
        if self._dangling:
            box_out = box_out + self._dangling
            spiders = [cls._spider(wiring.wire_types[w], 1) for w in self._dangling]
            box = cls.prod([boxes[0], *spiders]) if boxes else cls.prod(spiders)
        if out_wires != box_out:
            box = box._rewire([box_out.index(w) for w in out_wires])
        return box

    def __repr__(self) -> str:
        return "<SimpleContraction>"
