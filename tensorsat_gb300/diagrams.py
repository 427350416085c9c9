"""Wirings, boxes and diagrams: the host-side structures the contraction path consumes.

This module restates the parts of ``tensorsat/diagrams.py`` that the CNF contraction path
uses, with the same names, argument meanings, wire/slot numbering and errors:

* :class:`Wiring` (``tensorsat/diagrams.py:153-478``): slots, wires, out wires and
  :meth:`Wiring.compose`, whose wire numbering follows ``Wiring._compose``
  (``:387-461``): outer wires first, each connected component represented by its lowest
  outer wire, then the unmatched wires of every plugged wiring in slot order.
* :class:`Box` / :class:`TensorLikeBox` (``:693-1031``): the plugin interface a box class
  implements (``_contract2``, ``_rewire``, ``_spider``, ``_scalar``, ``_stack``,
  ``_getitem``, ``_union``, ``_as_scalar``) with the public wrappers that validate
  arguments (``contract2`` ``:811-844``, ``rewire``, ``prod`` ``:719-746``, ...).
* :class:`Diagram`, :class:`DiagramBuilder`, :class:`SelectedBlockPorts` and
  :class:`SelectedBuilderWires` (``:1217-1952``): building, ``>>`` sequential composition
  and :meth:`Diagram.flatten`.

Hash-consing, the slotted metaclass machinery, recipes and port-order structures of the
reference are not restated: they do not influence what gets contracted.
"""

from __future__ import annotations

from abc import ABC, abstractmethod
from collections.abc import Iterable, Mapping, Sequence
from types import MappingProxyType
from typing import Any, TypeAlias, Union

Slot: TypeAlias = int
Port: TypeAlias = int
Wire: TypeAlias = int
Slots: TypeAlias = tuple[Slot, ...]
Ports: TypeAlias = tuple[Port, ...]
Wires: TypeAlias = tuple[Wire, ...]


class Type(ABC):
    """Abstract base class for wire types."""


class TensorLikeType(Type):
    """A wire type with a tensor dimension (``tensorsat/diagrams.py:76-88``)."""

    @property
    @abstractmethod
    def tensor_dim(self) -> int: ...


Shape: TypeAlias = tuple[Type, ...]


class Shaped(ABC):
    """Objects with a shape (a tuple of types) and ports ``0..len(shape)-1``."""

    @property
    @abstractmethod
    def shape(self) -> Shape: ...

    @property
    def num_ports(self) -> int:
        return len(self.shape)

    @property
    def ports(self) -> Sequence[Port]:
        return range(self.num_ports)


class Wiring(Shaped):
    """An immutable wiring: a wire for each port of each slot, and out wires."""

    __slots__ = ("_wire_types", "_slot_wires_list", "_out_wires", "_slot_shapes", "_hash")

    def __init__(
        self,
        *,
        wire_types: Sequence[Type],
        slot_wires_list: Sequence[Sequence[Wire]],
        out_wires: Sequence[Wire],
    ) -> None:
        wire_types = tuple(wire_types)
        slot_wires_list = tuple(tuple(ws) for ws in slot_wires_list)
        out_wires = tuple(out_wires)
        num_wires = len(wire_types)
        for slot, ws in enumerate(slot_wires_list):
            for w in ws:
                if w not in range(num_wires):
                    raise ValueError(f"Invalid wire index {w} in slot mapping for slot {slot}.")
        for w in out_wires:
            if w not in range(num_wires):
                raise ValueError(f"Invalid wire index {w} in outer mapping.")
        self._wire_types = wire_types
        self._slot_wires_list = slot_wires_list
        self._out_wires = out_wires
        self._slot_shapes = tuple(tuple(wire_types[w] for w in ws) for ws in slot_wires_list)
        self._hash = hash((wire_types, slot_wires_list, out_wires))

    @property
    def wire_types(self) -> Shape:
        return self._wire_types

    @property
    def slot_wires_list(self) -> tuple[Wires, ...]:
        return self._slot_wires_list

    @property
    def out_wires(self) -> Wires:
        return self._out_wires

    @property
    def slot_shapes(self) -> tuple[Shape, ...]:
        return self._slot_shapes

    @property
    def shape(self) -> Shape:
        return tuple(self._wire_types[o] for o in self._out_wires)

    @property
    def num_slots(self) -> int:
        return len(self._slot_wires_list)

    @property
    def slots(self) -> Sequence[Slot]:
        return range(self.num_slots)

    def num_slot_ports(self, slot: Slot) -> int:
        return len(self._slot_shapes[slot])

    def slot_ports(self, slot: Slot) -> Sequence[Port]:
        return range(self.num_slot_ports(slot))

    @property
    def num_wires(self) -> int:
        return len(self._wire_types)

    @property
    def wires(self) -> Sequence[Wire]:
        return range(self.num_wires)

    def slot_wires(self, slot: Slot) -> Wires:
        if slot not in range(self.num_slots):
            raise ValueError(f"Invalid slot {slot}.")
        return self._slot_wires_list[slot]

    @property
    def dangling_wires(self) -> frozenset[Wire]:
        """Wires not connected to any slot port."""
        return frozenset(self.wires) - frozenset(w for ws in self._slot_wires_list for w in ws)

    @property
    def discarded_wires(self) -> frozenset[Wire]:
        return frozenset(self.wires) - set(self._out_wires)

    @property
    def wired_slots(self) -> Mapping[Wire, Slots]:
        res: dict[Wire, list[Slot]] = {}
        for slot, ws in enumerate(self._slot_wires_list):
            for w in ws:
                res.setdefault(w, []).append(slot)
        return MappingProxyType({w: tuple(s) for w, s in res.items()})

    def validate_slot_data(self, data: Mapping[Slot, Shaped], /) -> None:
        for slot, shaped in data.items():
            if slot not in self.slots:
                raise ValueError(f"Invalid slot {slot}.")
            if tuple(shaped.shape) != self._slot_shapes[slot]:
                raise ValueError(
                    f"Incompatible shape for data at slot {slot}:"
                    f" expected slot shape {self._slot_shapes[slot]},"
                    f"  got data with shape {shaped.shape}."
                )

    def compose(self, wirings: Mapping[Slot, "Wiring"]) -> "Wiring":
        """Plugs the given wirings into (some of) the slots of this wiring."""
        for slot, wiring in wirings.items():
            if slot not in self.slots:
                raise ValueError(f"Invalid slot {slot}.")
            if wiring.shape != self._slot_shapes[slot]:
                raise ValueError(
                    f"Incompatible shape in wiring composition for slot {slot}:"
                    f" expected slot shape {self._slot_shapes[slot]},"
                    f" got a wiring of shape {wiring.shape}."
                )
        return self._compose(wirings)

    def _compose(self, wirings: Mapping[Slot, "Wiring"]) -> "Wiring":
        # Union-find over outer wires ("o", w) and plugged wires ("i", slot, w): an outer
        # wire at a slot port is fused with the plugged wiring's out wire at that port.
        parent: dict[Any, Any] = {}

        def find(x: Any) -> Any:
            root = x
            while parent.get(root, root) != root:
                root = parent[root]
            while parent.get(x, x) != root:
                nxt = parent[x]
                parent[x] = root
                x = nxt
            return root

        def union(a: Any, b: Any) -> None:
            ra, rb = find(a), find(b)
            if ra != rb:
                parent[rb] = ra

        linked: set[Any] = set()
        for slot, wiring in wirings.items():
            for self_w, sub_w in zip(self._slot_wires_list[slot], wiring.out_wires):
                a, b = ("o", self_w), ("i", slot, sub_w)
                linked.update((a, b))
                union(a, b)
        # representative of a component: its lowest outer wire
        lowest: dict[Any, Wire] = {}
        for w in self.wires:
            r = find(("o", w))
            if r not in lowest:
                lowest[r] = w
        new_id: dict[Any, Wire] = {}
        wire_types: list[Type] = []
        for w in self.wires:
            rep = lowest[find(("o", w))]
            if rep != w:
                new_id[("o", w)] = new_id[("o", rep)]
            else:
                new_id[("o", w)] = len(wire_types)
                wire_types.append(self._wire_types[w])
        for slot, wiring in wirings.items():
            for w in wiring.wires:
                key = ("i", slot, w)
                if key in linked:
                    new_id[key] = new_id[("o", lowest[find(key)])]
                else:
                    new_id[key] = len(wire_types)
                    wire_types.append(wiring.wire_types[w])
        slot_wires_list: list[Wires] = []
        for slot in self.slots:
            if slot in wirings:
                sub = wirings[slot]
                slot_wires_list.extend(
                    tuple(new_id[("i", slot, w)] for w in ws) for ws in sub.slot_wires_list
                )
            else:
                slot_wires_list.append(tuple(new_id[("o", w)] for w in self._slot_wires_list[slot]))
        out_wires = tuple(new_id[("o", w)] for w in self._out_wires)
        return Wiring(wire_types=wire_types, slot_wires_list=slot_wires_list, out_wires=out_wires)

    def __eq__(self, other: Any) -> bool:
        if not isinstance(other, Wiring):
            return NotImplemented
        return (
            self._wire_types == other._wire_types
            and self._slot_wires_list == other._slot_wires_list
            and self._out_wires == other._out_wires
        )

    def __hash__(self) -> int:
        return self._hash

    def __repr__(self) -> str:
        attrs = []
        if self.num_wires:
            attrs.append(f"{self.num_wires} wire{'s' if self.num_wires != 1 else ''}")
        if self.num_slots:
            attrs.append(f"{self.num_slots} slot{'s' if self.num_slots != 1 else ''}")
        if self._out_wires:
            n = len(self._out_wires)
            attrs.append(f"{n} out port{'s' if n != 1 else ''}")
        return "<Wiring (empty)>" if not attrs else f"<Wiring: {', '.join(attrs)}>"


class WiringBuilder(Shaped):
    """Mutable builder of wirings (``tensorsat/diagrams.py:481-647``)."""

    def __init__(self) -> None:
        self._wire_types: list[Type] = []
        self._slot_wires_list: list[list[Wire]] = []
        self._out_wires: list[Wire] = []

    @property
    def shape(self) -> Shape:
        return tuple(self._wire_types[w] for w in self._out_wires)

    @property
    def num_wires(self) -> int:
        return len(self._wire_types)

    @property
    def wires(self) -> Sequence[Wire]:
        return range(self.num_wires)

    @property
    def wire_types(self) -> Shape:
        return tuple(self._wire_types)

    @property
    def num_slots(self) -> int:
        return len(self._slot_wires_list)

    @property
    def slot_shapes(self) -> tuple[Shape, ...]:
        return tuple(tuple(self._wire_types[w] for w in ws) for ws in self._slot_wires_list)

    @property
    def out_wires(self) -> Wires:
        return tuple(self._out_wires)

    @property
    def wiring(self) -> Wiring:
        return Wiring(
            wire_types=self._wire_types,
            slot_wires_list=self._slot_wires_list,
            out_wires=self._out_wires,
        )

    def add_wire(self, t: Type) -> Wire:
        return self.add_wires([t])[0]

    def add_wires(self, ts: Sequence[Type]) -> Wires:
        start = len(self._wire_types)
        self._wire_types.extend(ts)
        return tuple(range(start, len(self._wire_types)))

    def _validate_wires(self, wires: Sequence[Wire]) -> None:
        for w in wires:
            if w not in range(self.num_wires):
                raise ValueError(f"Invalid wire index {w}.")

    def add_out_ports(self, wires: Sequence[Wire]) -> Ports:
        self._validate_wires(wires)
        start = len(self._out_wires)
        self._out_wires.extend(wires)
        return tuple(range(start, len(self._out_wires)))

    def add_slot(self) -> Slot:
        self._slot_wires_list.append([])
        return len(self._slot_wires_list) - 1

    def add_slot_ports(self, slot: Slot, wires: Sequence[Wire]) -> Ports:
        if slot not in range(self.num_slots):
            raise ValueError(f"Invalid slot {slot}.")
        self._validate_wires(wires)
        start = len(self._slot_wires_list[slot])
        self._slot_wires_list[slot].extend(wires)
        return tuple(range(start, len(self._slot_wires_list[slot])))


BoxClass: TypeAlias = type


class Box(Shaped):
    """Abstract base class of boxes; subclasses implement the protected methods."""

    __slots__ = ("_name",)

    def __init__(self, name: str | None = None) -> None:
        self._name = name

    @property
    def name(self) -> str | None:
        return self._name

    @staticmethod
    def class_join(bases: Iterable[type]) -> type:
        """The most specific common box class of the given classes."""
        bases = list(bases)
        if not bases:
            return Box
        common = [c for c in bases[0].__mro__ if issubclass(c, Box)]
        for b in bases[1:]:
            common = [c for c in common if issubclass(b, c)]
        return common[0]

    @classmethod
    def can_be_contracted(cls) -> bool:
        abstract = getattr(cls, "__abstractmethods__", frozenset())
        return not ({"_contract2", "_rewire", "_spider"} & set(abstract))

    @classmethod
    def prod(cls, boxes: Iterable["Box"]) -> "Box":
        """Product of one or more boxes, ports in the order given
        (``tensorsat/diagrams.py:719-746``)."""
        boxes = tuple(boxes)
        for box in boxes:
            if not isinstance(box, cls):
                raise TypeError(
                    f"Boxes must be instances of box class {cls},"
                    f" found instance of box class {type(box)} instead."
                )
        if not boxes:
            raise ValueError("Products must involve at least one box.")
        res = boxes[0]
        for box in boxes[1:]:
            n, m = len(res.shape), len(box.shape)
            res = cls._contract2(res, range(n), box, range(n, n + m), range(n + m))
        return res

    @classmethod
    def spider(cls, t: Type, num_ports: int) -> "Box":
        if not isinstance(num_ports, int) or num_ports <= 0:
            raise ValueError("Number of ports must be strictly positive.")
        return cls._spider(t, num_ports)

    @classmethod
    @abstractmethod
    def _spider(cls, t: Type, num_ports: int) -> "Box": ...

    @classmethod
    def scalar(cls, scalar: bool, /) -> "Box":
        box = cls._scalar(scalar)
        assert box.shape == ()
        return box

    @classmethod
    @abstractmethod
    def _scalar(cls, scalar: bool, /) -> "Box": ...

    @classmethod
    def contract2(
        cls,
        lhs: "Box",
        lhs_wires: Sequence[Wire],
        rhs: "Box",
        rhs_wires: Sequence[Wire],
        out_wires: Sequence[Wire] | None = None,
    ) -> "Box":
        """Validates arguments, then contracts (``tensorsat/diagrams.py:811-844``)."""
        if len(lhs_wires) != len(lhs.shape):
            raise ValueError(
                f"Number of wires in lhs ({len(lhs_wires)}) does not match"
                f" the number of ports in lhs shape ({len(lhs.shape)})."
            )
        if len(rhs_wires) != len(rhs.shape):
            raise ValueError(
                f"Number of wires in rhs ({len(rhs_wires)}) does not match"
                f" the number of ports in rhs shape ({len(rhs.shape)})."
            )
        if out_wires is None:
            out_wires = sorted(set(lhs_wires).symmetric_difference(rhs_wires))
        else:
            extra = set(out_wires) - set(lhs_wires) - set(rhs_wires)
            if extra:
                raise ValueError("Every output wire must appear in LHR or RHS.")
        return cls._contract2(lhs, lhs_wires, rhs, rhs_wires, out_wires)

    @classmethod
    @abstractmethod
    def _contract2(cls, lhs, lhs_wires, rhs, rhs_wires, out_wires) -> "Box": ...

    @classmethod
    def union(cls, boxes: Iterable["Box"]) -> "Box":
        boxes = tuple(boxes)
        if not boxes:
            raise ValueError("Cannot take an empty union: no shape info available.")
        res = boxes[0]
        for box in boxes[1:]:
            if box.shape != res.shape:
                raise ValueError("Shapes of boxes in a union must coincide.")
            res = res._union(box)
        return res

    @classmethod
    def stack(cls, boxes: Iterable["Box"], port: int = 0, /) -> "Box":
        boxes = tuple(boxes)
        if not boxes:
            raise ValueError("Need at least one box to stack.")
        if port not in range(len(boxes[0].shape) + 1):
            raise ValueError(f"Invalid port index {port} for stacking.")
        return cls._stack(boxes, port)

    @classmethod
    @abstractmethod
    def _stack(cls, boxes: tuple["Box", ...], port: int = 0, /) -> "Box": ...

    def rewire(self, out_ports: Sequence[Port]) -> "Box":
        """Permutes, duplicates and/or drops ports of this box."""
        if not all(p in self.ports for p in out_ports):
            raise ValueError("Output ports must be valid for this box.")
        return self._rewire(out_ports)

    @abstractmethod
    def _rewire(self, out_ports: Sequence[Port]) -> "Box": ...

    @abstractmethod
    def _as_scalar(self) -> bool: ...

    def __bool__(self) -> bool:
        if self.shape:
            raise ValueError("Box is not a scalar.")
        return self._as_scalar()

    def __add__(self, other: "Box") -> "Box":
        if self.shape != other.shape:
            raise ValueError("Boxes in a union must have the same shape")
        return self._union(other)

    def __getitem__(self, idxs: tuple[int | slice, ...]) -> "Box":
        for idx in idxs:
            if isinstance(idx, slice) and idx != slice(None, None, None):
                raise NotImplementedError("Non-trivial slicing is not implemented.")
        return self._getitem(idxs)

    @abstractmethod
    def _getitem(self, idxs: tuple[int | slice, ...]) -> "Box": ...

    @abstractmethod
    def _union(self, other: "Box") -> "Box": ...

    def select(self, ports: Port | Sequence[Port]) -> "SelectedBlockPorts":
        return SelectedBlockPorts(self, ports)

    def __rshift__(self, other: Any) -> "Diagram":
        return self.select(self.ports) >> other

    def __repr__(self) -> str:
        n = len(self.shape)
        cls = type(self).__name__
        if self._name is None:
            return f"<{cls}: {n} ports>"
        return f"<{cls}: {n} ports, named {self._name!r}>"


class TensorLikeBox(Box):
    """Boxes whose shape consists of tensor-like types."""

    __slots__ = ()

    @property
    @abstractmethod
    def shape(self) -> tuple[TensorLikeType, ...]: ...

    @property
    def tensor_shape(self) -> tuple[int, ...]:
        return tuple(t.tensor_dim for t in self.shape)


Block: TypeAlias = Union[Box, "Diagram"]


class Diagram(Shaped):
    """A wiring together with blocks (boxes or diagrams) for (some of) its slots."""

    __slots__ = ("_wiring", "_blocks", "_seq_blocks")

    def __init__(self, wiring: Wiring, blocks: Mapping[Slot, Block]) -> None:
        wiring.validate_slot_data(blocks)
        self._wiring = wiring
        self._blocks = tuple(blocks.get(s) for s in wiring.slots)
        self._seq_blocks: tuple[Block, ...] | None = None

    @classmethod
    def _new(cls, wiring: Wiring, blocks: tuple[Block | None, ...]) -> "Diagram":
        self = object.__new__(cls)
        self._wiring = wiring
        self._blocks = blocks
        self._seq_blocks = None
        return self

    @property
    def wiring(self) -> Wiring:
        return self._wiring

    @property
    def blocks(self) -> tuple[Block | None, ...]:
        return self._blocks

    @property
    def shape(self) -> Shape:
        return self._wiring.shape

    @property
    def open_slots(self) -> Slots:
        return tuple(s for s, b in enumerate(self._blocks) if b is None)

    @property
    def num_open_slots(self) -> int:
        return self._blocks.count(None)

    @property
    def subdiagram_slots(self) -> Slots:
        return tuple(s for s, b in enumerate(self._blocks) if isinstance(b, Diagram))

    @property
    def subdiagrams(self) -> tuple["Diagram", ...]:
        return tuple(b for b in self._blocks if isinstance(b, Diagram))

    @property
    def boxes(self) -> tuple[Box, ...]:
        return tuple(b for b in self._blocks if isinstance(b, Box))

    @property
    def is_flat(self) -> bool:
        return not any(isinstance(b, Diagram) for b in self._blocks)

    @property
    def box_classes(self) -> frozenset[type]:
        res = {type(b) for b in self.boxes}
        for d in self.subdiagrams:
            res.update(d.box_classes)
        return frozenset(res)

    @property
    def box_class(self) -> type:
        return Box.class_join(self.box_classes)

    def flatten(self, *, cache: bool = True) -> "Diagram":
        """Recursively inlines sub-diagrams (``tensorsat/diagrams.py:1452-1481``)."""
        return self._flatten({} if cache else None)

    def _flatten(self, cache: dict[int, "Diagram"] | None) -> "Diagram":
        if cache is not None and id(self) in cache:
            return cache[id(self)]
        flat_subs = [d._flatten(cache) for d in self.subdiagrams]
        sub_slots = self.subdiagram_slots
        flat_wiring = self._wiring.compose(dict(zip(sub_slots, (d.wiring for d in flat_subs))))
        index = {slot: i for i, slot in enumerate(sub_slots)}
        flat_blocks: list[Block | None] = []
        for slot, block in enumerate(self._blocks):
            i = index.get(slot)
            if i is not None:
                flat_blocks.extend(flat_subs[i].blocks)
            else:
                flat_blocks.append(block)
        res = Diagram._new(flat_wiring, tuple(flat_blocks))
        if cache is not None:
            cache[id(self)] = res
        return res

    def select(self, ports: Port | Sequence[Port]) -> "SelectedBlockPorts":
        return SelectedBlockPorts(self, ports)

    def __rshift__(self, other: Any) -> "Diagram":
        return self.select(self.ports) >> other

    def __rrshift__(self, other: Box) -> "Diagram":
        return other.select(other.ports) >> self

    def __repr__(self) -> str:
        attrs = []
        if self._wiring.num_wires:
            attrs.append(f"{self._wiring.num_wires} wires")
        if self.num_open_slots:
            attrs.append(f"{self.num_open_slots} open slots")
        if self._blocks:
            attrs.append(f"{len(self._blocks)} blocks")
        if self._wiring.out_wires:
            attrs.append(f"{len(self._wiring.out_wires)} ports")
        return "<Diagram (empty)>" if not attrs else f"<Diagram: {', '.join(attrs)}>"


class SelectedBlockPorts:
    """Selected ports of a block, for ``>>`` composition (``tensorsat/diagrams.py:1544-1644``)."""

    __slots__ = ("block", "ports")

    def __init__(self, block: Block, ports: Port | Sequence[Port]) -> None:
        if isinstance(ports, int):
            ports = (ports,)
        ports = tuple(ports)
        for p in ports:
            if p not in block.ports:
                raise ValueError(f"Invalid port {p} selected for {block}")
        self.block = block
        self.ports = ports

    def __rshift__(self, other: Any) -> Diagram:
        self_ports = self.ports
        if isinstance(other, (Box, Diagram)):
            if other.num_ports < len(self_ports):
                raise ValueError(
                    f"Cannot sequentially compose: {len(self_ports)} selected on LHS,"
                    f" {other.num_ports} ports available on RHS."
                )
            other = SelectedBlockPorts(other, range(len(self_ports)))
        elif isinstance(other, SelectedBlockPorts):
            if len(other.ports) != len(self_ports):
                raise ValueError(
                    f"Cannot sequentially compose: {len(self_ports)} selected on LHS,"
                    f" {len(other.ports)} ports selected on RHS."
                )
        else:
            return NotImplemented
        blocks: list[Block] = []
        for blk in (self.block, other.block):
            seq = getattr(blk, "_seq_blocks", None) if isinstance(blk, Diagram) else None
            if seq:
                blocks.extend(seq)
            else:
                blocks.append(blk)
        first_in = tuple(p for p in blocks[0].ports if p not in self.ports)
        builder = DiagramBuilder()
        wires = builder.add_inputs(blocks[0].shape[i] for i in first_in)
        for blk in blocks:
            wires = blk @ builder[wires]
        builder.add_outputs(wires)
        diagram = builder.diagram()
        diagram._seq_blocks = tuple(blocks)
        return diagram


class DiagramBuilder:
    """Utility class to build diagrams (``tensorsat/diagrams.py:1647-1870``)."""

    __slots__ = ("_wiring", "_blocks")

    def __init__(self) -> None:
        self._wiring = WiringBuilder()
        self._blocks: dict[Slot, Block] = {}

    @property
    def wiring(self) -> WiringBuilder:
        return self._wiring

    @property
    def blocks(self) -> Mapping[Slot, Block]:
        return MappingProxyType(self._blocks)

    def diagram(self) -> Diagram:
        w = self._wiring.wiring
        return Diagram._new(w, tuple(self._blocks.get(s) for s in w.slots))

    def add_block(self, block: Block, inputs: Mapping[Port, Wire] = MappingProxyType({})) -> Wires:
        """Adds a slot holding ``block``; ports in ``inputs`` connect to the given wires,
        every other port gets a new wire (in port order), which is returned."""
        types = self._wiring._wire_types
        shape = block.shape
        for port, wire in inputs.items():
            if port not in range(len(shape)):
                raise ValueError(f"Invalid port {port} for block.")
            if wire not in range(len(types)):
                raise ValueError(f"Invalid wire index {wire}.")
            if shape[port] != types[wire]:
                raise ValueError(
                    f"Incompatible wire type for port {port}:"
                    f" port has type {shape[port]}, wire has type {types[wire]}."
                )
        out_ports = tuple(p for p in block.ports if p not in inputs)
        new_wires = self._wiring.add_wires([shape[p] for p in out_ports])
        mapping = {**inputs, **dict(zip(out_ports, new_wires))}
        slot = self._wiring.add_slot()
        self._wiring.add_slot_ports(slot, [mapping[p] for p in block.ports])
        self._blocks[slot] = block
        return new_wires

    def add_input(self, t: Type) -> Wire:
        return self.add_inputs((t,))[0]

    def add_inputs(self, ts: Iterable[Type]) -> Wires:
        wires = self._wiring.add_wires(list(ts))
        self._wiring.add_out_ports(wires)
        return wires

    def add_output(self, wire: Wire) -> Port:
        return self.add_outputs((wire,))[0]

    def add_outputs(self, wires: Iterable[Wire]) -> Ports:
        wires = tuple(wires)
        for w in wires:
            if w not in self._wiring.wires:
                raise ValueError(f"Invalid wire index {w}.")
        return self._wiring.add_out_ports(wires)

    def __getitem__(self, wires: Wire | Sequence[Wire]) -> "SelectedBuilderWires":
        return SelectedBuilderWires(self, wires)

    def __rmatmul__(self, block: Block) -> Wires:
        return self.add_block(block)


class SelectedBuilderWires:
    """Selected wires of a builder; ``block @ builder[wires]`` adds the block."""

    __slots__ = ("builder", "wires")

    def __init__(self, builder: DiagramBuilder, wires: Wire | Sequence[Wire]) -> None:
        if isinstance(wires, int):
            wires = (wires,)
        wires = tuple(wires)
        for w in wires:
            if w not in builder.wiring.wires:
                raise ValueError(f"Invalid wire {w} selected for {builder}")
        self.builder = builder
        self.wires = wires

    def __rmatmul__(self, other: Any) -> Wires:
        wires = self.wires
        if isinstance(other, (Box, Diagram)):
            if len(other.ports) < len(wires):
                raise ValueError(
                    f"Cannot apply block: {len(wires)} wires selected,"
                    f" {other.num_ports} ports available on RHS."
                )
            other = SelectedBlockPorts(other, range(len(wires)))
        elif not isinstance(other, SelectedBlockPorts):
            return NotImplemented
        elif len(other.ports) != len(wires):
            raise ValueError(
                f"Cannot apply block: {len(wires)} wires selected,"
                f" {len(other.ports)} ports selected on block."
            )
        return self.builder.add_block(other.block, dict(zip(other.ports, wires)))
