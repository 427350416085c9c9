"""Backend functions for ``autoray`` dispatch on boxes (``tensorsat/_autoray.py:29-83``).

``einsum("ab,bc->ac", lhs, rhs)`` parses the equation into wire lists and calls
``contract2`` of the boxes' class join, exactly like the reference shim through which
cotengra's ``tree.contract`` reaches ``FinRel._contract2``. The single-operand form,
which the reference leaves unimplemented (``_autoray.py:41-50``), contracts against the
scalar box ``True``. When ``autoray`` is installed, :func:`register` makes these the
``"tensorsat_gb300._autoray"`` backend of the box classes.
"""

from __future__ import annotations

from collections.abc import Sequence

from .diagrams import Box, TensorLikeBox


def _wire_ids(*terms: str) -> dict[str, int]:
    ids: dict[str, int] = {}
    for term in terms:
        for c in term:
            ids.setdefault(c, len(ids))
    return ids


def einsum(contraction: str, /, lhs: Box, rhs: Box | None = None) -> Box:
    """Contracts one or two boxes given in einsum notation."""
    inputs, out = contraction.replace(" ", "").split("->")
    if rhs is None:
        (lhs_term,) = inputs.split(",")
        ids = _wire_ids(lhs_term, out)
        cls = type(lhs)
        one = cls.scalar(True)
        return cls.contract2(lhs, [ids[c] for c in lhs_term], one, [], [ids[c] for c in out])
    lhs_term, rhs_term = inputs.split(",")
    ids = _wire_ids(lhs_term, rhs_term, out)
    cls = Box.class_join([type(lhs), type(rhs)])
    return cls.contract2(
        lhs, [ids[c] for c in lhs_term], rhs, [ids[c] for c in rhs_term], [ids[c] for c in out]
    )


def transpose(box: Box, perm: Sequence[int], /) -> Box:
    """Rearranges the ports of a box."""
    return box.rewire(perm)


def shape(box: TensorLikeBox) -> tuple[int, ...]:
    if not isinstance(box, TensorLikeBox):
        raise TypeError("Autoray shape is only supported by tensor-like boxes.")
    return box.tensor_shape


def stack(boxes: Sequence[Box], axis: int = 0) -> Box:
    """Stacks boxes along a new axis."""
    cls = Box.class_join([type(b) for b in boxes])
    return cls.stack(boxes, axis)


def register(box_class: type) -> bool:
    """Registers ``box_class`` with autoray (when installed); returns whether it did."""
    try:
        import autoray  # type: ignore[import-not-found]
    except ModuleNotFoundError:
        return False
    autoray.register_backend(box_class, "tensorsat_gb300._autoray")
    return True
