"""Boxes for binary circuits: the gate tensors of a CNF network.

Same names and truth tables as ``tensorsat/lib/bincirc.py:28-88`` (the relations are the
gates' function graphs), built as :class:`~tensorsat_gb300.lang.cuda_rel.CudaRel` boxes.
Their tensors stay on the host until a contraction first uses them.
"""

from __future__ import annotations

from types import MappingProxyType
from typing import Final, Mapping

from ..lang.cuda_rel import CudaRel, FinSet

bit: Final[FinSet] = FinSet(2)
"""The set {0, 1} of binary values."""


def bits(n: int) -> tuple[FinSet, ...]:
    """Shape consisting of the given number of bits."""
    if n < 0:
        raise ValueError("Number of bits must be non-negative.")
    return (bit,) * n


bits2: Final[tuple[FinSet, ...]] = bits(2)

not_: Final[CudaRel] = CudaRel.from_callable(bit, bit, lambda b: 1 - b, name="not_")
and_: Final[CudaRel] = CudaRel.from_callable(bits2, bit, lambda a, b: a & b, name="and_")
or_: Final[CudaRel] = CudaRel.from_callable(bits2, bit, lambda a, b: a | b, name="or_")
impl_: Final[CudaRel] = CudaRel.from_callable(bits2, bit, lambda a, b: (1 - a) | b, name="impl_")
biimpl_: Final[CudaRel] = CudaRel.from_callable(
    bits2, bit, lambda a, b: (a & b) | ((1 - a) & (1 - b)), name="biimpl_"
)
xor_: Final[CudaRel] = CudaRel.from_callable(bits2, bit, lambda a, b: a ^ b, name="xor_")
bit_0: Final[CudaRel] = CudaRel.singleton(bit, 0, name="bit_0")
bit_1: Final[CudaRel] = CudaRel.singleton(bit, 1, name="bit_1")
bit_unk: Final[CudaRel] = CudaRel.from_set(bit, {0, 1}, name="bit_unk")

binop_labels: Final[Mapping[CudaRel, str]] = MappingProxyType(
    {not_: "~", and_: "&", or_: "|", xor_: "^", impl_: "=>", biimpl_: "=", bit_0: "0",
     bit_1: "1", bit_unk: "?"}
)
