"""The device box class: finite relations as Boolean tensors held in GPU memory.

:class:`CudaRel` is the GB300 counterpart of ``FinRel`` (``tensorsat/lang/fin_rel.py:
162-493``): same constructors, same protected plugin methods, same semantics, with the
tensor held by PyTorch on the device and every operation executed by the native library
(``include/tensorsat_gb300.h``):

* ``_contract2`` -> ``tsg_contract2_or_and`` (``FinRel._contract2``, ``fin_rel.py:255-288``)
* ``_rewire``    -> ``tsg_rewire_or_and``    (``FinRel._rewire``, ``fin_rel.py:379-393``)
* ``_union``     -> ``tsg_union_or``         (``FinRel._union``, ``fin_rel.py:345-346``)
* ``_spider``    -> ``tsg_spider_fill``      (``FinRel._spider``, ``fin_rel.py:290-298``)

Constructors build small host tensors (gates, constants) without touching the GPU; the
first device operation moves them to the current CUDA device. Boxes are immutable, like
``FinRel`` (``fin_rel.py:310-326``): a box owns its tensor and never writes to it.
"""

from __future__ import annotations

from collections.abc import Callable, Iterable, Mapping, Sequence
from math import prod
from typing import Any, TypeAlias

import numpy as np
import torch

from .. import _device, _native
from ..diagrams import Port, TensorLikeBox, TensorLikeType, Type, Wire

Size: TypeAlias = int
El: TypeAlias = int
Point: TypeAlias = tuple[El, ...]


class FinSet(TensorLikeType):
    """The finite set ``{0, ..., size-1}``; one instance per size (``fin_rel.py:75-118``)."""

    __slots__ = ("_size",)
    _instances: dict[int, "FinSet"] = {}

    def __new__(cls, size: int) -> "FinSet":
        if not isinstance(size, (int, np.integer)):
            raise TypeError("Finite set size must be an integer.")
        size = int(size)
        if size <= 0:
            raise ValueError("Finite set size must be strictly positive.")
        inst = cls._instances.get(size)
        if inst is None:
            inst = super().__new__(cls)
            inst._size = size
            cls._instances[size] = inst
        return inst

    @property
    def size(self) -> Size:
        return self._size

    @property
    def tensor_dim(self) -> Size:
        return self._size

    def __repr__(self) -> str:
        return f"FinSet({self._size})"


def _extract_sizes(s: Any) -> tuple[Size, ...]:
    if isinstance(s, (int, np.integer)):
        return (int(s),)
    if isinstance(s, FinSet):
        return (s.size,)
    return tuple(int(x) if isinstance(x, (int, np.integer)) else x.tensor_dim for x in s)


def _wrap_el(x: El | Point) -> Point:
    return (int(x),) if isinstance(x, (int, np.integer)) else tuple(x)


class CudaRel(TensorLikeBox):
    """A finite relation, densely represented by a uint8 {0,1} tensor on the GPU."""

    __slots__ = ("_tensor", "_dev", "_hash")

    # -- constructors (host side, mirroring FinRel's) --------------------------------

    @classmethod
    def from_set(cls, shape: Any, points: Iterable[El | Point], *, name: str | None = None
                 ) -> "CudaRel":
        shape = _extract_sizes(shape)
        if any(d <= 0 for d in shape):
            raise ValueError("Zero dimension in shape.")
        data = np.zeros(shape, dtype=np.uint8)
        for point in points:
            point = _wrap_el(point)
            if len(point) != len(shape):
                raise ValueError(f"Length of {point = } is invalid for {shape = }.")
            if not all(0 <= i < d for i, d in zip(point, shape)):
                raise ValueError(f"Values of {point = } are invalid for {shape = }.")
            data[point] = 1
        return cls._new(torch.from_numpy(data), name)

    @classmethod
    def from_mapping(cls, input_shape: Any, output_shape: Any,
                     mapping: Mapping[Point, El | Point], *, name: str | None = None
                     ) -> "CudaRel":
        input_shape = _extract_sizes(input_shape)
        output_shape = _extract_sizes(output_shape)
        rel = cls.from_set(input_shape + output_shape,
                           (tuple(k) + _wrap_el(v) for k, v in mapping.items()), name=name)
        if len(mapping) != prod(input_shape):
            raise ValueError("Mapping does not cover the entire input space.")
        return rel

    @classmethod
    def singleton(cls, shape: Any, point: El | Point, *, name: str | None = None) -> "CudaRel":
        return cls.from_mapping((), shape, {(): point}, name=name)

    @classmethod
    def from_callable(cls, input_shape: Any, output_shape: Any, func: Callable[..., El | Point],
                      *, name: str | None = None) -> "CudaRel":
        input_shape = _extract_sizes(input_shape)
        output_shape = _extract_sizes(output_shape)
        mapping = {idx: func(*idx) for idx in np.ndindex(input_shape)}
        return cls.from_mapping(input_shape, output_shape, mapping, name=name)

    @classmethod
    def _new(cls, tensor: torch.Tensor, name: str | None = None) -> "CudaRel":
        self = object.__new__(cls)
        TensorLikeBox.__init__(self, name)
        self._tensor = tensor
        self._dev = tensor if tensor.device.type == "cuda" else None
        return self

    def __init__(self, *args: Any, **kwargs: Any) -> None:
        """Initialisation happens in :meth:`_new` (called by ``__new__``)."""

    def __new__(cls, tensor: Any = None, *args: Any, **kwargs: Any) -> "CudaRel":
        """Constructs a relation from a Boolean tensor (numpy or torch, values 0/1)."""
        if isinstance(tensor, np.ndarray):
            t = torch.from_numpy(np.require(tensor, requirements="C"))  # keeps 0-d arrays 0-d
        elif isinstance(tensor, torch.Tensor):
            t = tensor
        else:
            raise TypeError("CudaRel expects a numpy array or a torch tensor.")
        if t.dtype != torch.uint8:
            raise TypeError("Boolean tensors must have dtype uint8.")
        if t.numel() and int(t.max()) > 1:
            raise ValueError("Values in a Boolean tensor must be 0 or 1.")
        return cls._new(t.contiguous())

    # -- data ---------------------------------------------------------------------------

    @property
    def tensor(self) -> torch.Tensor:
        """The Boolean tensor (device tensor once the box has been used on the GPU)."""
        return self._dev if self._dev is not None else self._tensor

    def device_tensor(self) -> torch.Tensor:
        """The tensor on the current CUDA device (uploaded once, then cached)."""
        if self._dev is None:
            self._dev = _device.to_device_u8(self._tensor)
        return self._dev

    def numpy(self) -> np.ndarray:
        """Host copy of the tensor."""
        return self.tensor.detach().cpu().numpy()

    @property
    def shape(self) -> tuple[FinSet, ...]:
        return tuple(FinSet(d) for d in self._tensor.shape)

    # -- plugin methods (device) -----------------------------------------------------

    @classmethod
    def _contract2(cls, lhs: "CudaRel", lhs_wires: Sequence[Wire], rhs: "CudaRel",
                   rhs_wires: Sequence[Wire], out_wires: Sequence[Wire]) -> "CudaRel":
        lib = _native.lib()
        lt, rt = lhs.device_tensor(), rhs.device_tensor()
        lw, rw, ow = list(lhs_wires), list(rhs_wires), list(out_wires)
        ld, rd = list(lt.shape), list(rt.shape)
        dims = dict(zip(lw, ld))
        dims.update(zip(rw, rd))
        out_shape = [dims[w] for w in ow]
        out = torch.empty(out_shape, dtype=torch.uint8, device=lt.device)
        st = lib.tsg_contract2_or_and(
            lt.data_ptr(), len(lw), _native.i64_array(lw), _native.i64_array(ld),
            rt.data_ptr(), len(rw), _native.i64_array(rw), _native.i64_array(rd),
            len(ow), _native.i64_array(ow), out.data_ptr(), _device.stream_handle(),
        )
        _native.check(st)
        return cls._new(out)

    @classmethod
    def _spider(cls, t: Type, num_ports: int) -> "CudaRel":
        assert isinstance(t, FinSet)
        dev = _device.require_cuda()
        out = torch.empty((t.size,) * num_ports, dtype=torch.uint8, device=dev)
        _native.check(_native.lib().tsg_spider_fill(out.data_ptr(), t.size, num_ports,
                                                    _device.stream_handle()))
        return cls._new(out)

    @classmethod
    def _scalar(cls, scalar: bool, /) -> "CudaRel":
        return cls._new(torch.tensor(int(bool(scalar)), dtype=torch.uint8))

    @classmethod
    def _stack(cls, boxes: tuple["CudaRel", ...], port: int = 0, /) -> "CudaRel":
        return cls._new(torch.stack([b.device_tensor() for b in boxes], dim=port).contiguous())

    def _getitem(self, idxs: tuple[int | slice, ...]) -> "CudaRel":
        return CudaRel._new(self.device_tensor()[idxs].contiguous())

    def _union(self, other: "CudaRel") -> "CudaRel":
        a, b = self.device_tensor(), other.device_tensor()
        out = torch.empty_like(a)
        _native.check(_native.lib().tsg_union_or(a.data_ptr(), b.data_ptr(), out.data_ptr(),
                                                 a.numel(), _device.stream_handle()))
        return CudaRel._new(out)

    def _rewire(self, out_ports: Sequence[Port]) -> "CudaRel":
        t = self.device_tensor()
        ports = list(out_ports)
        dims = list(t.shape)
        out = torch.empty([dims[p] for p in ports], dtype=torch.uint8, device=t.device)
        _native.check(_native.lib().tsg_rewire_or_and(
            t.data_ptr(), len(dims), _native.i64_array(dims), len(ports),
            _native.i32_array(ports), out.data_ptr(), _device.stream_handle()))
        return CudaRel._new(out)

    def _as_scalar(self) -> bool:
        return bool(int(self.tensor.reshape(()).item()) == 1)

    # -- relation utilities (host readouts) -------------------------------------------

    def to_set(self) -> frozenset[Point]:
        """The set of points of the relation (inverse of :meth:`from_set`)."""
        arr = self.numpy()
        return frozenset(tuple(int(i) for i in idx) for idx in zip(*np.nonzero(arr)))

    def __eq__(self, other: Any) -> bool:
        if not isinstance(other, CudaRel):
            return NotImplemented
        if self is other:
            return True
        return np.array_equal(self.numpy(), other.numpy())

    def __hash__(self) -> int:
        try:
            return self._hash
        except AttributeError:
            self._hash = hash((tuple(self._tensor.shape), self.numpy().tobytes()))
            return self._hash


def leaf_array(box: Any) -> np.ndarray:
    """Host uint8 tensor of a CudaRel (or of any box exposing a numpy ``tensor``)."""
    if isinstance(box, CudaRel):
        return box.numpy()
    t = getattr(box, "tensor", None)
    if isinstance(t, np.ndarray):
        return t.astype(np.uint8, copy=False)
    raise TypeError(f"cannot read the tensor of {box!r}")
