"""Reference-side binding: a tensorsat box class backed by the tensorsat_gb300 C ABI.

:func:`make_finrel_cuda` defines, inside an installed ``tensorsat`` package, the box class
a tensorsat maintainer would add next to ``FinRel`` (``tensorsat/lang/fin_rel.py:162``):
a ``@final`` subclass of ``tensorsat.diagrams.TensorLikeBox`` whose protected plugin
methods call ``libtensorsat_gb300.so`` through ctypes. Because ``BoxMeta`` registers every
concrete box class with autoray (``tensorsat/diagrams.py:675-690``), cotengra's
``tree.contract`` then reaches ``tsg_contract2_or_and`` through
``tensorsat/_autoray.py:31-62`` with no further change to the reference.

Only this module touches the upstream package; the rest of tensorsat_gb300 is standalone.
"""

from __future__ import annotations

from typing import Any


def make_finrel_cuda(tensorsat_module: Any | None = None) -> type:
    """Creates the ``FinRelCuda`` box class against the given (or importable) tensorsat.

    Upstream boxes must be declared with ``typing.final`` and without public annotations
    (``tensorsat/_utils/meta.py:336-397``); the class below follows those rules.
    """
    from typing import final

    import numpy as np
    import torch

    from . import _device, _native

    if tensorsat_module is None:
        import tensorsat as tensorsat_module  # noqa: F401
    from tensorsat.diagrams import TensorLikeBox  # type: ignore[import-not-found]
    from tensorsat.lang.fin_rel import FinRel, FinSet  # type: ignore[import-not-found]

    def _dev(t: Any) -> torch.Tensor:
        if isinstance(t, np.ndarray):
            # np.array keeps 0-d scalars 0-d (np.ascontiguousarray would make them 1-d)
            t = torch.from_numpy(np.array(t, dtype=np.uint8, order="C", copy=True))
        return _device.to_device_u8(t)

    @final
    class FinRelCuda(TensorLikeBox):
        """FinRel with its Boolean tensor in GPU memory; every operation runs in the
        tensorsat_gb300 CUDA library."""

        __tensor: Any  # private annotation: the upstream metaclass turns it into a slot

        @classmethod
        def _new(cls, tensor: torch.Tensor) -> "FinRelCuda":
            self = super().__new__(cls)
            self._FinRelCuda__tensor = tensor
            return self

        @classmethod
        def from_finrel(cls, rel: Any) -> "FinRelCuda":
            return cls._new(_dev(np.asarray(rel.tensor)))

        @classmethod
        def from_array(cls, array: Any) -> "FinRelCuda":
            """The relation whose {0,1} tensor is ``array`` (copied to the device)."""
            return cls._new(_dev(np.asarray(array)))

        def to_finrel(self) -> Any:
            return FinRel._new(self._FinRelCuda__tensor.cpu().numpy())

        @property
        def shape(self) -> tuple:
            return tuple(FinSet(d) for d in self._FinRelCuda__tensor.shape)

        @classmethod
        def _contract2(cls, lhs, lhs_wires, rhs, rhs_wires, out_wires):
            lt, rt = lhs._FinRelCuda__tensor, rhs._FinRelCuda__tensor
            lw, rw, ow = list(lhs_wires), list(rhs_wires), list(out_wires)
            dims = dict(zip(lw, lt.shape))
            dims.update(zip(rw, rt.shape))
            out = torch.empty([dims[w] for w in ow], dtype=torch.uint8, device=lt.device)
            _native.check(_native.lib().tsg_contract2_or_and(
                lt.data_ptr(), len(lw), _native.i64_array(lw), _native.i64_array(lt.shape),
                rt.data_ptr(), len(rw), _native.i64_array(rw), _native.i64_array(rt.shape),
                len(ow), _native.i64_array(ow), out.data_ptr(), _device.stream_handle()))
            return cls._new(out)

        @classmethod
        def _spider(cls, t, num_ports):
            out = torch.empty((t.tensor_dim,) * num_ports, dtype=torch.uint8,
                              device=_device.require_cuda())
            _native.check(_native.lib().tsg_spider_fill(out.data_ptr(), t.tensor_dim,
                                                        num_ports, _device.stream_handle()))
            return cls._new(out)

        @classmethod
        def _scalar(cls, scalar):
            return cls._new(_dev(np.array(int(bool(scalar)), dtype=np.uint8)))

        @classmethod
        def _stack(cls, boxes, port=0):
            return cls._new(torch.stack([b._FinRelCuda__tensor for b in boxes], dim=port))

        def _getitem(self, idxs):
            return FinRelCuda._new(self._FinRelCuda__tensor[idxs].contiguous())

        def _union(self, other):
            a, b = self._FinRelCuda__tensor, other._FinRelCuda__tensor
            out = torch.empty_like(a)
            _native.check(_native.lib().tsg_union_or(a.data_ptr(), b.data_ptr(),
                                                     out.data_ptr(), a.numel(),
                                                     _device.stream_handle()))
            return FinRelCuda._new(out)

        def _rewire(self, out_ports):
            t = self._FinRelCuda__tensor
            ports = list(out_ports)
            out = torch.empty([t.shape[p] for p in ports], dtype=torch.uint8, device=t.device)
            _native.check(_native.lib().tsg_rewire_or_and(
                t.data_ptr(), t.ndim, _native.i64_array(t.shape), len(ports),
                _native.i32_array(ports), out.data_ptr(), _device.stream_handle()))
            return FinRelCuda._new(out)

        def _as_scalar(self):
            return int(self._FinRelCuda__tensor.reshape(()).item()) == 1

    return FinRelCuda
