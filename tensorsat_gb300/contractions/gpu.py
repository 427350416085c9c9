"""Tree-executor contractions on the GPU: the drop-in for ``CotengraContraction``.

:class:`GpuContraction` plays the role of ``CotengraContraction``
(``tensorsat/contractions/cotengra.py:51-131``): it is built once for a box class and a
wiring (planning a contraction tree with the project's own optimiser,
:mod:`tensorsat_gb300.planner`, in place of ``ctg.array_contract_tree``), exposes the tree
and its pop/append ``path``, and ``contract(diagram)`` returns the contracted box. Where
cotengra runs one einsum per tree node through ``tensorsat/_autoray.py:31-62``, this class
hands the whole tree to the native executor (``tsg_plan_run``): every node is a device
kernel and sliced wires run as batched groups of slices.

Beyond the reference, :meth:`GpuContraction.count` returns the exact model count: the same
tree contracted over the integers, either modulo 2^64 (exact when the count bound is below
2^64) or modulo up to four 31-bit primes recombined by the Chinese remainder theorem.
"""

from __future__ import annotations

import hashlib
import json
import math
import os
from dataclasses import dataclass
from pathlib import Path
from typing import Any, Sequence

import numpy as np
import torch

from .. import _device, _native, planner, sharding
from ..diagrams import Diagram, TensorLikeType, Wiring
from ..lang.cuda_rel import CudaRel, leaf_array
from .abc import Contraction

def _is_prime(n: int) -> bool:
    """Deterministic Miller-Rabin for n < 3.3e9 (bases 2, 3, 5, 7)."""
    if n < 2:
        return False
    for q in (2, 3, 5, 7):
        if n % q == 0:
            return n == q
    d, r = n - 1, 0
    while d % 2 == 0:
        d //= 2
        r += 1
    for a in (2, 3, 5, 7):
        x = pow(a, d, n)
        if x in (1, n - 1):
            continue
        for _ in range(r - 1):
            x = x * x % n
            if x == n - 1:
                break
        else:
            return False
    return True


def _primes_below(limit: int, count: int) -> tuple[int, ...]:
    out = []
    n = limit - 1
    while len(out) < count:
        if _is_prime(n):
            out.append(n)
        n -= 2 if n % 2 else 1
    return tuple(out)


PRIMES_31 = _primes_below(2**31, 64)
"""Moduli of the residue count ring: the largest primes below 2^31, in decreasing order
(2147483647, 2147483629, 2147483587, ...). A run carries at most 4 of them; counts that
need more run several passes."""

DEFAULT_TARGET_BITS = 26


@dataclass
class _Leaves:
    """How the wiring's slots become bit-network leaves."""

    leaf_wires: list[tuple[int, ...]]
    slot_of_leaf: list[int | None]
    synthetic: list[np.ndarray | None]
    diag_slots: frozenset[int]
    discard_factor: int
    out_unique: tuple[int, ...]
    wire_dims: dict[int, int]


def _prepare(wiring: Wiring) -> _Leaves:
    dims = {w: t.tensor_dim for w, t in enumerate(wiring.wire_types)}
    leaf_wires: list[tuple[int, ...]] = []
    slot_of_leaf: list[int | None] = []
    synthetic: list[np.ndarray | None] = []
    diag = set()
    for s, ws in enumerate(wiring.slot_wires_list):
        uniq = tuple(dict.fromkeys(ws))
        if len(uniq) != len(ws):
            diag.add(s)
        leaf_wires.append(uniq)
        slot_of_leaf.append(s)
        synthetic.append(None)
    out_set = set(wiring.out_wires)
    factor = 1
    for w in sorted(wiring.dangling_wires):
        if w in out_set:
            leaf_wires.append((w,))
            slot_of_leaf.append(None)
            synthetic.append(np.ones(dims[w], dtype=np.uint8))
        else:
            factor *= dims[w]
    while len(leaf_wires) < 2:
        leaf_wires.append(())
        slot_of_leaf.append(None)
        synthetic.append(np.ones((), dtype=np.uint8))
    return _Leaves(leaf_wires, slot_of_leaf, synthetic, frozenset(diag), factor,
                   tuple(dict.fromkeys(wiring.out_wires)), dims)


def _network(lw: _Leaves) -> planner.Network:
    """The bit network the planner sees (one tensor per prepared leaf)."""
    if any(d != 2 for w, d in lw.wire_dims.items()
           if any(w in ws for ws in lw.leaf_wires) or w in lw.out_unique):
        raise NotImplementedError(
            "GpuContraction executes bit networks: every connected wire must have"
            " dimension 2"
        )
    return planner.Network(lw.leaf_wires, {w: 2 for ws in lw.leaf_wires for w in ws},
                           lw.out_unique)


def plan_tree(wiring: Wiring, target_bits: int | None = 26, trials: int = 8,
              seed: int = 0) -> tuple[planner.ContractionTree, tuple[int, ...]]:
    """The (tree, sliced wires) that ``GpuContraction(box_class, wiring,
    target_bits=..., trials=..., seed=...)`` plans (``target_bits=None``: no slicing),
    computed without building the contraction (host only, so planning can run in worker
    processes and the result can be passed back as ``tree=`` / ``sliced=``)."""
    tree, sl = planner.optimize(_network(_prepare(wiring)), target_bits=target_bits,
                                trials=trials, seed=seed)
    return tree, tuple(sorted(sl))


_CHECKPOINT_FORMAT = "tensorsat_gb300.count_checkpoint/2"


def _write_json(path: Path, data: dict) -> None:
    tmp = path.with_name(path.name + ".tmp")
    tmp.write_text(json.dumps(data))
    os.replace(tmp, path)


def _functional_ports(t: np.ndarray) -> list[int]:
    """Ports whose value is a function of the other ports (exactly one 1 per assignment of
    the others), last port first (gates put their output last)."""
    if t.ndim == 0 or t.size > 1 << 12:
        return []
    return [p for p in reversed(range(t.ndim)) if np.all(t.sum(axis=p) == 1)]


def count_bound_bits(wiring: Wiring, arrays: Sequence[np.ndarray]) -> float:
    """log2 of an upper bound on every entry of the count tensor of a 0/1 network.

    A wire that one tensor determines from its other wires (a gate output, a constant)
    adds nothing, provided the determinations are acyclic: then every assignment of the
    remaining summed wires extends in at most one way. Every other summed wire adds
    log2(dim). Wires are oriented greedily (a gate's last port first) and the orientation
    is dropped altogether if it is cyclic."""
    determined: dict[int, tuple[int, ...]] = {}
    for ws, arr in zip(wiring.slot_wires_list, arrays):
        if len(set(ws)) != len(ws):
            continue
        for p in _functional_ports(np.asarray(arr)):
            if ws[p] not in determined:
                determined[ws[p]] = tuple(w for w in ws if w != ws[p])
                break
    # acyclicity: Kahn's algorithm over "determined wire <- its tensor's other wires"
    indeg = {w: sum(1 for u in deps if u in determined) for w, deps in determined.items()}
    users: dict[int, list[int]] = {}
    for w, deps in determined.items():
        for u in deps:
            if u in determined:
                users.setdefault(u, []).append(w)
    queue = [w for w, d in indeg.items() if d == 0]
    seen = 0
    while queue:
        u = queue.pop()
        seen += 1
        for w in users.get(u, ()):
            indeg[w] -= 1
            if indeg[w] == 0:
                queue.append(w)
    if seen != len(determined):
        determined = {}
    out = set(wiring.out_wires)
    bits = 0.0
    for w, t in enumerate(wiring.wire_types):
        if w in out or w in determined:
            continue
        bits += math.log2(t.tensor_dim)
    return bits


def crt(residues: Sequence[np.ndarray], moduli: Sequence[int]) -> np.ndarray:
    """Chinese remaindering of per-prime residue arrays into Python integers."""
    M = 1
    for p in moduli:
        M *= p
    shape = residues[0].shape
    flat = [r.reshape(-1) for r in residues]
    out = np.empty(flat[0].shape[0], dtype=object)
    coeffs = []
    for p in moduli:
        Mi = M // p
        coeffs.append(Mi * pow(Mi, -1, p))
    for i in range(out.shape[0]):
        out[i] = sum(int(r[i]) * c for r, c in zip(flat, coeffs)) % M
    return out.reshape(shape)


class NativePlan:
    """Owner of a ``tsg_plan`` handle built from a :class:`planner.SlicedPlan`."""

    def __init__(self, plan: planner.SlicedPlan) -> None:
        lib = _native.lib()
        arrs = plan.native_arrays()
        ranks = arrs["leaf_ranks"]
        sizes = [1 << int(r) for r in ranks]
        offsets = np.zeros(len(sizes), dtype=np.int64)
        off = 0
        for i, n in enumerate(sizes):
            offsets[i] = off
            off += (n + 15) // 16 * 16
        self.leaf_offsets = offsets
        self.leaf_sizes = sizes
        self.pool_bytes = max(off, 16)
        self.num_sliced = len(plan.sliced)
        self.num_steps = len(plan.tree.steps)
        self._arrs = arrs
        handle = _native.c_void_p()
        lsp = np.ascontiguousarray(arrs["leaf_slice_pos"], dtype=np.int32)
        st = lib.tsg_plan_create(
            len(ranks), _native.ptr_i32(ranks), _native.ptr_i64(offsets), self.num_sliced,
            _native.ptr_i32(lsp), len(arrs["step_out_bits"]),
            _native.ptr_i32(np.ascontiguousarray(arrs["step_operands"])),
            _native.ptr_i32(arrs["step_out_bits"]), _native.ptr_i32(arrs["step_sum_bits"]),
            _native.ptr_i32(arrs["step_lhs_pos"]), _native.ptr_i32(arrs["step_rhs_pos"]),
            _native.ctypes.byref(handle),
        )
        _native.check(st)
        self.handle = handle
        self._lib = lib

    def workspace_bytes(self, ring: int, num_primes: int, group: int) -> int:
        out = _native.c_int64()
        _native.check(self._lib.tsg_plan_workspace_bytes(self.handle, ring, num_primes, group,
                                                         _native.ctypes.byref(out)))
        return int(out.value)

    def launch_count(self, begin: int, end: int, group: int, ring: int | None = None,
                     num_primes: int = 1) -> int:
        """Kernel launches of one run over slices [begin, end); with ``ring`` the exact
        count for that ring (fused steps launch nothing), else every step's launch."""
        out = _native.c_int64()
        if ring is None:
            _native.check(self._lib.tsg_plan_launch_count(self.handle, begin, end, group,
                                                          _native.ctypes.byref(out)))
        else:
            _native.check(self._lib.tsg_plan_launches(self.handle, ring, num_primes, begin,
                                                      end, group, _native.ctypes.byref(out)))
        return int(out.value)

    def fused_steps(self, ring: int, primes: Sequence[int], group: int,
                    tree: planner.ContractionTree) -> dict[int, int]:
        """{consumer step: producer step} of the steps a run in ``ring`` fuses (the
        producer is computed inside its consumer and never stored)."""
        kinds = self.describe(ring, primes, group)
        L = tree.num_leaves
        out = {}
        for s, k in enumerate(kinds):
            if int(k[0]) != _native.TSG_KERNEL_FUSED:
                continue
            for x in tree.steps[s]:
                if x >= L and int(kinds[x - L][0]) == _native.TSG_KERNEL_NONE:
                    out[s] = x - L
        return out

    def describe(self, ring: int, primes: Sequence[int], group: int) -> np.ndarray:
        """(steps, 4) int32: per tree step the kernel family (``TSG_KERNEL_*``) and its
        template parameters V, NE, NK, as ``tsg_plan_run`` would launch them for a slice
        group of ``group`` (host only, no GPU needed)."""
        parr = (_native.c_uint32 * max(1, len(primes)))(*primes)
        out = np.zeros((self.num_steps, 4), dtype=np.int32)
        _native.check(self._lib.tsg_plan_describe(self.handle, ring, len(primes), parr, group,
                                                  _native.ptr_i32(out)))
        return out

    def validate(self, ring: int, primes: Sequence[int], begin: int, end: int, group: int) -> None:
        """Host-side bounds check of every launch (no GPU needed)."""
        parr = (_native.c_uint32 * max(1, len(primes)))(*primes)
        _native.check(self._lib.tsg_plan_validate(self.handle, ring, len(primes), parr, begin,
                                                  end, group))

    def run(self, ring: int, primes: Sequence[int], pool: torch.Tensor, begin: int, end: int,
            group: int, workspace: torch.Tensor, result: torch.Tensor, accumulate: bool,
            stream: int) -> None:
        parr = (_native.c_uint32 * max(1, len(primes)))(*primes)
        st = self._lib.tsg_plan_run(
            self.handle, ring, len(primes), parr, pool.data_ptr(), begin, end, group,
            workspace.data_ptr(), workspace.numel(), result.data_ptr(), int(bool(accumulate)),
            stream,
        )
        _native.check(st)

    def run_timed(self, ring: int, primes: Sequence[int], pool: torch.Tensor, begin: int,
                  end: int, group: int, workspace: torch.Tensor, result: torch.Tensor,
                  accumulate: bool, stream: int) -> list[float]:
        """:meth:`run` with CUDA events around every launch; waits for the run and returns
        the device milliseconds of each tree step (summed over slice groups), followed by
        those of the root reductions."""
        parr = (_native.c_uint32 * max(1, len(primes)))(*primes)
        n = len(self._arrs["step_out_bits"])
        ms = (_native.ctypes.c_float * (n + 1))()
        st = self._lib.tsg_plan_run_timed(
            self.handle, ring, len(primes), parr, pool.data_ptr(), begin, end, group,
            workspace.data_ptr(), workspace.numel(), result.data_ptr(), int(bool(accumulate)),
            stream, ms,
        )
        _native.check(st)
        return list(ms)

    def __del__(self) -> None:
        h = getattr(self, "handle", None)
        if h is not None and h.value:
            try:
                self._lib.tsg_plan_destroy(h)
            except Exception:  # pragma: no cover - interpreter shutdown
                pass
            self.handle = None


class GpuContraction(Contraction):
    """Contraction of bit networks (all wires of dimension 2) by the GPU tree executor.

    :param optimize: accepted for signature parity with ``CotengraContraction``; every
        value selects the project's min-fill tree search (``"greedy"``, ``"auto"``, ...).
    :param target_bits: slice until every intermediate has at most ``2**target_bits``
        entries (``None``: never slice).
    :param trials: randomized elimination orders tried; the cheapest tree is kept.
    :param tree, sliced: use this tree (and sliced wires) instead of searching.
    """

    def __init__(
        self,
        box_class: type,
        wiring: Wiring,
        *,
        optimize: Any = "auto",
        target_bits: int | None = DEFAULT_TARGET_BITS,
        trials: int = 8,
        seed: int = 0,
        tree: planner.ContractionTree | None = None,
        sliced: Sequence[int] | None = None,
        canonicalize: bool = True,
        sort_contraction_indices: bool = False,
    ) -> None:
        super().__init__(box_class, wiring)
        if wiring.num_wires == 0 and wiring.num_slots == 0:
            raise ValueError("Cannot define contraction for empty wiring.")
        for t in wiring.wire_types:
            if not isinstance(t, TensorLikeType):
                raise ValueError("Wiring must have tensor-like wire types.")
        self._optimize = optimize
        self._leaves = _prepare(wiring)
        lw = self._leaves
        net = _network(lw)
        self._network = net
        if tree is None:
            tree, sl = planner.optimize(net, target_bits=target_bits, trials=trials, seed=seed)
        else:
            sl = frozenset(sliced or ())
        self._tree = tree
        self._plan = planner.SlicedPlan(tree, tuple(sorted(sl)), list(lw.leaf_wires))
        self._native: NativePlan | None = None
        # (diagram, device pool) of the last cached diagram; the diagram itself is held so
        # that its id cannot be reused by a new diagram while the entry lives
        self._pool_cache: tuple[Diagram, torch.Tensor] | None = None

    # -- plan inspection ------------------------------------------------------------

    @property
    def tree(self) -> planner.ContractionTree:
        return self._tree

    @property
    def path(self) -> tuple[tuple[int, int], ...]:
        """The tree as a pop/append path over the prepared leaves."""
        return self._tree.linear_path()

    @property
    def sliced_wires(self) -> tuple[int, ...]:
        return self._plan.sliced

    @property
    def num_slices(self) -> int:
        return self._plan.num_slices

    @property
    def sliced_plan(self) -> planner.SlicedPlan:
        return self._plan

    @property
    def discard_factor(self) -> int:
        """Factor of the count contributed by wires connected to nothing (each summed
        freely); :meth:`run` results exclude it, :meth:`count` includes it."""
        return self._leaves.discard_factor

    def stats(self) -> dict[str, float]:
        sl = frozenset(self._plan.sliced)
        tot, peak, wr = self._tree.cost(sl)
        return {
            "steps": len(self._tree.steps),
            "log2_index_space_per_slice": tot,
            "peak_bits": peak,
            "log2_written_per_slice": wr,
            "num_sliced": len(sl),
            "log2_total_index_space": tot + len(sl),
        }

    def native_plan(self) -> NativePlan:
        if self._native is None:
            self._native = NativePlan(self._plan)
        return self._native

    # -- leaves -----------------------------------------------------------------------

    def leaf_pool(self, diagram: Diagram, cache: bool = True) -> torch.Tensor:
        """The diagram's leaf tensors packed into one device uint8 buffer (one host-to-
        device copy for host leaves; cached for the last diagram unless ``cache`` is
        False)."""
        if cache and self._pool_cache is not None and self._pool_cache[0] is diagram:
            return self._pool_cache[1]
        dev = _device.require_cuda()
        host, device_leaves = self._host_pool(diagram)
        pool = torch.from_numpy(host).to(dev, non_blocking=False)
        self._finish_pool(pool, device_leaves)
        if cache:
            self._pool_cache = (diagram, pool)
        return pool

    def _host_pool(self, diagram: Diagram) -> tuple[np.ndarray, list[tuple[int, Any]]]:
        """The host part of the leaf pool (host leaves and synthetic leaves at their
        offsets, zeros elsewhere) and the leaves that :meth:`_finish_pool` writes on the
        device (device-resident boxes and slots with repeated wires)."""
        npl = self.native_plan()
        lw = self._leaves
        host = np.zeros(npl.pool_bytes, dtype=np.uint8)
        device_leaves: list[tuple[int, Any]] = []
        boxes = diagram.blocks
        for l, (slot, syn) in enumerate(zip(lw.slot_of_leaf, lw.synthetic)):
            off = int(npl.leaf_offsets[l])
            if syn is not None:
                host[off: off + syn.size] = syn.reshape(-1)
                continue
            box = boxes[slot]
            on_device = isinstance(box, CudaRel) and box._tensor.device.type == "cuda"
            if slot in lw.diag_slots or on_device:
                device_leaves.append((l, box))
                continue
            arr = (box._tensor.numpy() if isinstance(box, CudaRel) else leaf_array(box))
            arr = arr.reshape(-1)
            host[off: off + arr.size] = arr
        return host, device_leaves

    def leaf_digest(self, diagram: Diagram) -> str:
        """SHA-256 of the diagram's leaf values as this contraction packs them (host and
        synthetic leaves at their pool offsets, then every device-resident or diagonal
        leaf by id). Two diagrams with this wiring have equal digests exactly when they
        contract the same leaf tensors."""
        host, device_leaves = self._host_pool(diagram)
        h = hashlib.sha256(host.tobytes())
        for l, box in device_leaves:
            if isinstance(box, CudaRel):
                arr = box._tensor.detach().cpu().numpy()
            else:
                arr = leaf_array(box)
            h.update(f"leaf {l} {tuple(arr.shape)}".encode())
            h.update(np.ascontiguousarray(arr, dtype=np.uint8).tobytes())
        return h.hexdigest()

    def _finish_pool(self, pool: torch.Tensor, device_leaves: list[tuple[int, Any]]) -> None:
        """Writes the device leaves of :meth:`_host_pool` into a device pool that already
        holds the host part (on the current stream)."""
        dev = _device.require_cuda()
        npl = self.native_plan()
        lw = self._leaves
        stream = _device.stream_handle()
        for l, box in device_leaves:
            off = int(npl.leaf_offsets[l])
            slot = lw.slot_of_leaf[l]
            t = box.device_tensor() if isinstance(box, CudaRel) else _device.to_device_u8(
                torch.from_numpy(leaf_array(box)))
            if slot in lw.diag_slots:
                ws = list(self._wiring.slot_wires_list[slot])
                uniq = list(lw.leaf_wires[l])
                one = torch.ones((), dtype=torch.uint8, device=dev)
                st = _native.lib().tsg_contract2_or_and(
                    t.data_ptr(), len(ws), _native.i64_array(ws), _native.i64_array(t.shape),
                    one.data_ptr(), 0, _native.i64_array([]), _native.i64_array([]),
                    len(uniq), _native.i64_array(uniq), pool.data_ptr() + off, stream)
                _native.check(st)
            else:
                pool[off: off + t.numel()].copy_(t.reshape(-1))

    # -- execution --------------------------------------------------------------------

    def choose_group(self, ring: int, num_primes: int, budget_bytes: int | None = None,
                     max_group: int = 4096) -> int:
        """Largest power-of-two slice group whose workspace fits the budget (default: 40%
        of free device memory)."""
        npl = self.native_plan()
        if npl.num_sliced == 0:
            return 1
        if budget_bytes is None:
            free, _ = torch.cuda.mem_get_info()
            budget_bytes = int(free * 0.4)
        g = min(self.num_slices, max_group)
        while g > 1 and npl.workspace_bytes(ring, num_primes, g) > budget_bytes:
            g //= 2
        return g

    def run(self, diagram: Diagram | None, ring: int, primes: Sequence[int] = (),
            slice_range: tuple[int, int] | None = None, group: int | None = None,
            pool: torch.Tensor | None = None, workspace: torch.Tensor | None = None,
            result: torch.Tensor | None = None, accumulate: bool = False,
            cache_leaves: bool = True) -> torch.Tensor:
        """Runs the tree executor over a slice range and returns the device result
        (uint8 / uint64 / uint32[planes] over the root's 2^bits entries)."""
        dev = _device.require_cuda()
        npl = self.native_plan()
        if pool is None:
            if diagram is None:
                raise ValueError("run() needs a diagram or a leaf pool")
            self.validate(diagram)
            pool = self.leaf_pool(diagram, cache=cache_leaves)
        planes = len(primes) if ring == _native.TSG_RING_MODP else 1
        b, e = slice_range if slice_range is not None else (0, self.num_slices)
        if group is None:
            group = self.choose_group(ring, planes)
        if workspace is None:
            workspace = torch.empty(npl.workspace_bytes(ring, planes, group), dtype=torch.uint8,
                                    device=dev)
        entries = 1 << len(self._leaves.out_unique)
        if result is None:
            if ring == _native.TSG_RING_OR_AND:
                result = torch.zeros(entries, dtype=torch.uint8, device=dev)
            elif ring == _native.TSG_RING_U64:
                result = torch.zeros(entries, dtype=torch.int64, device=dev)
            else:
                result = torch.zeros(planes * entries, dtype=torch.int32, device=dev)
        npl.run(ring, primes, pool, b, e, group, workspace, result, accumulate,
                _device.stream_handle())
        return result

    @staticmethod
    def check_device() -> None:
        """Synchronizes the current stream and raises if a kernel recorded a device-side
        failure (a bounded wait that gave up)."""
        _native.check(_native.lib().tsg_take_device_error(_device.stream_handle()))

    def contract(self, diagram: Diagram, *, progbar: bool = False, order: Any = None,
                 autojit: Any = "auto", group: int | None = None,
                 slice_range: tuple[int, int] | None = None,
                 cache_leaves: bool = True, process_group: Any = None,
                 workspace: torch.Tensor | None = None) -> CudaRel:
        """Validates and contracts the diagram in the OR-AND semiring; returns the result
        box (a scalar box for a SAT network: ``bool(box)`` is the SAT bit).

        ``slice_range`` restricts the run to slices ``[begin, end)`` (the OR of those
        slices only). With a ``torch.distributed`` ``process_group`` every rank of the
        group contracts its own contiguous share of the slices and one all-reduce ORs the
        shares, so every rank returns the whole result (see :meth:`shard_range`).
        ``workspace`` (uint8 device buffer of at least ``tsg_plan_workspace_bytes``) is
        used instead of a new allocation. ``progbar``, ``order`` and ``autojit`` are
        accepted for signature parity with ``CotengraContraction.contract`` and have no
        effect."""
        self.validate(diagram)
        if process_group is None:
            res = self.run(diagram, _native.TSG_RING_OR_AND, group=group,
                           slice_range=slice_range, cache_leaves=cache_leaves,
                           workspace=workspace)
            self.check_device()
            return self._box_from_root(res)
        group = self._shard_group(_native.TSG_RING_OR_AND, 1, group, process_group)
        local = self.shard_range(slice_range, group, process_group)
        entries = 1 << len(self._leaves.out_unique)
        if local[0] < local[1]:
            root = self._ring_root(diagram, _native.TSG_RING_OR_AND, (), local, group,
                                   cache_leaves, workspace)
        else:
            root = np.zeros(entries, dtype=np.uint8)
        root = sharding.allreduce_or(torch.from_numpy(root.astype(np.int32)).to(
            sharding.collective_device(process_group)), group=process_group)
        return self._box_from_root(torch.from_numpy(root.cpu().numpy().astype(np.uint8)))

    # -- slices across ranks ------------------------------------------------------------

    def shard_range(self, slice_range: tuple[int, int] | None, group: int,
                    process_group: Any = None) -> tuple[int, int]:
        """This rank's share of ``slice_range`` (default: every slice): with a process
        group the range is split into contiguous pieces, one per rank in rank order, each
        starting at a multiple of ``group`` (ranks launch whole slice groups); without one
        the whole range. A share may be empty."""
        b, e = slice_range if slice_range is not None else (0, self.num_slices)
        if not 0 <= b <= e <= self.num_slices:
            raise ValueError(f"slice range {(b, e)} outside [0, {self.num_slices}]")
        if process_group is None:
            return (b, e)
        import torch.distributed as dist

        if b % group:
            raise ValueError("a sharded slice range must start at a multiple of the group")
        world = dist.get_world_size(process_group)
        rank = dist.get_rank(process_group)
        lo, hi = sharding.slice_ranges(e - b, world, group)[rank]
        return (b + lo, b + hi)

    def _shard_group(self, ring: int, planes: int, group: int | None,
                     process_group: Any) -> int:
        """The slice group of a run; sharded runs agree on it before splitting (every
        rank's share starts at a multiple of it), so it must be given or the same on every
        rank: the default takes the smallest choice over the ranks."""
        if group is not None or self.num_slices == 1:
            return 1 if self.num_slices == 1 else group
        g = self.choose_group(ring, planes)
        if process_group is not None:
            g = sharding.allreduce_min_int(g, process_group)
        return g

    def _ring_root(self, diagram: Diagram, ring: int, primes: Sequence[int],
                   slice_range: tuple[int, int], group: int, cache_leaves: bool,
                   workspace: torch.Tensor | None = None) -> np.ndarray:
        """Root entries of one device run over ``slice_range``, on the host: uint8 [entries]
        (OR-AND), uint64 [entries] (U64) or uint32 [planes, entries] (MODP, plain
        residues). Raises if a kernel recorded a device-side failure."""
        res = self.run(diagram, ring, primes=primes, group=group, slice_range=slice_range,
                       cache_leaves=cache_leaves, workspace=workspace)
        self.check_device()
        host = res.cpu().numpy()
        if ring == _native.TSG_RING_U64:
            return host.view(np.uint64)
        if ring == _native.TSG_RING_MODP:
            return host.view(np.uint32).reshape(len(primes), -1)
        return host

    def _box_from_root(self, res: torch.Tensor) -> CudaRel:
        """Result box from the OR-AND root entries (over the distinct out wires)."""
        lw = self._leaves
        k = len(lw.out_unique)
        box = CudaRel._new(res.reshape((2,) * k))
        if tuple(self._wiring.out_wires) != lw.out_unique:
            box = box._rewire([lw.out_unique.index(w) for w in self._wiring.out_wires])
        return box

    def count(self, diagram: Diagram, *, ring: str = "auto", num_primes: int | None = None,
              group: int | None = None, slice_range: tuple[int, int] | None = None,
              cache_leaves: bool = True, process_group: Any = None,
              workspace: torch.Tensor | None = None) -> Any:
        """Exact model count (``int``) of a closed network, or a numpy object array of
        counts indexed by the out wires.

        ``ring="u64"`` counts modulo 2^64, ``"modp"`` modulo ``num_primes`` 31-bit primes
        with CRT, ``"auto"`` picks u64 when the count bound is below 2^64 and otherwise
        enough primes for the bound. ``slice_range`` restricts the run to slices
        ``[begin, end)``: the result is then that range's share of the count (shares of
        disjoint ranges add up to the count). With a ``torch.distributed``
        ``process_group`` (one rank per GPU) every rank counts its own contiguous share
        of the slices (:meth:`shard_range`) with no exchange while contracting, and one
        all-reduce adds the shares (per prime mod p, or mod 2^64), so every rank returns
        the whole count. ``workspace`` (uint8 device buffer of at least
        ``tsg_plan_workspace_bytes`` for the ring and group) is used instead of a new
        allocation.
        """
        self.validate(diagram)
        arrays = []
        for blk in diagram.blocks:
            try:
                arrays.append(leaf_array(blk))
            except TypeError:
                arrays.append(np.zeros((), dtype=np.uint8))
        bound = count_bound_bits(self._wiring, arrays)
        if ring == "auto":
            ring = "u64" if bound < 64 else "modp"
        entries = 1 << len(self._leaves.out_unique)
        if ring == "u64":
            if bound >= 64:
                raise OverflowError("count bound exceeds 2^64: use ring='modp'")
            g = self._shard_group(_native.TSG_RING_U64, 1, group, process_group)
            local = self.shard_range(slice_range, g, process_group)
            if local[0] < local[1]:
                vals = self._ring_root(diagram, _native.TSG_RING_U64, (), local, g,
                                       cache_leaves, workspace)
            else:
                vals = np.zeros(entries, dtype=np.uint64)
            if process_group is not None:
                vals = sharding.allreduce_u64(vals, process_group)
            counts = np.array([int(v) for v in vals], dtype=object)
        elif ring == "modp":
            if num_primes is None:
                num_primes = 1
                while sum(math.log2(p) for p in PRIMES_31[:num_primes]) <= bound:
                    num_primes += 1
            if num_primes > len(PRIMES_31):
                raise OverflowError(f"count bound 2^{bound:.0f} exceeds the residue range")
            primes = PRIMES_31[:num_primes]
            if sum(math.log2(p) for p in primes) <= bound:
                raise OverflowError(
                    f"count bound 2^{bound:.0f} needs more than {num_primes} 31-bit primes"
                )
            g = self._shard_group(_native.TSG_RING_MODP, min(num_primes, _native.TSG_MAX_PRIMES),
                                  group, process_group)
            local = self.shard_range(slice_range, g, process_group)
            residues = []
            for i in range(0, num_primes, _native.TSG_MAX_PRIMES):
                chunk = primes[i: i + _native.TSG_MAX_PRIMES]
                if local[0] < local[1]:
                    planes = self._ring_root(diagram, _native.TSG_RING_MODP, chunk, local, g,
                                             cache_leaves, workspace)
                else:
                    planes = np.zeros((len(chunk), entries), dtype=np.uint32)
                if process_group is not None:
                    summed = sharding.allreduce_residues(
                        torch.from_numpy(planes.astype(np.int64)).to(
                            sharding.collective_device(process_group)),
                        chunk, group=process_group)
                    planes = summed.cpu().numpy()
                residues.extend(planes[p] for p in range(len(chunk)))
            counts = crt(residues, primes)
        else:
            raise ValueError(f"unknown count ring {ring!r}")
        return self._counts_from_root(counts)

    # -- leaf variants of one wiring ----------------------------------------------------

    def run_variants(self, diagrams: Sequence[Diagram], ring: int, primes: Sequence[int] = (),
                     group: int | None = None) -> list[np.ndarray]:
        """Contracts many diagrams of this wiring (leaf variants: the assignment-search
        idiom) in one launch sequence (``tsg_plan_run_variants``): every step runs once
        per slice group for all variants, the variant index being an extra batch axis.
        Returns each variant's root entries on the host, laid out as :meth:`run`'s."""
        if not diagrams:
            raise ValueError("run_variants needs at least one diagram")
        for d in diagrams:
            self.validate(d)
        dev = _device.require_cuda()
        npl = self.native_plan()
        n = len(diagrams)
        nv = 1 << (n - 1).bit_length()
        stride = 1 << max(4, (npl.pool_bytes - 1).bit_length())
        parts = [self._host_pool(d) for d in diagrams]
        host = np.zeros(nv * stride, dtype=np.uint8)
        for v in range(nv):  # padding variants repeat the first diagram
            h, _ = parts[v] if v < n else parts[0]
            host[v * stride: v * stride + h.size] = h
        pool = torch.from_numpy(host).to(dev)
        for v in range(nv):
            dl = parts[v][1] if v < n else parts[0][1]
            if dl:
                self._finish_pool(pool[v * stride: v * stride + npl.pool_bytes], dl)
        planes = len(primes) if ring == _native.TSG_RING_MODP else 1
        if group is None:
            group = self._variant_group(ring, planes, nv)
        lib = _native.lib()
        need = _native.c_int64()
        _native.check(lib.tsg_plan_variants_workspace_bytes(npl.handle, ring, planes, group, nv,
                                                            _native.ctypes.byref(need)))
        ws = torch.empty(max(need.value, 256), dtype=torch.uint8, device=dev)
        entries = 1 << len(self._leaves.out_unique)
        esize = {_native.TSG_RING_OR_AND: 1, _native.TSG_RING_U64: 8}.get(ring, 4)
        per = entries * esize * planes
        res = torch.zeros(nv * per, dtype=torch.uint8, device=dev)
        parr = (_native.c_uint32 * max(1, len(primes)))(*primes)
        _native.check(lib.tsg_plan_run_variants(
            npl.handle, ring, len(primes), parr, pool.data_ptr(), stride, nv, group,
            ws.data_ptr(), ws.numel(), res.data_ptr(), 0, _device.stream_handle()))
        self.check_device()
        flat = res.cpu().numpy()
        dt = {_native.TSG_RING_OR_AND: np.uint8, _native.TSG_RING_U64: np.uint64}.get(ring, np.uint32)
        out = []
        for v in range(n):
            a = flat[v * per: (v + 1) * per].view(dt)
            out.append(a.reshape(planes, -1) if ring == _native.TSG_RING_MODP else a)
        return out

    def _variant_group(self, ring: int, planes: int, variants: int) -> int:
        """Largest power-of-two slice group whose variant workspace fits 40% of free device
        memory."""
        npl = self.native_plan()
        if npl.num_sliced == 0:
            return 1
        free, _ = torch.cuda.mem_get_info()
        budget = int(free * 0.4)
        lib = _native.lib()
        g = self.num_slices
        need = _native.c_int64()
        while g > 1:
            _native.check(lib.tsg_plan_variants_workspace_bytes(
                npl.handle, ring, planes, g, variants, _native.ctypes.byref(need)))
            if need.value <= budget:
                break
            g //= 2
        return g

    def contract_variants(self, diagrams: Sequence[Diagram], *,
                          group: int | None = None) -> list[CudaRel]:
        """OR-AND contraction of many diagrams of this wiring in one launch sequence
        (:meth:`run_variants`): one result box per diagram (``bool(box)`` is its SAT bit
        for a closed network)."""
        roots = self.run_variants(diagrams, _native.TSG_RING_OR_AND, group=group)
        return [self._box_from_root(torch.from_numpy(r.copy())) for r in roots]

    def count_variants(self, diagrams: Sequence[Diagram], *, num_primes: int | None = None,
                       group: int | None = None) -> list[Any]:
        """Exact model counts of many diagrams of this wiring in one launch sequence, modulo
        31-bit primes with CRT (enough primes for the largest count bound, at most 4)."""
        bounds = []
        for d in diagrams:
            arrays = []
            for blk in d.blocks:
                try:
                    arrays.append(leaf_array(blk))
                except TypeError:
                    arrays.append(np.zeros((), dtype=np.uint8))
            bounds.append(count_bound_bits(self._wiring, arrays))
        need = 1
        while sum(math.log2(p) for p in PRIMES_31[:need]) <= max(bounds):
            need += 1
        if num_primes is None:
            num_primes = need
        if num_primes < need or num_primes > _native.TSG_MAX_PRIMES:
            raise OverflowError(f"the variants' count bounds need {need} primes (at most "
                                f"{_native.TSG_MAX_PRIMES} per run)")
        primes = PRIMES_31[:num_primes]
        roots = self.run_variants(diagrams, _native.TSG_RING_MODP, primes, group=group)
        return [self._counts_from_root(crt([r[p] for p in range(num_primes)], primes))
                for r in roots]

    # -- plans and checkpoints --------------------------------------------------------

    def plan_dict(self) -> dict:
        """The tree and sliced wires (``planner.plan_to_dict``) with the prepared leaf
        wires they index, as JSON data."""
        d = planner.plan_to_dict(self._tree, self._plan.sliced)
        d["leaf_wires"] = [list(ws) for ws in self._leaves.leaf_wires]
        return d

    def save_plan(self, path: str | os.PathLike) -> None:
        """Writes :meth:`plan_dict` as JSON (atomically: a temporary file, then a rename),
        so another process can skip planning with :meth:`from_plan`."""
        _write_json(Path(path), self.plan_dict())

    @classmethod
    def from_plan(cls, box_class: type, wiring: Wiring,
                  plan: dict | str | os.PathLike) -> "GpuContraction":
        """A contraction for ``wiring`` that runs a saved plan (a :meth:`plan_dict` or the
        path of a :meth:`save_plan` file) instead of planning. Raises ValueError when the
        plan was made for other leaves."""
        data = plan if isinstance(plan, dict) else json.loads(Path(plan).read_text())
        tree, sliced = planner.plan_from_dict(data)
        if [tuple(ws) for ws in data.get("leaf_wires", [])] != \
                [tuple(ws) for ws in _prepare(wiring).leaf_wires]:
            raise ValueError("the plan was made for a different wiring")
        return cls(box_class, wiring, tree=tree, sliced=sliced)

    def count_checkpointed(self, diagram: Diagram, path: str | os.PathLike, *,
                           chunk_slices: int, ring: str = "modp",
                           num_primes: int | None = None, group: int | None = None) -> int:
        """Exact model count of a closed network, run ``chunk_slices`` slices at a time.
        After every chunk its count (chunks are disjoint slice ranges, whose counts add
        up) is recorded in the JSON file at ``path`` together with the plan; a later call
        with the same file skips the recorded chunks, so an interrupted run resumes where
        it stopped. The file also records a digest of the leaf tensors
        (:meth:`leaf_digest`). Raises ValueError when the file belongs to another plan,
        other arguments or other leaves (another instance with the same wiring)."""
        if self._leaves.out_unique:
            raise ValueError("count_checkpointed counts closed networks only")
        if chunk_slices < 1:
            raise ValueError("chunk_slices must be positive")
        path = Path(path)
        settings = {"ring": ring, "num_primes": num_primes, "chunk_slices": int(chunk_slices)}
        plan = self.plan_dict()
        leaves = self.leaf_digest(diagram)
        done: dict[str, str] = {}
        if path.exists():
            state = json.loads(path.read_text())
            if state.get("format") != _CHECKPOINT_FORMAT or state.get("plan") != plan or \
                    state.get("settings") != settings:
                raise ValueError(f"{path} records another plan or other count arguments")
            if state.get("leaves") != leaves:
                raise ValueError(f"{path} records the counts of other leaf tensors (another "
                                 "instance with the same wiring)")
            done = dict(state["done"])
        ns = self.num_slices
        # every chunk starts at a multiple of the slice group (a power of two)
        if group is None:
            code = _native.TSG_RING_U64 if ring == "u64" else _native.TSG_RING_MODP
            group = self.choose_group(code, 1 if ring == "u64" else _native.TSG_MAX_PRIMES)
        group = min(group, chunk_slices & -chunk_slices)
        for begin in range(0, ns, chunk_slices):
            key = str(begin)
            if key in done:
                continue
            rng = (begin, min(ns, begin + chunk_slices))
            done[key] = str(int(self.count(diagram, ring=ring, num_primes=num_primes,
                                           group=group, slice_range=rng)))
            _write_json(path, {"format": _CHECKPOINT_FORMAT, "plan": plan,
                               "settings": settings, "leaves": leaves, "done": done})
        return sum(int(v) for v in done.values())

    def _counts_from_root(self, counts: np.ndarray) -> Any:
        """Counts (``int`` for a closed network, an object array over the out wires
        otherwise) from the exact root entries of a run (discarded wires excluded)."""
        lw = self._leaves
        counts = counts * lw.discard_factor
        k = len(lw.out_unique)
        if k == 0:
            return int(counts[0])
        arr = counts.reshape((2,) * k)
        outs = self._wiring.out_wires
        if tuple(outs) == lw.out_unique:
            return arr
        # expand repeated / permuted out wires (diagonal entries, zeros elsewhere)
        full = np.zeros((2,) * len(outs), dtype=object)
        for idx in np.ndindex(*full.shape):
            vals = {}
            ok = True
            for w, v in zip(outs, idx):
                if vals.setdefault(w, v) != v:
                    ok = False
                    break
            full[idx] = arr[tuple(vals[w] for w in lw.out_unique)] if ok else 0
        return full

    def __repr__(self) -> str:
        return "<GpuContraction>"
