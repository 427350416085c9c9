"""Batched contraction of many networks in one native call (``tsg_batch_run``).

The reference contracts one diagram per ``Contraction.contract`` call
(``tensorsat/contractions/abc.py:92``). A batch of networks of uneven sizes (for example
random CNF instances with different variable and clause counts) is planned network by
network (one :class:`~tensorsat_gb300.contractions.gpu.GpuContraction` each), then run
by one C call. That call checks every instance and every launch on the host, then issues
all kernels of all instances on one stream with one shared workspace. It neither
allocates nor synchronises, so :meth:`BatchContraction.capture` records it into a CUDA
graph, and each replay reruns the whole batch with a single launch from the host.

Serving form: :meth:`BatchContraction.count` and :meth:`BatchContraction.contract` with
``graph=True`` capture their run once and replay it on later calls, and
:meth:`BatchContraction.load` copies the leaves of new diagrams with the same wirings into
the captured leaf pools in place, so a stream of inputs pays one host-to-device copy, one
graph launch and one read-back per batch.

:meth:`BatchContraction.serve` pipelines such a stream: while the GPU contracts one batch
of inputs, the host packs the next batch's leaves into the other of two pinned staging
buffers and reads back the previous batch's answers.

Results are the same as running each network through its own
:class:`~tensorsat_gb300.contractions.gpu.GpuContraction`: SAT bits in the OR-AND
semiring, exact model counts modulo 31-bit primes recombined by CRT.
"""

from __future__ import annotations

import ctypes
import math
from collections.abc import Iterable, Iterator, Sequence
from typing import Any

import numpy as np
import torch

from .. import _device, _native
from ..diagrams import Diagram
from ..lang.cuda_rel import CudaRel, leaf_array
from .gpu import PRIMES_31, GpuContraction, count_bound_bits, crt

__all__ = ["BatchContraction", "BatchGraph"]


def _ptr_array(values: Sequence[int]) -> Any:
    return (ctypes.c_void_p * max(1, len(values)))(*values)


def _host_results(results: Sequence[torch.Tensor]) -> list[np.ndarray]:
    """Host copies of the results of a batch: their bytes gathered on the device, then one
    device-to-host copy, then a numpy view of each result."""
    if not results:
        return []
    raw = [r.reshape(-1).view(torch.uint8) for r in results]
    flat = torch.cat(raw).cpu().numpy()
    out, off = [], 0
    for r, b in zip(results, raw):
        n = b.numel()
        dt = {torch.uint8: np.uint8, torch.int32: np.int32, torch.int64: np.int64}[r.dtype]
        out.append(flat[off: off + n].view(dt).reshape(tuple(r.shape)).copy())
        off += n
    return out


class BatchGraph:
    """A captured batch run: :meth:`replay` reruns every instance of the batch into the
    same result buffers with one graph launch."""

    def __init__(self, graph: torch.cuda.CUDAGraph, results: list[torch.Tensor],
                 groups: list[int], launches: int, keep: list[Any]) -> None:
        self._graph = graph
        self.results = results
        self.groups = groups      # slice group of each instance
        self.launches = launches  # kernel launches recorded in the graph
        self._keep = keep  # workspace, pools and argument arrays the graph points to

    def replay(self) -> list[torch.Tensor]:
        self._graph.replay()
        return self.results


class BatchContraction:
    """Plans a batch of flat diagrams (each closed or with open outputs) and contracts them
    together: :meth:`contract` gives one result box per diagram, :meth:`count` one exact
    model count per diagram."""

    def __init__(self, box_class: type[CudaRel], diagrams: Sequence[Diagram], *,
                 target_bits: int | None = 26, trials: int = 2, seed: int = 0,
                 trees: Sequence[tuple[Any, Sequence[int]]] | None = None,
                 lanes: int = 16, packed: bool = True) -> None:
        """``trees`` optionally gives each diagram's (tree, sliced wires), for example from
        :func:`~tensorsat_gb300.contractions.gpu.plan_tree` run in worker processes;
        otherwise every diagram is planned here with ``target_bits``, ``trials`` and
        ``seed``. ``lanes`` (1..32) is the number of concurrent lanes the batch's
        instances are spread over (``tsg_batch_run_lanes``): each lane is a stream with its
        own workspace region, so the small launches of different instances overlap.
        ``packed`` (default) runs each lane's instances in packs, level by level of their
        trees, with the small steps of every pack member in shared launches
        (``tsg_batch_run_packed``); otherwise every step of every instance is its own
        launch (``tsg_batch_run_lanes``). Both give the same answers."""
        if not diagrams:
            raise ValueError("A batch needs at least one diagram.")
        if not 1 <= lanes <= 32:
            raise ValueError("lanes must lie in 1..32")
        self.lanes = min(lanes, len(diagrams))
        self.packed = bool(packed)
        self._diagrams = list(diagrams)
        if trees is not None and len(trees) != len(self._diagrams):
            raise ValueError(f"expected {len(self._diagrams)} trees, got {len(trees)}")
        self._contractions = [
            GpuContraction(box_class, d.wiring, target_bits=target_bits, trials=trials,
                           seed=seed)
            if trees is None else
            GpuContraction(box_class, d.wiring, tree=trees[i][0], sliced=trees[i][1])
            for i, d in enumerate(self._diagrams)]
        for c, d in zip(self._contractions, self._diagrams):
            c.validate(d)
        self._pools: list[torch.Tensor] | None = None
        self._graphs: dict[tuple, BatchGraph] = {}
        self.last_launches = 0  # kernel launches of the last run (or capture)
        self._staging: torch.Tensor | None = None    # pinned host copy of the leaf pools
        self._staged: torch.cuda.Event | None = None  # the staging buffer's last copies
        self._serve_stage: list[torch.Tensor | None] = [None, None]  # serve()'s two buffers
        self._need: int | None = None                # cached primes_needed()
        self._need_pool: np.ndarray | None = None    # host leaves it was computed from

    @property
    def contractions(self) -> list[GpuContraction]:
        return self._contractions

    def __len__(self) -> int:
        return len(self._contractions)

    # -- native arguments -------------------------------------------------------------

    def pools(self) -> list[torch.Tensor]:
        """Device leaf pools of every instance (uploaded once)."""
        if self._pools is None:
            self._pools = [c.leaf_pool(d, cache=False)
                           for c, d in zip(self._contractions, self._diagrams)]
        return self._pools

    def load(self, diagrams: Sequence[Diagram] | None = None) -> int:
        """Copies the leaves of ``diagrams`` (the batch's wirings, in order; default: the
        batch's own diagrams) into the batch's device leaf pools in place and returns the
        bytes copied. Later runs, and replays of graphs captured from this batch, contract
        the new leaves. Host leaves go through one pinned staging buffer (one asynchronous
        copy per instance on the current stream); device leaves are copied on the device.
        """
        if diagrams is not None:
            diagrams = list(diagrams)
            if len(diagrams) != len(self):
                raise ValueError(f"expected {len(self)} diagrams, got {len(diagrams)}")
            for c, d in zip(self._contractions, diagrams):
                c.validate(d)
            self._diagrams = diagrams
        if self._pools is None:
            return sum(p.numel() for p in self.pools())
        parts = [c._host_pool(d) for c, d in zip(self._contractions, self._diagrams)]
        total = sum(host.size for host, _ in parts)
        if self._staged is not None:
            self._staged.synchronize()  # the previous copies have read the staging buffer
        if self._staging is None or self._staging.numel() < total:
            self._staging = torch.empty(max(1, total), dtype=torch.uint8, pin_memory=True)
        stage = self._staging.numpy()
        off = 0
        for c, pool, (host, device_leaves) in zip(self._contractions, self._pools, parts):
            if pool.numel() != host.size:
                raise RuntimeError("leaf pool size changed")
            stage[off: off + host.size] = host
            pool.copy_(self._staging[off: off + host.size], non_blocking=True)
            c._finish_pool(pool, device_leaves)
            off += host.size
        self._staged = torch.cuda.Event()
        self._staged.record()
        self._keep_bound(stage[:total], [dl for _, dl in parts])
        return total

    def groups(self, ring: int, planes: int, budget_bytes: int | None = None) -> list[int]:
        """Slice group per instance: the largest power of two whose workspace fits the
        budget (default: 40% of free device memory) divided by the lanes (every lane holds
        the workspace of its largest instance)."""
        if budget_bytes is None:
            free, _ = torch.cuda.mem_get_info()
            budget_bytes = int(free * 0.4)
        per_lane = max(1, budget_bytes // self.lanes)
        return [c.choose_group(ring, planes, per_lane) for c in self._contractions]

    def workspace_bytes(self, ring: int, planes: int, groups: Sequence[int]) -> int:
        lib = _native.lib()
        handles = _ptr_array([c.native_plan().handle.value for c in self._contractions])
        out = ctypes.c_int64()
        fn = lib.tsg_batch_packed_workspace_bytes if self.packed else \
            lib.tsg_batch_lanes_workspace_bytes
        _native.check(fn(len(self), handles, ring, planes, _native.i64_array(list(groups)),
                         self.lanes, ctypes.byref(out)))
        return int(out.value)

    def _results(self, ring: int, planes: int) -> list[torch.Tensor]:
        """One result buffer per instance, as views into one flat device buffer (16-byte
        aligned slots), so that all results come back to the host in one copy
        (:func:`_host_results`)."""
        dev = _device.require_cuda()
        dtype = {_native.TSG_RING_OR_AND: torch.uint8, _native.TSG_RING_U64: torch.int64}.get(
            ring, torch.int32)
        esize = torch.tensor([], dtype=dtype).element_size()
        sizes = []
        for c in self._contractions:
            entries = 1 << len(c._leaves.out_unique)
            sizes.append(entries * (planes if ring == _native.TSG_RING_MODP else 1))
        offsets, off = [], 0
        for n in sizes:
            offsets.append(off)
            off += (n * esize + 15) // 16 * 16
        flat = torch.zeros(max(off, 16), dtype=torch.uint8, device=dev)
        return [flat[o: o + n * esize].view(dtype) for o, n in zip(offsets, sizes)]

    def _call(self, ring: int, primes: Sequence[int], groups: Sequence[int],
              workspace: torch.Tensor, results: Sequence[torch.Tensor], stream: int) -> list:
        lib = _native.lib()
        pools = self.pools()
        args = [
            _ptr_array([c.native_plan().handle.value for c in self._contractions]),
            (_native.c_uint32 * max(1, len(primes)))(*primes),
            _ptr_array([p.data_ptr() for p in pools]),
            _native.i64_array(list(groups)),
            _ptr_array([r.data_ptr() for r in results]),
        ]
        if self.packed:
            launches = ctypes.c_int64()
            st = lib.tsg_batch_run_packed(len(self), args[0], ring, len(primes), args[1],
                                          args[2], args[3], self.lanes, workspace.data_ptr(),
                                          workspace.numel(), args[4], stream,
                                          ctypes.byref(launches))
            self.last_launches = int(launches.value)
        else:
            st = lib.tsg_batch_run_lanes(len(self), args[0], ring, len(primes), args[1],
                                         args[2], args[3], self.lanes, workspace.data_ptr(),
                                         workspace.numel(), args[4], stream)
            self.last_launches = sum(
                c.native_plan().launch_count(0, c.num_slices, g, ring, max(1, len(primes)))
                for c, g in zip(self._contractions, groups))
        _native.check(st)
        return args

    def _workspace(self, ring: int, planes: int, groups: Sequence[int],
                   workspace: torch.Tensor | None) -> torch.Tensor:
        need = self.workspace_bytes(ring, planes, groups)
        if workspace is not None:
            if workspace.numel() < need:
                raise ValueError(f"the batch needs a workspace of {need} bytes")
            return workspace
        return torch.empty(max(1, need), dtype=torch.uint8, device=_device.require_cuda())

    def run(self, ring: int, primes: Sequence[int] = (), groups: Sequence[int] | None = None,
            workspace: torch.Tensor | None = None) -> list[torch.Tensor]:
        """One ``tsg_batch_run`` call over every instance; returns each instance's device
        result (layout as :meth:`GpuContraction.run`). ``workspace`` (uint8, at least
        :meth:`workspace_bytes`) may be shared with other batches run on the same stream."""
        planes = len(primes) if ring == _native.TSG_RING_MODP else 1
        if groups is None:
            groups = self.groups(ring, planes)
        ws = self._workspace(ring, planes, groups, workspace)
        results = self._results(ring, planes)
        self._call(ring, primes, groups, ws, results, _device.stream_handle())
        GpuContraction.check_device()
        return results

    def capture(self, ring: int, primes: Sequence[int] = (), groups: Sequence[int] | None = None,
                workspace: torch.Tensor | None = None) -> BatchGraph:
        """Records one batch run into a CUDA graph (after one uncaptured run, which sets up
        the kernels' attributes); :meth:`BatchGraph.replay` reruns it. Graphs replayed on
        one stream may share one ``workspace``."""
        dev = _device.require_cuda()
        planes = len(primes) if ring == _native.TSG_RING_MODP else 1
        if groups is None:
            groups = self.groups(ring, planes)
        ws = self._workspace(ring, planes, groups, workspace)
        results = self._results(ring, planes)
        self._call(ring, primes, groups, ws, results, _device.stream_handle())
        torch.cuda.synchronize(dev)
        graph = torch.cuda.CUDAGraph()
        with torch.cuda.graph(graph):
            args = self._call(ring, primes, groups, ws, results,
                              torch.cuda.current_stream(dev).cuda_stream)
        return BatchGraph(graph, results, list(groups), self.last_launches,
                          [ws, self.pools(), args, list(primes)])

    def _replay(self, ring: int, primes: Sequence[int], groups: Sequence[int] | None,
                workspace: torch.Tensor | None) -> list[torch.Tensor]:
        """Replays this batch's cached graph for (ring, primes, groups), capturing it on
        first use (with ``workspace``, which the graph keeps); returns its result buffers,
        which the next replay overwrites."""
        res = self._replay_graph(ring, primes, groups, workspace).replay()
        GpuContraction.check_device()
        return res

    # -- answers ----------------------------------------------------------------------

    def contract(self, groups: Sequence[int] | None = None, *, graph: bool = False,
                 workspace: torch.Tensor | None = None) -> list[CudaRel]:
        """OR-AND contraction of every diagram: one result box per diagram (a scalar box
        for a SAT network: ``bool(box)`` is its SAT bit), read back to the host in one
        copy. ``graph=True`` replays a graph captured on the first such call (see
        :meth:`load` for new inputs)."""
        if graph:
            res = self._replay(_native.TSG_RING_OR_AND, (), groups, workspace)
        else:
            res = self.run(_native.TSG_RING_OR_AND, groups=groups, workspace=workspace)
        host = _host_results(res)
        return [c._box_from_root(torch.from_numpy(h)) for c, h in zip(self._contractions, host)]

    def count_bounds(self) -> list[float]:
        """log2 upper bound on each diagram's model count (free variables of its oriented
        gate network)."""
        bounds = []
        for c, d in zip(self._contractions, self._diagrams):
            arrays = []
            for blk in d.blocks:
                try:
                    arrays.append(leaf_array(blk))
                except TypeError:
                    arrays.append(np.zeros((), dtype=np.uint8))
            bounds.append(count_bound_bits(c._wiring, arrays))
        return bounds

    def primes_needed(self) -> int:
        """31-bit primes whose product exceeds every diagram's count bound. Cached: a new
        input batch (:meth:`load`, :meth:`serve`) whose leaf entries are all at most the
        ones the bound was computed from keeps it, since a count only grows with its leaf
        entries (all non-negative)."""
        if self._need is None:
            bound = max(self.count_bounds())
            n = 1
            while sum(math.log2(p) for p in PRIMES_31[:n]) <= bound:
                n += 1
            self._need = n
            parts = [c._host_pool(d) for c, d in zip(self._contractions, self._diagrams)]
            self._need_pool = (None if any(dl for _, dl in parts)
                               else np.concatenate([h for h, _ in parts]))
        return self._need

    def _keep_bound(self, staged: np.ndarray, device_leaves: Sequence[Any]) -> None:
        """Drops the cached prime count unless the staged host leaves of a new input batch
        are entrywise at most those it was computed from (and no leaf is on the device)."""
        ref = self._need_pool
        if ref is None or any(device_leaves) or staged.size != ref.size or \
                not bool(np.all(staged <= ref)):
            self._need = None

    def count(self, num_primes: int | None = None,
              groups: Sequence[int] | None = None, *, graph: bool = False,
              workspace: torch.Tensor | None = None) -> list[Any]:
        """Exact model count of every diagram (``int`` for closed networks, a numpy object
        array over the out wires otherwise), from one batched run modulo ``num_primes``
        31-bit primes (default: as many as the largest count bound of the batch needs, at
        most 4 per run). ``graph=True`` replays a graph captured on the first such call
        (see :meth:`load` for new inputs)."""
        need = self.primes_needed()
        if num_primes is None:
            num_primes = need
        if num_primes < need:
            raise OverflowError(f"the batch's count bounds need {need} 31-bit primes")
        if num_primes > _native.TSG_MAX_PRIMES:
            raise OverflowError(
                f"the batch needs {num_primes} primes; one batched run carries at most "
                f"{_native.TSG_MAX_PRIMES} (count such networks with GpuContraction.count)")
        primes = PRIMES_31[:num_primes]
        if graph:
            res = self._replay(_native.TSG_RING_MODP, primes, groups, workspace)
        else:
            res = self.run(_native.TSG_RING_MODP, primes, groups=groups, workspace=workspace)
        out = []
        for c, h in zip(self._contractions, _host_results(res)):
            planes = h.view(np.uint32).reshape(num_primes, -1)
            counts = crt([planes[p] for p in range(num_primes)], primes)
            out.append(c._counts_from_root(counts))
        return out

    def _stage(self, diagrams: Sequence[Diagram], slot: int) -> list:
        """Validates ``diagrams`` (this batch's wirings, in order) and packs their host
        leaves into pinned staging buffer ``slot`` (0 or 1); returns the device leaves
        that :meth:`GpuContraction._finish_pool` writes."""
        diagrams = list(diagrams)
        if len(diagrams) != len(self):
            raise ValueError(f"expected {len(self)} diagrams, got {len(diagrams)}")
        for c, d in zip(self._contractions, diagrams):
            c.validate(d)
        parts = [c._host_pool(d) for c, d in zip(self._contractions, diagrams)]
        total = sum(host.size for host, _ in parts)
        buf = self._serve_stage[slot]
        if buf is None or buf.numel() < total:
            buf = torch.empty(max(1, total), dtype=torch.uint8, pin_memory=True)
            self._serve_stage[slot] = buf
        stage = buf.numpy()
        off = 0
        for pool, (host, _) in zip(self.pools(), parts):
            if pool.numel() != host.size:
                raise RuntimeError("leaf pool size changed")
            stage[off: off + host.size] = host
            off += host.size
        return [dl for _, dl in parts]

    def serve(self, batches: Iterable[Sequence[Diagram]], num_primes: int | None = None, *,
              groups: Sequence[int] | None = None, sat_groups: Sequence[int] | None = None,
              workspace: torch.Tensor | None = None) -> Iterator[tuple[list[Any], list[CudaRel]]]:
        """Serves a stream of input batches (each a list of diagrams with this batch's
        wirings, in order) and yields, per batch, its exact model counts and OR-AND result
        boxes (as :meth:`count` and :meth:`contract` give them; ``bool(box)`` is a closed
        network's SAT bit). One graph per ring is captured on
        the first batch and replayed for every batch; while the GPU contracts batch k, the
        host packs batch k+1's leaves into the other of two pinned staging buffers and
        reads back batch k-1's answers, so a pass costs about the larger of the host and
        the device time instead of their sum."""
        need = self.primes_needed()
        if num_primes is None:
            num_primes = need
        if num_primes < need or num_primes > _native.TSG_MAX_PRIMES:
            raise OverflowError(f"the batch's count bounds need {need} 31-bit primes "
                                f"(at most {_native.TSG_MAX_PRIMES} per run)")
        primes = PRIMES_31[:num_primes]
        dev = _device.require_cuda()
        stream = torch.cuda.current_stream(dev)
        if self._pools is None:
            self.pools()
        copied = [torch.cuda.Event(), torch.cuda.Event()]  # staging buffer free again
        for ev in copied:
            ev.record(stream)
        g_count = g_sat = None
        pending = None  # (done event, pinned results, sizes) of the batch in flight
        slot = 0
        for diagrams in batches:
            copied[slot].synchronize()  # the copies out of this buffer (two batches ago) ran
            diagrams = list(diagrams)
            device_leaves = self._stage(diagrams, slot)
            buf = self._serve_stage[slot]
            self._diagrams = diagrams
            self._keep_bound(buf.numpy()[:sum(p.numel() for p in self._pools)],
                             device_leaves)
            if self.primes_needed() > num_primes:
                raise OverflowError(f"a served batch needs {self._need} 31-bit primes; the "
                                    f"stream was started with {num_primes}")
            off = 0
            for c, pool, dl in zip(self._contractions, self._pools, device_leaves):
                n = pool.numel()
                pool.copy_(buf[off: off + n], non_blocking=True)
                c._finish_pool(pool, dl)
                off += n
            copied[slot].record(stream)
            if g_count is None:
                g_count = self._replay_graph(_native.TSG_RING_MODP, primes, groups, workspace)
                g_sat = self._replay_graph(_native.TSG_RING_OR_AND, (), sat_groups, workspace)
            g_count.replay()
            g_sat.replay()
            res = g_count.results + g_sat.results
            flat = torch.cat([r.reshape(-1).view(torch.uint8) for r in res])
            host = torch.empty(flat.numel(), dtype=torch.uint8, pin_memory=True)
            host.copy_(flat, non_blocking=True)
            # the failure record as of this batch, read with the results (no stream sync)
            flag = torch.zeros(1, dtype=torch.int32, pin_memory=True)
            _native.check(_native.lib().tsg_peek_device_error_async(flag.data_ptr(),
                                                                    stream.cuda_stream))
            done = torch.cuda.Event()
            done.record(stream)
            if pending is not None:
                yield self._serve_answers(*pending, primes)
            pending = (done, host, flag, [(r.dtype, tuple(r.shape),
                                           r.numel() * r.element_size()) for r in res])
            slot ^= 1
        if pending is not None:
            yield self._serve_answers(*pending, primes)

    def _replay_graph(self, ring: int, primes: Sequence[int], groups: Sequence[int] | None,
                      workspace: torch.Tensor | None) -> BatchGraph:
        key = (ring, tuple(primes), None if groups is None else tuple(groups))
        g = self._graphs.get(key)
        if g is None:
            g = self.capture(ring, primes, groups, workspace)
            self._graphs[key] = g
        return g

    def _serve_answers(self, done: torch.cuda.Event, host: torch.Tensor, flag: torch.Tensor,
                       sizes: list, primes: Sequence[int]) -> tuple[list[Any], list[CudaRel]]:
        done.synchronize()
        if int(flag[0]) != 0:
            GpuContraction.check_device()  # synchronizes, clears and raises the failure
        raw = host.numpy()
        arrays, off = [], 0
        for dtype, shape, nbytes in sizes:
            dt = {torch.uint8: np.uint8, torch.int32: np.int32, torch.int64: np.int64}[dtype]
            arrays.append(raw[off: off + nbytes].view(dt).reshape(shape))
            off += nbytes
        n = len(self)
        counts = []
        for c, h in zip(self._contractions, arrays[:n]):
            planes = h.view(np.uint32).reshape(len(primes), -1)
            counts.append(c._counts_from_root(crt([planes[p] for p in range(len(primes))],
                                                  primes)))
        boxes = [c._box_from_root(torch.from_numpy(h.copy()))
                 for c, h in zip(self._contractions, arrays[n:])]
        return counts, boxes

    def __repr__(self) -> str:
        return f"<BatchContraction of {len(self)} networks>"
