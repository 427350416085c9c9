"""Contraction planning for bit-indexed tensor networks: trees, slicing and layouts.

The reference delegates path search to cotengra (``ctg.array_contract_tree`` in
``tensorsat/contractions/cotengra.py:78-85``), which is not vendored. This module is the
project's own optimiser:

* :func:`build_tree` turns a wire elimination order into a binary contraction tree. Every
  wire that is neither an output wire nor needed by another remaining tensor is summed at
  the first step where that becomes true (cotengra's index bookkeeping, as opposed to
  ``SimpleContraction`` which keeps every wire until the root,
  ``tensorsat/contractions/simple.py:263-272``).
* :func:`minfill_order` produces elimination orders (min-fill with random tie breaking)
  after a growth-free simplification pass that absorbs gates and unit tensors.
* :func:`slice_tree` picks wires to slice (fix per slice) until every intermediate holds at
  most ``2**target_bits`` entries; slices are independent sub-contractions combined by OR
  (SAT) or sum (counts), like cotengra's sliced ``tree.contract``.
* :class:`SlicedPlan` fixes the wire order (the HBM layout) of every intermediate and
  emits the integer arrays consumed by ``tsg_plan_create``.

Answers never depend on the tree; trees only change cost.
"""

from __future__ import annotations

import ctypes
import math
import random
from dataclasses import dataclass, field
from typing import Sequence

import numpy as np

from . import _native

TSG_MAX_BITS = 62


@dataclass
class Network:
    """A tensor network over wires: leaf wire tuples, wire dims and open (output) wires."""

    leaf_wires: list[tuple[int, ...]]
    wire_dims: dict[int, int]
    out_wires: tuple[int, ...] = ()

    def __post_init__(self) -> None:
        for ws in self.leaf_wires:
            if len(set(ws)) != len(ws):
                raise ValueError("leaf tensors must carry distinct wires")
            for w in ws:
                if w not in self.wire_dims:
                    raise ValueError(f"wire {w} has no dimension")
        for w in self.out_wires:
            if w not in self.wire_dims:
                raise ValueError(f"output wire {w} has no dimension")

    @property
    def all_bits(self) -> bool:
        return all(d == 2 for d in self.wire_dims.values())


@dataclass
class ContractionTree:
    """Binary contraction tree in SSA form.

    Node ids ``0..L-1`` are the leaves; step ``s`` creates node ``L+s`` from
    ``steps[s] = (a, b)``. ``node_wires[x]`` is the wire set of node ``x``;
    ``summed[s]`` the wires summed at step ``s``.
    """

    num_leaves: int
    steps: list[tuple[int, int]]
    node_wires: list[frozenset[int]]
    out_wires: tuple[int, ...]

    @property
    def root(self) -> int:
        return self.num_leaves + len(self.steps) - 1

    def step_union(self, s: int) -> frozenset[int]:
        a, b = self.steps[s]
        return self.node_wires[a] | self.node_wires[b]

    def summed(self, s: int) -> frozenset[int]:
        return self.step_union(s) - self.node_wires[self.num_leaves + s]

    def cost(self, sliced: frozenset[int] = frozenset()) -> tuple[float, int, float]:
        """(log2 total index-space size, max intermediate bits, log2 written entries)."""
        tot = 0.0
        wr = 0.0
        peak = 0
        L = self.num_leaves
        for s in range(len(self.steps)):
            u = len(self.step_union(s) - sliced)
            o = len(self.node_wires[L + s] - sliced)
            tot += 2.0**u
            wr += 2.0**o
            peak = max(peak, o)
        return (math.log2(tot) if tot > 0 else 0.0, peak, math.log2(wr) if wr > 0 else 0.0)

    def linear_path(self) -> tuple[tuple[int, int], ...]:
        """The tree as an opt_einsum-style pop/append path (the format of
        ``SimpleContraction``, ``tensorsat/contractions/simple.py:38-46``)."""
        live = list(range(self.num_leaves))
        path = []
        for s, (a, b) in enumerate(self.steps):
            i = live.index(a)
            j = live.index(b)
            path.append((i, j))
            for x in sorted((i, j), reverse=True):
                live.pop(x)
            live.append(self.num_leaves + s)
        return tuple(path)


PLAN_FORMAT = "tensorsat_gb300.plan/1"


def plan_to_dict(tree: ContractionTree, sliced: Sequence[int]) -> dict:
    """A tree and its sliced wires as plain JSON data (format ``PLAN_FORMAT``)."""
    return {
        "format": PLAN_FORMAT,
        "num_leaves": tree.num_leaves,
        "steps": [list(ab) for ab in tree.steps],
        "node_wires": [sorted(ws) for ws in tree.node_wires],
        "out_wires": list(tree.out_wires),
        "sliced": sorted(int(w) for w in sliced),
    }


def plan_from_dict(data: dict) -> tuple[ContractionTree, tuple[int, ...]]:
    """Inverse of :func:`plan_to_dict`; raises ValueError on another format or a
    malformed tree (steps must consume earlier nodes, node wire sets must match)."""
    if not isinstance(data, dict) or data.get("format") != PLAN_FORMAT:
        raise ValueError(f"not a {PLAN_FORMAT} plan")
    L = int(data["num_leaves"])
    steps = [(int(a), int(b)) for a, b in data["steps"]]
    node_wires = [frozenset(int(w) for w in ws) for ws in data["node_wires"]]
    if len(node_wires) != L + len(steps):
        raise ValueError("plan: node_wires must list every leaf and step")
    for s, (a, b) in enumerate(steps):
        if not (0 <= a < L + s and 0 <= b < L + s and a != b):
            raise ValueError(f"plan: step {s} must combine two earlier nodes")
    tree = ContractionTree(L, steps, node_wires, tuple(int(w) for w in data["out_wires"]))
    return tree, tuple(int(w) for w in data["sliced"])


def _primal(tensors: dict[int, frozenset[int]], protect: frozenset[int]) -> dict[int, set[int]]:
    adj: dict[int, set[int]] = {}
    for ws in tensors.values():
        for w in ws:
            if w in protect:
                continue
            nb = adj.setdefault(w, set())
            nb.update(x for x in ws if x != w and x not in protect)
    return adj


def build_tree(net: Network, order: Sequence[int]) -> ContractionTree:
    """Builds the contraction tree that eliminates wires in ``order``.

    Eliminating wire ``w`` merges every remaining tensor that carries ``w``, pairwise,
    smallest union first. Leftover tensors (disjoint components, output-only tensors) are
    merged at the end by smallest union.
    """
    L = len(net.leaf_wires)
    out = frozenset(net.out_wires)
    node_wires: list[frozenset[int]] = [frozenset(ws) for ws in net.leaf_wires]
    live: dict[int, frozenset[int]] = {i: node_wires[i] for i in range(L)}
    holders: dict[int, set[int]] = {}
    for i, ws in live.items():
        for w in ws:
            holders.setdefault(w, set()).add(i)
    steps: list[tuple[int, int]] = []

    def merge(a: int, b: int) -> int:
        wa, wb = live.pop(a), live.pop(b)
        union = wa | wb
        keep = []
        for w in union:
            hs = holders[w]
            hs.discard(a)
            hs.discard(b)
            if hs or w in out:
                keep.append(w)
        x = L + len(steps)
        steps.append((a, b))
        res = frozenset(keep)
        node_wires.append(res)
        live[x] = res
        for w in res:
            holders[w].add(x)
        return x

    def merge_group(group: list[int]) -> None:
        group = list(group)
        while len(group) > 1:
            best = None
            for i in range(len(group)):
                wi = live[group[i]]
                for j in range(i + 1, len(group)):
                    u = len(wi | live[group[j]])
                    if best is None or u < best[0]:
                        best = (u, i, j)
            _, i, j = best
            a, b = group[i], group[j]
            x = merge(a, b)
            group = [g for k, g in enumerate(group) if k not in (i, j)] + [x]

    for w in order:
        hs = holders.get(w)
        if not hs or len(hs) < 2:
            continue
        merge_group(sorted(hs, key=lambda i: (len(live[i]), i)))
    rest = sorted(live, key=lambda i: (len(live[i]), i))
    merge_group(rest)
    return ContractionTree(L, steps, node_wires, tuple(net.out_wires))


def simplify_order(net: Network) -> list[int]:
    """Growth-free eliminations: wires whose elimination yields a tensor no larger than
    the largest tensor it absorbs (gates, NOT/unit tensors, clause trees)."""
    out = frozenset(net.out_wires)
    tensors = {i: frozenset(ws) for i, ws in enumerate(net.leaf_wires)}
    holders: dict[int, set[int]] = {}
    for i, ws in tensors.items():
        for w in ws:
            holders.setdefault(w, set()).add(i)
    order: list[int] = []
    nxt = len(tensors)
    changed = True
    while changed:
        changed = False
        for w in sorted(holders):
            if w in out:
                continue
            hs = holders[w]
            if not hs:
                continue
            union = frozenset().union(*(tensors[i] for i in hs))
            # wires still needed outside this bucket
            res = frozenset(
                x for x in union if x in out or (holders[x] - hs)
            )
            if len(res) <= max(len(tensors[i]) for i in hs):
                order.append(w)
                for i in list(hs):
                    for x in tensors[i]:
                        holders[x].discard(i)
                    del tensors[i]
                tensors[nxt] = res
                for x in res:
                    holders[x].add(nxt)
                for x in union - res:
                    holders[x].clear()
                nxt += 1
                changed = True
    return order


def minfill_order(net: Network, rng: random.Random, prefix: Sequence[int] = ()) -> list[int]:
    """Min-fill elimination order (ties broken at random) of the non-output wires,
    starting after the eliminations in ``prefix``."""
    out = frozenset(net.out_wires)
    # replay the prefix on the hypergraph
    tensors = {i: frozenset(ws) for i, ws in enumerate(net.leaf_wires)}
    holders: dict[int, set[int]] = {}
    for i, ws in tensors.items():
        for w in ws:
            holders.setdefault(w, set()).add(i)
    nxt = len(tensors)
    done: set[int] = set()
    for w in prefix:
        hs = holders.get(w, set())
        done.add(w)
        if not hs:
            continue
        union = frozenset().union(*(tensors[i] for i in hs))
        res = frozenset(x for x in union if x in out or (holders[x] - hs))
        for i in list(hs):
            for x in tensors[i]:
                holders[x].discard(i)
            del tensors[i]
        tensors[nxt] = res
        for x in res:
            holders[x].add(nxt)
        nxt += 1
        done.update(union - res)
    adj = _primal(tensors, out)
    for w in list(adj):
        if w in done:
            del adj[w]
    for w in adj:
        adj[w] -= done
    order = list(prefix)
    alive = set(adj)
    while alive:
        best = None
        cands: list[int] = []
        for v in alive:
            nb = adj[v]
            nbl = list(nb)
            f = 0
            for i in range(len(nbl)):
                ai = adj[nbl[i]]
                for j in range(i + 1, len(nbl)):
                    if nbl[j] not in ai:
                        f += 1
            key = (f, len(nb))
            if best is None or key < best:
                best = key
                cands = [v]
            elif key == best:
                cands.append(v)
        v = rng.choice(cands)
        nb = list(adj[v])
        for a in nb:
            adj[a].discard(v)
            for b in nb:
                if a != b:
                    adj[a].add(b)
        alive.discard(v)
        del adj[v]
        order.append(v)
    return order


def subset_dp(n: int, num_wires: int, bits: Sequence[int], keep: int, live: int,
              max_bits: int | None) -> tuple[float, np.ndarray, np.ndarray]:
    """Cheapest binary contraction of ``n`` inputs by dynamic programming over their
    subsets (native ``tsg_plan_subset_dp``). Wire sets are Python ints over
    ``num_wires`` bit positions: ``bits[i]`` the wires of input i, ``keep`` the wires the
    result keeps, ``live`` the unsliced ones. Returns (total cost, split, kept): the cost
    is the sum over steps of 2^(live wires of both operands), ``split[m]`` the part of
    subset m holding its lowest input in m's cheapest split, ``kept[m]`` (uint64 words)
    the wires m's partial result keeps (those of m that ``keep`` or an input outside m
    carries). With ``max_bits`` no partial result but the whole may keep more than
    ``max_bits`` live wires (cost infinity when that cannot be met)."""
    words = max(1, (num_wires + 63) // 64)
    mask = (1 << 64) - 1

    def to_words(v: int) -> list[int]:
        return [(v >> (64 * w)) & mask for w in range(words)]

    b = np.array([to_words(v) for v in bits], dtype=np.uint64).reshape(-1)
    k = np.array(to_words(keep), dtype=np.uint64)
    lv = np.array(to_words(live), dtype=np.uint64)
    split = np.zeros(1 << n, dtype=np.uint32)
    kept = np.zeros((1 << n) * words, dtype=np.uint64)
    best = ctypes.c_double()
    u64p = ctypes.POINTER(ctypes.c_uint64)
    _native.check(_native.lib().tsg_plan_subset_dp(
        n, words, b.ctypes.data_as(u64p), k.ctypes.data_as(u64p), lv.ctypes.data_as(u64p),
        -1 if max_bits is None else int(max_bits), ctypes.byref(best),
        split.ctypes.data_as(ctypes.POINTER(ctypes.c_uint32)), kept.ctypes.data_as(u64p)))
    return best.value, split, kept.reshape(1 << n, words)


def reconfigure(tree: ContractionTree, subtree_size: int = 10, passes: int = 4,
                sliced: frozenset[int] = frozenset(), max_bits: int | None = None
                ) -> ContractionTree:
    """Subtree reconfiguration. For every internal node x, the subtree below x is cut at
    up to ``subtree_size`` (at most 20) inputs (expanding its most expensive steps first)
    and replaced by the cheapest binary contraction of those inputs, found by dynamic
    programming over subsets (:func:`subset_dp`). A partial contraction of a subset S keeps a wire when x keeps it or an input
    outside S carries it. Cost is the tree's index-space cost per slice: the sum over
    steps of 2^|wires of both operands, sliced wires excluded|. With ``max_bits`` no new
    intermediate may exceed 2^max_bits entries per slice. The root and every leaf are
    unchanged, so the answers are too."""
    if subtree_size > 20:
        raise ValueError("subtree_size must be at most 20")
    L = tree.num_leaves
    wires: dict[int, frozenset[int]] = dict(enumerate(tree.node_wires))
    children: dict[int, tuple[int, int]] = {L + s: ab for s, ab in enumerate(tree.steps)}
    root = tree.root
    next_id = L + len(tree.steps)

    def step_cost(x: int) -> float:
        a, b = children[x]
        return 2.0 ** len((wires[a] | wires[b]) - sliced)

    for _ in range(max(0, passes)):
        improved = False
        todo = [root]
        seen = []
        while todo:  # internal nodes, root first
            x = todo.pop()
            seen.append(x)
            for c in children[x]:
                if c in children:
                    todo.append(c)
        for x in seen:
            if x not in children:
                continue  # removed by an earlier replacement
            frontier = list(children[x])
            internal = [x]
            while len(frontier) < subtree_size:
                inner = [f for f in frontier if f in children]
                if not inner:
                    break
                big = max(inner, key=step_cost)
                frontier.remove(big)
                internal.append(big)
                frontier.extend(children[big])
            n = len(frontier)
            if n < 3:
                continue
            old = sum(step_cost(y) for y in internal)
            # wires as bit sets over the wires present in the subtree
            index: dict[int, int] = {}
            for f in frontier:
                for w in wires[f]:
                    index.setdefault(w, len(index))
            bits = [sum(1 << index[w] for w in wires[f]) for f in frontier]
            keep_x = sum(1 << index[w] for w in wires[x] if w in index)
            live = sum(1 << i for w, i in index.items() if w not in sliced)
            full = (1 << n) - 1
            best_full, split, kept = subset_dp(n, len(index), bits, keep_x, live, max_bits)
            if not best_full < old * (1 - 1e-9):
                continue
            # rebuild the subtree below x from the splits; x keeps its id and wires
            for y in internal:
                if y != x:
                    del children[y]
                    del wires[y]

            def build(m: int) -> int:
                nonlocal next_id
                if m & (m - 1) == 0:
                    return frontier[m.bit_length() - 1]
                a = int(split[m])
                na, nb = build(a), build(m ^ a)
                if m == full:
                    y = x
                else:
                    y = next_id
                    next_id += 1
                    inv = {v: k for k, v in index.items()}
                    km = sum(int(k) << (64 * w) for w, k in enumerate(kept[m]))
                    wires[y] = frozenset(inv[i] for i in range(km.bit_length()) if km >> i & 1)
                children[y] = (na, nb)
                return y

            build(full)
            improved = True
        if not improved:
            break
    # re-linearise in post order: leaves keep their ids, steps are numbered L + s
    steps: list[tuple[int, int]] = []
    node_wires = [tree.node_wires[i] for i in range(L)]
    new_id: dict[int, int] = {i: i for i in range(L)}
    stack = [(root, False)]
    while stack:
        x, done = stack.pop()
        if x in new_id:
            continue
        a, b = children[x]
        if done:
            steps.append((new_id[a], new_id[b]))
            new_id[x] = L + len(steps) - 1
            node_wires.append(wires[x])
        else:
            stack.append((x, True))
            stack.append((b, False))
            stack.append((a, False))
    return ContractionTree(L, steps, node_wires, tree.out_wires)


class _WireMatrix:
    """The steps' wire sets of a tree as 0/1 matrices over its wires (rows: steps), for
    evaluating many candidate slicings at once. Sums over steps run in step order
    (sequential accumulation), so every value equals :meth:`ContractionTree.cost`'s."""

    def __init__(self, tree: ContractionTree) -> None:
        L = tree.num_leaves
        self.wires = sorted(set().union(*tree.node_wires)) if tree.node_wires else []
        col = {w: i for i, w in enumerate(self.wires)}
        n = len(tree.steps)
        self.union = np.zeros((n, len(self.wires)), dtype=np.int64)
        self.out = np.zeros((n, len(self.wires)), dtype=np.int64)
        for s in range(n):
            for w in tree.step_union(s):
                self.union[s, col[w]] = 1
            for w in tree.node_wires[L + s]:
                self.out[s, col[w]] = 1
        self.col = col

    def sizes(self, sliced: Sequence[int]) -> tuple[np.ndarray, np.ndarray]:
        """Per step: unsliced wires of the step's index space and of its result."""
        u = self.union.sum(axis=1)
        o = self.out.sum(axis=1)
        for w in sliced:
            if w in self.col:
                u = u - self.union[:, self.col[w]]
                o = o - self.out[:, self.col[w]]
        return u, o


def _log2_total(u: np.ndarray) -> np.ndarray:
    """log2 of the sum over steps (axis 0, in step order) of 2^u, per column; 0 for an
    empty sum, like :meth:`ContractionTree.cost`."""
    if u.shape[0] == 0:
        return np.zeros(u.shape[1:])
    tot = np.add.accumulate(np.ldexp(1.0, u), axis=0)[-1]  # exact powers, summed in order
    return np.array([math.log2(t) if t > 0 else 0.0 for t in np.atleast_1d(tot)]).reshape(
        np.shape(tot))


def slice_tree(tree: ContractionTree, target_bits: int, forbid: frozenset[int] = frozenset()
               ) -> frozenset[int]:
    """Greedy slicing: repeatedly slice the wire of a largest intermediate that lowers the
    peak most, breaking ties by the smallest total (all-slices) cost (then the smallest
    wire). All candidate wires of a round are evaluated at once on the steps' wire
    matrices."""
    m = _WireMatrix(tree)
    sliced: list[int] = []
    u, o = m.sizes(())
    while True:
        peak = int(o.max()) if o.size else 0
        if peak <= target_bits:
            return frozenset(sliced)
        at_peak = o == peak
        cands = sorted(w for w in m.wires
                       if w not in forbid and w not in sliced and
                       bool(m.out[at_peak, m.col[w]].any()))
        if not cands:
            raise ValueError(
                f"cannot slice below 2^{peak} entries: the largest intermediates only carry"
                " output wires"
            )
        cols = [m.col[w] for w in cands]
        u2 = u[:, None] - m.union[:, cols]
        p2 = (o[:, None] - m.out[:, cols]).max(axis=0)
        t2 = _log2_total(u2)
        best = None
        for i, w in enumerate(cands):
            key = (int(p2[i]), float(t2[i]) + len(sliced) + 1)
            if best is None or key < best[0]:
                best = (key, w)
        w = best[1]
        sliced.append(w)
        u = u - m.union[:, m.col[w]]
        o = o - m.out[:, m.col[w]]


def unslice(tree: ContractionTree, sliced: frozenset[int], target_bits: int) -> frozenset[int]:
    """Drops sliced wires that are no longer needed to keep every intermediate within
    2^target_bits entries (each dropped wire halves the number of slices)."""
    m = _WireMatrix(tree)
    sl = set(sliced)
    _, o = m.sizes(sorted(sl))
    for w in sorted(sliced):
        back = o + (m.out[:, m.col[w]] if w in m.col else 0)
        if (int(back.max()) if back.size else 0) <= target_bits:
            sl.discard(w)
            o = back
    return frozenset(sl)


def plan_bytes(tree: ContractionTree, sliced: frozenset[int]) -> float:
    """Algorithmic HBM bytes of the whole contraction (every slice; 4-byte intermediates,
    1-byte leaves): each step reads both operands and writes its result once."""
    L = tree.num_leaves
    tot = 0.0
    for s, (a, b) in enumerate(tree.steps):
        for x in (a, b):
            tot += 2.0 ** len(tree.node_wires[x] - sliced) * (1 if x < L else 4)
        tot += 2.0 ** len(tree.node_wires[L + s] - sliced) * 4
    return tot * 2.0 ** len(sliced)


def optimize(net: Network, *, target_bits: int | None = 26, trials: int = 8, seed: int = 0,
             method: str = "minfill", reconf: int = 10) -> tuple[ContractionTree, frozenset[int]]:
    """Searches ``trials`` randomized elimination orders and returns the best (tree,
    sliced wires) by (peak bits after slicing, total bytes over all slices).

    Each order's tree is improved by subtree reconfiguration (subtrees of up to ``reconf``
    inputs; 0 turns it off), sliced to ``target_bits``, reconfigured again under that
    slicing (no intermediate above the cap), and freed of sliced wires it no longer
    needs."""
    rng = random.Random(seed)
    prefix = simplify_order(net)
    forbid = frozenset(net.out_wires)
    if target_bits is not None:
        # the root holds every output wire: no slicing can go below that
        target_bits = max(target_bits, len(forbid))
    best = None
    for t in range(max(1, trials)):
        if method != "minfill":
            raise ValueError(f"unknown optimisation method {method!r}")
        order = minfill_order(net, rng, prefix)
        tree = build_tree(net, order)
        if reconf >= 3:
            tree = reconfigure(tree, reconf)
        if target_bits is None:
            sliced = frozenset()
        else:
            sliced = slice_tree(tree, target_bits, forbid)
            if reconf >= 3 and sliced:
                tree = reconfigure(tree, reconf, sliced=sliced, max_bits=target_bits)
                sliced = unslice(tree, sliced, target_bits)
        peak = tree.cost(sliced)[1]
        key = (peak, plan_bytes(tree, sliced))
        if best is None or key < best[0]:
            best = (key, tree, sliced)
    return best[1], best[2]


@dataclass
class SlicedPlan:
    """A tree, its sliced wires, and the wire order (layout) of every node.

    Leaves keep their given wire order (sliced wires included). Intermediates are laid
    out top down, each from its consumer's needs: the root follows the output wires; in a
    step whose result order is fixed, the larger operand (the one carrying more result
    wires) takes the result's order for its kept wires, with its summed wires above them;
    the smaller operand takes ``new wires (not in the larger) | summed wires | shared
    wires in the result's order``. Along a chain of steps the lowest bits are therefore
    the longest-lived wires, so the large operand reads coalesce and match the output
    (vector loads), and the small operand either follows the same low wires or does not
    carry them (one load serves several outputs).
    """

    tree: ContractionTree
    sliced: tuple[int, ...]
    leaf_wires: list[tuple[int, ...]]
    node_order: list[tuple[int, ...]] = field(default_factory=list)

    def __post_init__(self) -> None:
        t = self.tree
        L = t.num_leaves
        sl = frozenset(self.sliced)
        n_nodes = L + len(t.steps)
        order: list[tuple[int, ...] | None] = [None] * n_nodes
        for l, ws in enumerate(self.leaf_wires):
            order[l] = tuple(ws)
        if t.steps:
            order[n_nodes - 1] = tuple(dict.fromkeys(t.out_wires))
        for s in range(len(t.steps) - 1, -1, -1):
            out_order = [w for w in order[L + s] if w not in sl]
            out_set = frozenset(out_order)
            a, b = t.steps[s]
            wa = t.node_wires[a] - sl
            wb = t.node_wires[b] - sl
            ca = len(wa & out_set)
            cb = len(wb & out_set)
            big, small = (a, b) if (ca, len(wa)) >= (cb, len(wb)) else (b, a)
            wbig = wa if big == a else wb
            wsmall = wb if big == a else wa
            summed = sorted((wa | wb) - out_set)
            if big >= L:
                kept = [w for w in out_order if w in wbig]
                top = [w for w in summed if w in wbig]
                order[big] = tuple(top + kept)
                assert frozenset(order[big]) == wbig
            if small >= L:
                new = [w for w in out_order if w in wsmall and w not in wbig]
                mid = [w for w in summed if w in wsmall]
                shared = [w for w in out_order if w in wsmall and w in wbig]
                order[small] = tuple(new + mid + shared)
                assert frozenset(order[small]) == wsmall
        self.node_order = [o if o is not None else () for o in order]

    @property
    def num_slices(self) -> int:
        return 1 << len(self.sliced)

    def step_bits(self, s: int) -> tuple[list[int], list[int]]:
        """(output wires by bit index, summed wires by bit index) of step ``s``."""
        t = self.tree
        L = t.num_leaves
        outw = list(reversed(self.node_order[L + s]))  # bit i = wire order[-1-i]
        sl = frozenset(self.sliced)
        summed = sorted(t.step_union(s) - t.node_wires[L + s] - sl)
        return outw, summed

    def native_arrays(self) -> dict[str, np.ndarray]:
        """Integer arrays for ``tsg_plan_create`` (leaf offsets are left to the caller)."""
        t = self.tree
        L = t.num_leaves
        nsl = len(self.sliced)
        slice_index = {w: j for j, w in enumerate(self.sliced)}
        leaf_ranks = np.array([len(ws) for ws in self.leaf_wires], dtype=np.int32)
        leaf_slice_pos = np.full((L, max(nsl, 1)), -1, dtype=np.int32)
        for l, ws in enumerate(self.leaf_wires):
            r = len(ws)
            for i, w in enumerate(ws):
                j = slice_index.get(w)
                if j is not None:
                    leaf_slice_pos[l, j] = r - 1 - i
        ns = len(t.steps)
        ops = np.zeros((ns, 2), dtype=np.int32)
        out_bits = np.zeros(ns, dtype=np.int32)
        sum_bits = np.zeros(ns, dtype=np.int32)
        pos = np.full((2, ns, TSG_MAX_BITS), -1, dtype=np.int32)
        for s, (a, b) in enumerate(t.steps):
            outw, summed = self.step_bits(s)
            if len(outw) + len(summed) > TSG_MAX_BITS:
                raise ValueError("a contraction step exceeds 62 index bits")
            out_bits[s] = len(outw)
            sum_bits[s] = len(summed)
            for o, x in enumerate((a, b)):
                ops[s, o] = x if x < L else -(x - L) - 1
                xo = self.node_order[x]
                r = len(xo)
                bitpos = {w: r - 1 - i for i, w in enumerate(xo)}
                for i, w in enumerate(list(outw) + list(summed)):
                    p = bitpos.get(w)
                    if p is not None:
                        pos[o, s, i] = p
        return {
            "leaf_ranks": leaf_ranks,
            "leaf_slice_pos": np.ascontiguousarray(leaf_slice_pos[:, :nsl]) if nsl else
            np.zeros((L, 0), dtype=np.int32),
            "step_operands": ops,
            "step_out_bits": out_bits,
            "step_sum_bits": sum_bits,
            "step_lhs_pos": np.ascontiguousarray(pos[0]),
            "step_rhs_pos": np.ascontiguousarray(pos[1]),
        }

    def step_bytes_per_slice(self, elem_bytes: int, planes: int = 1,
                             fused: dict[int, int] | None = None) -> list[float]:
        """Algorithmic HBM bytes of each step for one slice: the step reads both operands
        once and writes its result once (leaves are uint8, other tensors elem_bytes *
        planes). ``fused`` maps a consumer step to the producer step it computes itself:
        the producer then moves nothing, and the consumer reads the producer's two
        operands instead of the producer's result."""
        t = self.tree
        L = t.num_leaves
        sl = frozenset(self.sliced)
        fused = fused or {}
        away = set(fused.values())

        def size(x: int) -> float:
            n = 2.0 ** len(t.node_wires[x] - sl)
            return n if x < L else n * elem_bytes * planes

        out = []
        for s, (a, b) in enumerate(t.steps):
            if s in away:
                out.append(0.0)
                continue
            tot = 0.0
            for x in (a, b):
                if x >= L and x - L == fused.get(s):
                    tot += sum(size(y) for y in t.steps[x - L])
                else:
                    tot += size(x)
            tot += size(L + s)
            out.append(tot)
        return out

    def bytes_per_slice(self, elem_bytes: int, planes: int = 1,
                        fused: dict[int, int] | None = None) -> float:
        """Algorithmic HBM bytes of one slice, all steps (see step_bytes_per_slice)."""
        return float(sum(self.step_bytes_per_slice(elem_bytes, planes, fused)))
