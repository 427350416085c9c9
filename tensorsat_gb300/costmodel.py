"""Learned cost model: a message-passing network over contraction trees that predicts a
tree's device time per slice, used to rank candidate trees of an instance.

The reference picks trees with cotengra's hyper-optimiser
(``tensorsat/contractions/cotengra.py:78-85``), absent here; the project's planner ranks its
candidates by algorithmic bytes. This model is trained on the solver's own measurements
(``tsg_plan_run_timed`` of each candidate tree on the GPU) and ranks candidates by
predicted time; the planner's ranking stays the fallback. Answers never depend on it:
every tree gives the same SAT bit and count.

Network (hidden width 128, BF16 weights and activations, FP32 accumulation):

* the graph is the contraction tree: one node per leaf (a clause or gate tensor of the
  instance's hypergraph) and per step, edges from each step to its two operands;
* node features: leaf rank and live bits; for a step its output, summed and operand bits,
  slice dependence, algorithmic bytes, and the kernel family and template parameters the
  executor chose for it in the count ring and in the OR-AND ring (``tsg_plan_describe``);
* an input layer, then 3 message-passing layers h <- ReLU([h | sum of children's h] W + b),
  then a sum over the tree's nodes and a linear head: the predicted log device time per
  slice (count ring with 3 primes plus the OR-AND ring).

The dense layers run on the tensor cores (``tsg_cm_gemm_bf16``: tcgen05.mma kind::f16,
FP32 accumulation in tensor memory); the children sums, their transpose, the weight
gradients and Adam are the library's own kernels (``tsg_cm_*``). PyTorch only holds the
buffers and does the small glue (casts, masks, the per-tree sums of the readout).
"""

from __future__ import annotations

import math
from dataclasses import dataclass
from typing import Any, Sequence

import numpy as np
import torch

from . import _device, _native, planner

HIDDEN = 128
FEATURES = 64  # node feature width (zero-padded; a multiple of the GEMM's K step)
LAYERS = 3
NUM_PRIMES = 3


# -- graphs ----------------------------------------------------------------------------


def _family_onehot(kind: Sequence[int]) -> list[float]:
    v = [0.0] * 6
    fam = int(kind[0])
    if 0 <= fam < 6:
        v[fam] = 1.0
    return v + [int(kind[1]) / 16.0, int(kind[2]) / 4.0, int(kind[3]) / 16.0]


def tree_graph(contraction: Any, group: int, primes: Sequence[int]) -> dict:
    """Node features and child lists of a contraction's tree (host only).

    Returns ``x`` (nodes x FEATURES float32), ``children`` (per node its operand nodes)
    and ``slices`` (the tree's slice count)."""
    tree = contraction.tree
    L = tree.num_leaves
    sl = frozenset(contraction.sliced_wires)
    npl = contraction.native_plan()
    km = npl.describe(_native.TSG_RING_MODP, primes, group)
    ko = npl.describe(_native.TSG_RING_OR_AND, (), group)
    bytes_m = contraction.sliced_plan.step_bytes_per_slice(4, len(primes))
    n = L + len(tree.steps)
    x = np.zeros((n, FEATURES), dtype=np.float32)
    dep = [bool(tree.node_wires[i] & sl) for i in range(L)] + [False] * len(tree.steps)
    children: list[tuple[int, ...]] = [()] * n
    for i in range(L):
        rank = len(tree.node_wires[i])
        live = len(tree.node_wires[i] - sl)
        x[i, :4] = [1.0, rank / 32.0, live / 32.0, float(dep[i])]
    for s, (a, b) in enumerate(tree.steps):
        v = L + s
        dep[v] = dep[a] or dep[b]
        out = len(tree.node_wires[v] - sl)
        k = len(tree.step_union(s) - tree.node_wires[v] - sl)
        la = len(tree.node_wires[a] - sl)
        lb = len(tree.node_wires[b] - sl)
        feats = [0.0, 1.0, out / 32.0, k / 8.0, (out + k) / 32.0, la / 32.0, lb / 32.0,
                 float(dep[v]), math.log2(max(bytes_m[s], 1.0)) / 40.0,
                 float(a < L), float(b < L)]
        feats += _family_onehot(km[s]) + _family_onehot(ko[s])
        x[v, :len(feats)] = feats
        children[v] = (a, b)
    return {"x": x, "children": children, "slices": contraction.num_slices}


@dataclass
class Batch:
    """Several trees as one node array padded to a multiple of 128 rows."""

    x: torch.Tensor          # (Np, FEATURES) bf16
    x32: torch.Tensor        # (Np, FEATURES) fp32
    cstart: torch.Tensor     # (Np + 1,) int32, CSR of children
    child: torch.Tensor      # (E,) int32
    parent: torch.Tensor     # (Np,) int32, -1 for roots and padding
    graph: torch.Tensor      # (Np,) int64 graph of each node (padding: G, dropped)
    graphs: int
    nodes: int


def make_batch(graphs: Sequence[dict], device: torch.device) -> Batch:
    n = sum(g["x"].shape[0] for g in graphs)
    npad = max(128, (n + 127) // 128 * 128)
    x = np.zeros((npad, FEATURES), dtype=np.float32)
    parent = np.full(npad, -1, dtype=np.int32)
    gid = np.full(npad, len(graphs), dtype=np.int64)
    counts = np.zeros(npad + 1, dtype=np.int64)
    child = []
    off = 0
    for gi, g in enumerate(graphs):
        m = g["x"].shape[0]
        x[off: off + m] = g["x"]
        gid[off: off + m] = gi
        for v, ch in enumerate(g["children"]):
            counts[off + v + 1] = len(ch)
            for u in ch:
                child.append(off + u)
                parent[off + u] = off + v
        off += m
    cstart = np.cumsum(counts).astype(np.int32)
    xt = torch.from_numpy(x).to(device)
    return Batch(xt.to(torch.bfloat16), xt, torch.from_numpy(cstart).to(device),
                 torch.from_numpy(np.asarray(child or [0], dtype=np.int32)).to(device),
                 torch.from_numpy(parent).to(device), torch.from_numpy(gid).to(device),
                 len(graphs), n)


# -- the network -----------------------------------------------------------------------


def _gemm(a: torch.Tensor, b: torch.Tensor, bias: torch.Tensor | None, relu: bool,
          out: torch.Tensor) -> torch.Tensor:
    """out = a @ b.T (+ bias, ReLU) on the tensor cores; a (M x K) and b (N x K) BF16."""
    m, k = a.shape
    n = b.shape[0]
    _native.check(_native.lib().tsg_cm_gemm_bf16(
        m, n, k, a.data_ptr(), b.data_ptr(), None if bias is None else bias.data_ptr(),
        int(relu), out.data_ptr(), out.stride(0), int(out.dtype == torch.float32),
        _device.stream_handle()))
    return out


class CostModel:
    """3-layer message-passing cost model (see the module docstring)."""

    def __init__(self, seed: int = 0, device: torch.device | None = None) -> None:
        self.device = device or _device.require_cuda()
        g = torch.Generator().manual_seed(seed)

        def init(rows: int, cols: int) -> torch.Tensor:
            return (torch.randn(rows, cols, generator=g) * math.sqrt(2.0 / cols)).to(self.device)

        # FP32 master weights, stored out x in (the GEMM's K-contiguous B operand)
        self.params: dict[str, torch.Tensor] = {"w_in": init(HIDDEN, FEATURES),
                                                "b_in": torch.zeros(HIDDEN, device=self.device)}
        for l in range(LAYERS):
            self.params[f"w{l}"] = init(HIDDEN, 2 * HIDDEN)
            self.params[f"b{l}"] = torch.zeros(HIDDEN, device=self.device)
        self.params["w_out"] = (torch.randn(HIDDEN, generator=g) * 0.01).to(self.device)
        self.params["b_out"] = torch.zeros(1, device=self.device)
        self.adam = {k: (torch.zeros_like(v), torch.zeros_like(v)) for k, v in self.params.items()}
        self.step = 0
        self.y_mean = 0.0
        self.y_std = 1.0

    def _bf16(self, name: str) -> torch.Tensor:
        return self.params[name].to(torch.bfloat16).contiguous()

    def forward(self, batch: Batch, keep: bool = False):
        """Predicted (normalised) log time per tree; with ``keep`` also the activations the
        backward pass needs."""
        np_ = batch.x.shape[0]
        lib = _native.lib()
        stream = _device.stream_handle()
        h = torch.empty((np_, HIDDEN), dtype=torch.bfloat16, device=self.device)
        _gemm(batch.x, self._bf16("w_in"), self.params["b_in"], True, h)
        acts = [h]
        hcs = []
        for l in range(LAYERS):
            hc = torch.empty((np_, 2 * HIDDEN), dtype=torch.bfloat16, device=self.device)
            hc[:, :HIDDEN] = h
            _native.check(lib.tsg_cm_child_sum(h.data_ptr(), batch.cstart.data_ptr(),
                                               batch.child.data_ptr(), hc[:, HIDDEN:].data_ptr(),
                                               np_, HIDDEN, 2 * HIDDEN, stream))
            h = torch.empty((np_, HIDDEN), dtype=torch.bfloat16, device=self.device)
            _gemm(hc, self._bf16(f"w{l}"), self.params[f"b{l}"], True, h)
            hcs.append(hc)
            acts.append(h)
        hf = h.float()
        pooled = torch.zeros((batch.graphs + 1, HIDDEN), device=self.device)
        pooled.index_add_(0, batch.graph, hf)
        pooled = pooled[: batch.graphs]
        pred = pooled @ self.params["w_out"] + self.params["b_out"]
        if keep:
            return pred, {"acts": acts, "hcs": hcs, "pooled": pooled}
        return pred

    def _backward(self, batch: Batch, cache: dict, dpred: torch.Tensor) -> dict:
        lib = _native.lib()
        stream = _device.stream_handle()
        np_ = batch.x.shape[0]
        grads = {"w_out": cache["pooled"].T @ dpred, "b_out": dpred.sum().reshape(1)}
        dpool = dpred[:, None] * self.params["w_out"][None, :]
        zero = torch.zeros((1, HIDDEN), device=self.device)
        dh = torch.cat([dpool, zero])[batch.graph]  # (Np, HIDDEN) fp32; padding rows 0
        for l in reversed(range(LAYERS)):
            out = cache["acts"][l + 1]
            dz = dh * (out > 0).float()
            hc = cache["hcs"][l]
            gw = torch.empty((HIDDEN, 2 * HIDDEN), device=self.device)
            hc32 = hc.float().contiguous()
            _native.check(lib.tsg_cm_gemm_at_b(dz.data_ptr(), HIDDEN, hc32.data_ptr(),
                                               2 * HIDDEN, np_, gw.data_ptr(), stream))
            grads[f"w{l}"] = gw
            grads[f"b{l}"] = dz.sum(0)
            # d[h | c] = dz @ W: two tensor-core GEMMs of 128 output columns each (B = W^T
            # halves, K = HIDDEN contiguous)
            wt = self.params[f"w{l}"].T.contiguous().to(torch.bfloat16)  # (2H, H)
            dhc = torch.empty((np_, 2 * HIDDEN), dtype=torch.float32, device=self.device)
            dzb = dz.to(torch.bfloat16).contiguous()
            _gemm(dzb, wt[:HIDDEN].contiguous(), None, False, dhc[:, :HIDDEN])
            _gemm(dzb, wt[HIDDEN:].contiguous(), None, False, dhc[:, HIDDEN:])
            dh = dhc[:, :HIDDEN].contiguous()
            dc = dhc[:, HIDDEN:].contiguous()
            _native.check(lib.tsg_cm_parent_add(dc.data_ptr(), HIDDEN, batch.parent.data_ptr(),
                                                dh.data_ptr(), np_, HIDDEN, stream))
        out = cache["acts"][0]
        dz = dh * (out > 0).float()
        gw = torch.empty((HIDDEN, FEATURES), device=self.device)
        _native.check(lib.tsg_cm_gemm_at_b(dz.data_ptr(), HIDDEN, batch.x32.data_ptr(), FEATURES,
                                           np_, gw.data_ptr(), stream))
        grads["w_in"] = gw
        grads["b_in"] = dz.sum(0)
        return grads

    def train_step(self, batch: Batch, y: torch.Tensor, lr: float = 1e-3) -> float:
        """One Adam step on the mean squared error of the normalised log times."""
        pred, cache = self.forward(batch, keep=True)
        yn = (y - self.y_mean) / self.y_std
        err = pred - yn
        loss = float((err * err).mean())
        grads = self._backward(batch, cache, 2.0 * err / err.numel())
        self.step += 1
        lib = _native.lib()
        stream = _device.stream_handle()
        for k, w in self.params.items():
            m, v = self.adam[k]
            g = grads[k].contiguous()
            _native.check(lib.tsg_cm_adam(w.data_ptr(), g.data_ptr(), m.data_ptr(), v.data_ptr(),
                                          w.numel(), lr, 0.9, 0.999, 1e-8, self.step, stream))
        return loss

    def predict(self, batch: Batch) -> np.ndarray:
        """Predicted log device milliseconds per slice of every tree of the batch."""
        with torch.no_grad():
            pred = self.forward(batch)
        _native.check(_native.lib().tsg_cm_take_error(_device.stream_handle()))
        return pred.cpu().numpy() * self.y_std + self.y_mean

    def fit(self, graphs: Sequence[dict], log_ms: Sequence[float], epochs: int = 200,
            batch_trees: int = 64, lr: float = 2e-3, seed: int = 0) -> list[float]:
        """Trains on trees with measured log milliseconds per slice; returns the mean loss
        per epoch."""
        y_all = np.asarray(log_ms, dtype=np.float32)
        self.y_mean = float(y_all.mean())
        self.y_std = float(y_all.std() or 1.0)
        rng = np.random.default_rng(seed)
        idx = np.arange(len(graphs))
        history = []
        for ep in range(epochs):
            rng.shuffle(idx)
            losses = []
            for i in range(0, len(idx), batch_trees):
                sel = idx[i: i + batch_trees]
                b = make_batch([graphs[j] for j in sel], self.device)
                y = torch.from_numpy(y_all[sel]).to(self.device)
                losses.append(self.train_step(b, y, lr * (0.5 ** (ep // max(1, epochs // 3)))))
            history.append(float(np.mean(losses)))
        _native.check(_native.lib().tsg_cm_take_error(_device.stream_handle()))
        return history

    def state(self) -> dict[str, np.ndarray]:
        out = {k: v.cpu().numpy() for k, v in self.params.items()}
        out["y_norm"] = np.asarray([self.y_mean, self.y_std], dtype=np.float64)
        return out

    def load_state(self, state: dict) -> None:
        for k in self.params:
            self.params[k] = torch.from_numpy(np.asarray(state[k], dtype=np.float32)).to(self.device)
        self.y_mean, self.y_std = (float(x) for x in state["y_norm"])


# -- candidates, measurements, ranking ----------------------------------------------------


CANDIDATE_SETTINGS = [
    # (target_bits, trials, reconf, seed): the planner's usual setting first
    (26, 8, 10, 0), (26, 1, 10, 1), (26, 1, 0, 2), (24, 2, 10, 3), (26, 2, 6, 4),
    (26, 1, 10, 5), (22, 2, 10, 6), (26, 1, 0, 7),
]


def candidate_settings(count: int) -> list[tuple[int, int, int, int]]:
    """``count`` planner settings: the fixed list above, then single randomised orders with
    seeds 8, 9, ... cycling through slicing caps 26/25/24 and reconfiguration sizes 10/6/0."""
    out = list(CANDIDATE_SETTINGS[:count])
    seed = len(CANDIDATE_SETTINGS)
    while len(out) < count:
        out.append(((26, 25, 24)[seed % 3], 1, (10, 6, 0)[(seed // 3) % 3], seed))
        seed += 1
    return out


def candidate_trees(wiring: Any, count: int, target_bits: int = 26,
                    settings: Sequence[tuple[int, int, int, int]] | None = None
                    ) -> list[tuple[Any, tuple]]:
    """Up to ``count`` distinct (tree, sliced wires) of the planner for ``wiring``, from
    varied settings (randomised elimination orders, with and without subtree
    reconfiguration, tighter slicing caps); the first is the planner's usual choice.
    ``settings`` replaces :func:`candidate_settings` (a share of them, for parallel
    workers whose lists are merged with :func:`distinct`)."""
    from .contractions.gpu import _network, _prepare

    net = _network(_prepare(wiring))
    out, seen = [], set()
    for tb, trials, reconf, seed in (candidate_settings(count) if settings is None else settings):
        if len(out) >= count:
            break
        tree, sl = planner.optimize(net, target_bits=min(tb, target_bits), trials=trials,
                                    seed=seed, reconf=reconf)
        key = (tuple(tree.steps), tuple(sorted(sl)))
        if key in seen:
            continue
        seen.add(key)
        out.append((tree, tuple(sorted(sl))))
    return out


def _cnf_candidates(args: tuple) -> list[tuple[Any, tuple]]:
    """Worker: candidate trees of one CNF instance's clause network for some settings."""
    from .lib.sat import CNFInstance

    num_vars, clauses, count, settings = args
    return candidate_trees(CNFInstance(num_vars, clauses).clause_diagram().wiring, count,
                           settings=settings)


def cnf_candidates(pool: Any, instances: Sequence[Any], count: int,
                   parts: int = 8) -> list[list[tuple[Any, tuple]]]:
    """The planner candidates (:func:`candidate_trees`) of the clause network of every
    CNF instance, each instance's settings split over ``parts`` tasks of ``pool`` (a
    process pool; start it with ``spawn``, or before the first CUDA call). The planner's
    usual choice stays first."""
    settings = candidate_settings(count)
    jobs = [(c.num_vars, [tuple(cl) for cl in c.clauses], count, settings[p::parts])
            for c in instances for p in range(parts)]
    res = pool.map(_cnf_candidates, jobs, chunksize=1)
    out = []
    for i in range(len(instances)):
        share = res[i * parts:(i + 1) * parts]
        merged = [x[k] for k in range(max(len(x) for x in share)) for x in share if k < len(x)]
        out.append(distinct(merged))
    return out


def distinct(trees: Sequence[tuple[Any, tuple]]) -> list[tuple[Any, tuple]]:
    """The (tree, sliced wires) pairs without repeats, in their first order."""
    out, seen = [], set()
    for tree, sl in trees:
        key = (tuple(tree.steps), tuple(sorted(sl)))
        if key not in seen:
            seen.add(key)
            out.append((tree, sl))
    return out


def measure(contraction: Any, diagram: Any, primes: Sequence[int], group: int,
            passes: int = 2) -> float:
    """Device milliseconds per slice of one slice group (count ring with ``primes`` plus the
    OR-AND ring), mean over ``passes`` after a warm-up pass (``tsg_plan_run_timed``)."""
    npl = contraction.native_plan()
    dev = _device.require_cuda()
    pool = contraction.leaf_pool(diagram)
    stream = _device.stream_handle()
    g = min(group, contraction.num_slices)
    total = 0.0
    for ring, pr, planes in ((_native.TSG_RING_MODP, primes, len(primes)),
                             (_native.TSG_RING_OR_AND, (), 1)):
        ws = torch.empty(npl.workspace_bytes(ring, planes, g), dtype=torch.uint8, device=dev)
        res = torch.zeros(64, dtype=torch.uint8, device=dev)
        for k in range(passes + 1):
            ms = npl.run_timed(ring, pr, pool, 0, g, g, ws, res, False, stream)
            if k > 0:
                total += sum(ms) / passes
        del ws
    contraction.check_device()
    return total / g


def rank(model: CostModel, contractions: Sequence[Any], group: int,
         primes: Sequence[int]) -> list[float]:
    """Predicted device milliseconds per instance (per slice x slices) of each candidate."""
    graphs = [tree_graph(c, min(group, c.num_slices), primes) for c in contractions]
    pred = model.predict(make_batch(graphs, model.device))
    return [float(math.exp(p) * g["slices"]) for p, g in zip(pred, graphs)]
