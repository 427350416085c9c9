"""The project's autotuner: per-step kernel choices and the slice group of a plan, timed
on the GPU and cached as JSON beside the plan files.

The reference leaves its knobs to cotengra (``optimize`` and ``order`` keyword arguments,
``tensorsat/contractions/cotengra.py:62-64,104-106``), which choose the path only. Here
the path is fixed by the planner and the answers do not depend on any kernel choice, so
the tuner only looks for speed:

1. For each candidate slice group (the largest that fits the memory budget and up to two
   halvings of it), it times one slice group of the plan with ``tsg_plan_run_timed`` (a
   CUDA event after every launch) in four configurations: the executor's own choices; no
   fused step; tile kernels only; every possible fusion (and, for residue counts, every
   tile step with one residue plane per block instead of all planes in one thread).
2. Per decision it keeps the faster alternative: a fusion when the fused consumer took
   less than the producer plus its consumer unfused; a streamed step when it beat the
   tile kernel; a tile step's plane split when it beat the in-thread plane loop.
3. It times that mixed configuration too and keeps the fastest, per slice.

The choice is a list of per-step options (``TSG_STEP_NO_STREAM``, ``TSG_STEP_NO_FUSE``,
``TSG_STEP_FUSE``, applied with ``tsg_plan_set_step_options``) and a group, stored with
the timings under a key of the plan, the ring, the moduli and the GPU's name.
"""

from __future__ import annotations

import hashlib
import json
import os
from pathlib import Path
from typing import Any, Sequence

import numpy as np

from . import _native

TUNE_FORMAT = "tensorsat_gb300.tune/1"


def plan_key(contraction: Any) -> str:
    """SHA-256 of the contraction's plan (tree, sliced wires, leaf wires)."""
    data = json.dumps(contraction.plan_dict(), sort_keys=True, separators=(",", ":"))
    return hashlib.sha256(data.encode()).hexdigest()


def entry_key(contraction: Any, ring: int, primes: Sequence[int], gpu: str) -> str:
    return f"{plan_key(contraction)}|ring={ring}|primes={','.join(map(str, primes))}|{gpu}"


def set_options(contraction: Any, ring: int, options: Sequence[int] | None) -> None:
    """Applies per-step options (None clears them) to the contraction's native plan."""
    npl = contraction.native_plan()
    arr = None if options is None else np.ascontiguousarray(options, dtype=np.int32)
    if arr is not None and arr.shape != (npl.num_steps,):
        raise ValueError(f"expected {npl.num_steps} step options")
    _native.check(_native.lib().tsg_plan_set_step_options(
        npl.handle, ring, None if arr is None else _native.ptr_i32(arr)))


def fuse_all(contraction: Any, ring: int) -> None:
    """Asks for every fusion the plan's structure allows in ``ring`` (TSG_STEP_FUSE on
    every step)."""
    set_options(contraction, ring, [_native.TSG_STEP_FUSE] * contraction.native_plan().num_steps)


def _timed(contraction: Any, ring: int, primes: Sequence[int], pool: Any, begin: int,
           group: int, options: Sequence[int] | None, passes: int) -> tuple[list[float], list]:
    """Per-step device milliseconds (mean over ``passes`` after one warm-up pass) of one
    slice group under ``options``, and the kinds each step launched with."""
    import torch

    from . import _device

    set_options(contraction, ring, options)
    npl = contraction.native_plan()
    planes = len(primes) if ring == _native.TSG_RING_MODP else 1
    dev = _device.require_cuda()
    ws = torch.empty(npl.workspace_bytes(ring, planes, group), dtype=torch.uint8, device=dev)
    entries = 1 << len(contraction._leaves.out_unique)
    res = torch.zeros(planes * entries * 8, dtype=torch.uint8, device=dev)
    stream = _device.stream_handle()
    end = min(contraction.num_slices, begin + group)
    acc = None
    for k in range(passes + 1):
        ms = npl.run_timed(ring, primes, pool, begin, end, group, ws, res, False, stream)
        if k > 0:
            acc = ms if acc is None else [a + b for a, b in zip(acc, ms)]
    contraction.check_device()
    kinds = npl.describe(ring, primes, group).tolist()
    del ws
    return [a / passes for a in acc], kinds


def tune(contraction: Any, diagram: Any, ring: int, primes: Sequence[int] = (),
         budget_bytes: int | None = None, passes: int = 2, max_halvings: int = 2) -> dict:
    """Times the candidate configurations of ``contraction`` in ``ring`` on the current
    GPU and returns the chosen entry (options, group, timings); the options stay applied.

    Configurations per candidate group: the executor's own choices; no fused step; no
    fused and no streamed step (tile kernels only); every possible fusion (streamed fused
    consumers included). Per decision the faster measured alternative is kept: a fusion
    when its consumer took less time than producer plus consumer unfused, a streamed step
    when it beat the tile kernel. The mixed configuration is timed too; the fastest
    configuration per slice wins."""
    import torch

    npl = contraction.native_plan()
    planes = len(primes) if ring == _native.TSG_RING_MODP else 1
    pool = contraction.leaf_pool(diagram)
    ns = contraction.num_slices
    top = contraction.choose_group(ring, planes, budget_bytes)
    groups = []
    g = top
    for _ in range(max_halvings + 1):
        if g < 1 or g in groups:
            break
        groups.append(g)
        g //= 2
    n = npl.num_steps
    L = contraction.tree.num_leaves
    NS, NF, FU = _native.TSG_STEP_NO_STREAM, _native.TSG_STEP_NO_FUSE, _native.TSG_STEP_FUSE
    PS = _native.TSG_STEP_PLANE_SPLIT
    configs = {"executor": [0] * n, "no_fuse": [NF] * n, "tile": [NS | NF] * n,
               "fuse": [FU] * n}
    if ring == _native.TSG_RING_MODP and len(primes) > 1:
        configs["plane_split"] = [NF | PS] * n
    trials = []
    for g in groups:
        ms, kinds = {}, {}
        for name, opts in configs.items():
            ms[name], kinds[name] = _timed(contraction, ring, primes, pool, 0, g, opts, passes)
        mixed = [0] * n
        # fusions: every pair the "fuse" configuration formed, kept when faster
        for s in range(n):
            if kinds["fuse"][s][0] != _native.TSG_KERNEL_FUSED:
                continue
            prod = [x - L for x in contraction.tree.steps[s]
                    if x >= L and kinds["fuse"][x - L][0] == _native.TSG_KERNEL_NONE]
            if not prod:
                continue
            p = prod[0]
            if ms["fuse"][s] < ms["no_fuse"][s] + ms["no_fuse"][p]:
                mixed[p] |= FU
            else:
                mixed[p] |= NF
        # streaming: kept where it beat the tile kernel (unfused steps)
        for s in range(n):
            if kinds["no_fuse"][s][0] == _native.TSG_KERNEL_STREAM and \
                    ms["tile"][s] < ms["no_fuse"][s]:
                mixed[s] |= NS
        # MODP tile steps: all residue planes in one thread, or one plane per block
        if "plane_split" in configs:
            for s in range(n):
                if kinds["no_fuse"][s][0] == _native.TSG_KERNEL_TILE and \
                        ms["plane_split"][s] < ms["no_fuse"][s] and not mixed[s] & NS:
                    mixed[s] |= PS
        ms["mixed"], _ = _timed(contraction, ring, primes, pool, 0, g, mixed, passes)
        slices = min(ns, g)
        for name, opts in list(configs.items()) + [("mixed", mixed)]:
            trials.append({"group": g, "config": name, "options": list(opts),
                           "ms": sum(ms[name]), "ms_per_slice": sum(ms[name]) / slices})
    best = min(trials, key=lambda t: t["ms_per_slice"])
    base = next(t for t in trials if t["group"] == top and t["config"] == "executor")
    set_options(contraction, ring, best["options"])
    torch.cuda.synchronize()
    return {
        "ring": ring, "primes": list(primes), "group": best["group"],
        "options": best["options"], "config": best["config"],
        "ms_per_slice": best["ms_per_slice"], "default_ms_per_slice": base["ms_per_slice"],
        "gain": base["ms_per_slice"] / best["ms_per_slice"],
        "trials": [{k: v for k, v in t.items() if k != "options"} for t in trials],
    }


def gpu_name() -> str:
    import torch

    return torch.cuda.get_device_name(torch.cuda.current_device())


def load(path: str | os.PathLike, contraction: Any, ring: int, primes: Sequence[int],
         gpu: str | None = None) -> dict | None:
    """The cached entry for this plan, ring, moduli and GPU in ``path`` (None if absent)."""
    path = Path(path)
    if not path.exists():
        return None
    data = json.loads(path.read_text())
    if data.get("format") != TUNE_FORMAT:
        raise ValueError(f"{path} is not a {TUNE_FORMAT} file")
    return data["entries"].get(entry_key(contraction, ring, primes, gpu or gpu_name()))


def apply(contraction: Any, entry: dict) -> int:
    """Applies a cached entry's options; returns its slice group."""
    set_options(contraction, entry["ring"], entry["options"])
    return int(entry["group"])


def load_or_tune(path: str | os.PathLike, contraction: Any, diagram: Any, ring: int,
                 primes: Sequence[int] = (), budget_bytes: int | None = None) -> dict:
    """The cached entry (applied), or a new tuning stored in ``path`` (written atomically)."""
    gpu = gpu_name()
    entry = load(path, contraction, ring, primes, gpu)
    if entry is not None:
        apply(contraction, entry)
        return entry
    entry = tune(contraction, diagram, ring, primes, budget_bytes)
    path = Path(path)
    data = json.loads(path.read_text()) if path.exists() else {"format": TUNE_FORMAT,
                                                             "entries": {}}
    data["entries"][entry_key(contraction, ring, primes, gpu)] = entry
    tmp = path.with_name(path.name + ".tmp")
    tmp.write_text(json.dumps(data, indent=1))
    os.replace(tmp, path)
    return entry
