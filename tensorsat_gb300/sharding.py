"""Sharding slices across ranks (one process per GPU).

Slices of a sliced contraction are independent sub-contractions, so ranks own disjoint,
contiguous slice ranges and need no data exchange while contracting. The only exchange
is the final combination of the per-rank results: a sum (counts: mod 2^64 or mod each
prime) or an OR (SAT bits) of a few words, done with one ``torch.distributed`` all-reduce
(NCCL between GPUs, Gloo on CPU). This mirrors how the reference combines slices with
``+`` (``Box.__add__`` -> ``FinRel._union``, ``tensorsat/diagrams.py:965-970``).
"""

from __future__ import annotations

from typing import Any, Sequence

import numpy as np
import torch


def slice_ranges(num_slices: int, world_size: int, group: int = 1) -> list[tuple[int, int]]:
    """Contiguous per-rank slice ranges; every range start is a multiple of ``group``
    (a power of two) so ranks can launch whole groups. Ranges may be empty."""
    if world_size < 1:
        raise ValueError("world_size must be positive")
    if group < 1 or group & (group - 1):
        raise ValueError("group must be a power of two")
    blocks = (num_slices + group - 1) // group
    out = []
    for r in range(world_size):
        b0 = blocks * r // world_size
        b1 = blocks * (r + 1) // world_size
        out.append((min(b0 * group, num_slices), min(b1 * group, num_slices)))
    return out


def combine_counts(partials: Sequence[int], moduli: Sequence[int] | None = None) -> int:
    """Sum of per-rank counts (optionally reduced mod the product of ``moduli``)."""
    total = sum(int(p) for p in partials)
    if moduli:
        M = 1
        for p in moduli:
            M *= p
        total %= M
    return total


def allreduce_residues(residues: torch.Tensor, moduli: Sequence[int], group=None) -> torch.Tensor:
    """All-reduces per-prime residues (int64 tensor [planes, entries]) and reduces each
    plane mod its prime. Residues < 2^31 summed over < 2^32 ranks cannot overflow int64."""
    import torch.distributed as dist

    out = residues.to(torch.int64).clone()
    dist.all_reduce(out, op=dist.ReduceOp.SUM, group=group)
    mods = torch.tensor(list(moduli), dtype=torch.int64, device=out.device).reshape(-1, 1)
    return out % mods


def allreduce_or(bits: torch.Tensor, group=None) -> torch.Tensor:
    """All-reduces SAT bits by OR (as MAX over {0,1})."""
    import torch.distributed as dist

    out = bits.to(torch.int32).clone()
    dist.all_reduce(out, op=dist.ReduceOp.MAX, group=group)
    return out


def collective_device(group: Any = None) -> torch.device:
    """Where a collective's tensors live: the current GPU for NCCL groups, the host for
    Gloo."""
    import torch.distributed as dist

    if dist.get_backend(group) == "nccl":
        return torch.device("cuda", torch.cuda.current_device())
    return torch.device("cpu")


def allreduce_u64(values: np.ndarray, group: Any = None) -> np.ndarray:
    """All-reduces uint64 counts by their sum mod 2^64. Each value travels as two 32-bit
    halves in int64 lanes (sums of halves over < 2^31 ranks cannot overflow), and the
    halves are recombined on the host."""
    import torch.distributed as dist

    v = np.ascontiguousarray(values, dtype=np.uint64).reshape(-1)
    halves = np.stack([(v & np.uint64(0xFFFFFFFF)).astype(np.int64),
                       (v >> np.uint64(32)).astype(np.int64)])
    t = torch.from_numpy(halves).to(collective_device(group))
    dist.all_reduce(t, op=dist.ReduceOp.SUM, group=group)
    lo, hi = t.cpu().numpy()
    return np.array([(int(a) + (int(b) << 32)) & 0xFFFFFFFFFFFFFFFF for a, b in zip(lo, hi)],
                    dtype=np.uint64)


def allreduce_min_int(value: int, group: Any = None) -> int:
    """The smallest of one integer per rank (every rank gets it)."""
    import torch.distributed as dist

    t = torch.tensor([int(value)], dtype=torch.int64, device=collective_device(group))
    dist.all_reduce(t, op=dist.ReduceOp.MIN, group=group)
    return int(t.item())
