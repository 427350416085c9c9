"""Device plumbing: CUDA availability, streams and raw pointers of torch tensors.

PyTorch provides device memory and streams only; every contraction runs in the native
library. Nothing here computes on the host.
"""

from __future__ import annotations

import torch


class CudaUnavailableError(RuntimeError):
    """Raised when a contraction is requested without a CUDA device."""


def require_cuda() -> torch.device:
    """The current CUDA device; raises when CUDA is unavailable (there is no CPU path)."""
    if not torch.cuda.is_available():
        raise CudaUnavailableError(
            "tensorsat_gb300 contracts on a CUDA device (sm_103a); none is available"
        )
    return torch.device("cuda", torch.cuda.current_device())


def stream_handle(stream: torch.cuda.Stream | None = None) -> int:
    """cudaStream_t of the given (default: current) torch stream, as an int."""
    s = stream if stream is not None else torch.cuda.current_stream()
    return int(s.cuda_stream)


def to_device_u8(t: torch.Tensor) -> torch.Tensor:
    """A contiguous uint8 CUDA copy (or the tensor itself when already one)."""
    dev = require_cuda()
    if t.device.type == "cuda" and t.dtype == torch.uint8 and t.is_contiguous():
        return t
    return t.to(device=dev, dtype=torch.uint8).contiguous()
