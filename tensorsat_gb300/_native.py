"""ctypes binding of ``libtensorsat_gb300.so`` (the C ABI declared in
``include/tensorsat_gb300.h``).

The library is the only compute path of this package: there is no CPU fallback. Loading
fails loudly (``NativeLibraryError``) when the library is missing and cannot be built.
"""

from __future__ import annotations

import ctypes
import os
import threading
from ctypes import POINTER, c_char_p, c_int32, c_int64, c_uint32, c_void_p

from . import _build

TSG_OK = 0
TSG_ERR_INVALID_ARGUMENT = 1
TSG_ERR_UNSUPPORTED = 2
TSG_ERR_TOO_LARGE = 3
TSG_ERR_WORKSPACE = 4
TSG_ERR_CUDA = 5
TSG_ERR_TIMEOUT = 6

TSG_RING_OR_AND = 0
TSG_RING_MODP = 1
TSG_RING_U64 = 2

TSG_MAX_BITS = 62
TSG_MAX_PRIMES = 4

TSG_KERNEL_GENERAL = 0
TSG_KERNEL_TILE = 1
TSG_KERNEL_STREAM = 2
TSG_KERNEL_FUSED = 3
TSG_KERNEL_NONE = 4
TSG_KERNEL_SUM = 5
TSG_STEP_NO_STREAM = 1
TSG_STEP_NO_FUSE = 2
TSG_STEP_FUSE = 4
TSG_STEP_PLANE_SPLIT = 8

EXPORTED_SYMBOLS = (
    "tsg_last_error",
    "tsg_abi_version",
    "tsg_contract2_or_and",
    "tsg_contract2_count_u64",
    "tsg_contract2_modp",
    "tsg_rewire_or_and",
    "tsg_union_or",
    "tsg_spider_fill",
    "tsg_plan_create",
    "tsg_plan_destroy",
    "tsg_plan_workspace_bytes",
    "tsg_plan_root_bits",
    "tsg_plan_launch_count",
    "tsg_plan_run",
    "tsg_plan_run_timed",
    "tsg_batch_workspace_bytes",
    "tsg_batch_run",
    "tsg_plan_validate",
    "tsg_take_device_error",
    "tsg_static_scratch_bytes",
    "tsg_plan_run_static",
    "tsg_plan_subset_dp",
    "tsg_plan_describe",
    "tsg_set_wait_limit_ns",
    "tsg_wait_limit_ns",
    "tsg_debug_stall_producer",
    "tsg_plan_launches",
    "tsg_set_fusion",
    "tsg_fusion_enabled",
    "tsg_batch_lanes_workspace_bytes",
    "tsg_batch_run_lanes",
    "tsg_batch_packed_workspace_bytes",
    "tsg_peek_device_error_async",
    "tsg_batch_run_packed",
    "tsg_plan_set_step_options",
    "tsg_plan_variants_workspace_bytes",
    "tsg_plan_run_variants",
    "tsg_cm_gemm_bf16",
    "tsg_cm_take_error",
    "tsg_cm_set_gemm_mode",
    "tsg_cm_child_sum",
    "tsg_cm_parent_add",
    "tsg_cm_gemm_at_b",
    "tsg_cm_adam",
)


class NativeLibraryError(RuntimeError):
    """The native CUDA library is unavailable."""


class TsgError(RuntimeError):
    """A C ABI call returned a non-OK status."""

    def __init__(self, status: int, message: str) -> None:
        super().__init__(f"[tsg status {status}] {message}")
        self.status = status


class TsgValueError(TsgError, ValueError):
    """Invalid argument reported by the native library (ValueError upstream)."""


_lock = threading.Lock()
_lib: ctypes.CDLL | None = None

_i32p = POINTER(c_int32)
_i64p = POINTER(c_int64)


def _declare(lib: ctypes.CDLL) -> None:
    lib.tsg_last_error.restype = c_char_p
    lib.tsg_last_error.argtypes = []
    lib.tsg_abi_version.restype = c_int32
    lib.tsg_abi_version.argtypes = []
    c2 = [c_void_p, c_int32, _i64p, _i64p, c_void_p, c_int32, _i64p, _i64p, c_int32, _i64p,
          c_void_p, c_void_p]
    lib.tsg_contract2_or_and.restype = c_int32
    lib.tsg_contract2_or_and.argtypes = c2
    lib.tsg_contract2_count_u64.restype = c_int32
    lib.tsg_contract2_count_u64.argtypes = c2
    lib.tsg_contract2_modp.restype = c_int32
    lib.tsg_contract2_modp.argtypes = [c_void_p, c_int32, _i64p, _i64p, c_void_p, c_int32, _i64p,
                                       _i64p, c_int32, _i64p, c_int32, POINTER(c_uint32),
                                       c_void_p, c_void_p]
    lib.tsg_rewire_or_and.restype = c_int32
    lib.tsg_rewire_or_and.argtypes = [c_void_p, c_int32, _i64p, c_int32, _i32p, c_void_p,
                                      c_void_p]
    lib.tsg_union_or.restype = c_int32
    lib.tsg_union_or.argtypes = [c_void_p, c_void_p, c_void_p, c_int64, c_void_p]
    lib.tsg_spider_fill.restype = c_int32
    lib.tsg_spider_fill.argtypes = [c_void_p, c_int64, c_int32, c_void_p]
    lib.tsg_plan_create.restype = c_int32
    lib.tsg_plan_create.argtypes = [c_int32, _i32p, _i64p, c_int32, _i32p, c_int32, _i32p,
                                    _i32p, _i32p, _i32p, _i32p, POINTER(c_void_p)]
    lib.tsg_plan_destroy.restype = None
    lib.tsg_plan_destroy.argtypes = [c_void_p]
    lib.tsg_plan_workspace_bytes.restype = c_int32
    lib.tsg_plan_workspace_bytes.argtypes = [c_void_p, c_int32, c_int32, c_int64, _i64p]
    lib.tsg_plan_root_bits.restype = c_int32
    lib.tsg_plan_root_bits.argtypes = [c_void_p, _i32p]
    lib.tsg_plan_launch_count.restype = c_int32
    lib.tsg_plan_launch_count.argtypes = [c_void_p, c_int64, c_int64, c_int64, _i64p]
    lib.tsg_plan_run.restype = c_int32
    lib.tsg_plan_run.argtypes = [c_void_p, c_int32, c_int32, POINTER(c_uint32), c_void_p,
                                 c_int64, c_int64, c_int64, c_void_p, c_int64, c_void_p,
                                 c_int32, c_void_p]
    lib.tsg_plan_run_timed.restype = c_int32
    lib.tsg_plan_run_timed.argtypes = [c_void_p, c_int32, c_int32, POINTER(c_uint32), c_void_p,
                                       c_int64, c_int64, c_int64, c_void_p, c_int64, c_void_p,
                                       c_int32, c_void_p, POINTER(ctypes.c_float)]
    lib.tsg_batch_workspace_bytes.restype = c_int32
    lib.tsg_batch_workspace_bytes.argtypes = [c_int32, POINTER(c_void_p), c_int32, c_int32, _i64p,
                                              _i64p]
    lib.tsg_batch_run.restype = c_int32
    lib.tsg_batch_run.argtypes = [c_int32, POINTER(c_void_p), c_int32, c_int32, POINTER(c_uint32),
                                  POINTER(c_void_p), _i64p, c_void_p, c_int64, POINTER(c_void_p),
                                  c_void_p]
    lib.tsg_take_device_error.restype = c_int32
    lib.tsg_take_device_error.argtypes = [c_void_p]
    lib.tsg_static_scratch_bytes.restype = c_int64
    lib.tsg_static_scratch_bytes.argtypes = []
    lib.tsg_plan_run_static.restype = c_int32
    lib.tsg_plan_run_static.argtypes = [c_void_p, c_int32, c_int32, POINTER(c_uint32), c_void_p,
                                        c_int64, c_int64, c_int64, c_void_p, c_int32, c_void_p]
    lib.tsg_plan_validate.restype = c_int32
    lib.tsg_plan_validate.argtypes = [c_void_p, c_int32, c_int32, POINTER(c_uint32), c_int64,
                                      c_int64, c_int64]
    lib.tsg_plan_describe.restype = c_int32
    lib.tsg_plan_describe.argtypes = [c_void_p, c_int32, c_int32, POINTER(c_uint32), c_int64,
                                      _i32p]
    lib.tsg_batch_lanes_workspace_bytes.restype = c_int32
    lib.tsg_batch_lanes_workspace_bytes.argtypes = [c_int32, POINTER(c_void_p), c_int32, c_int32,
                                                    _i64p, c_int32, _i64p]
    lib.tsg_batch_run_lanes.restype = c_int32
    lib.tsg_batch_run_lanes.argtypes = [c_int32, POINTER(c_void_p), c_int32, c_int32,
                                        POINTER(c_uint32), POINTER(c_void_p), _i64p, c_int32,
                                        c_void_p, c_int64, POINTER(c_void_p), c_void_p]
    lib.tsg_peek_device_error_async.restype = c_int32
    lib.tsg_peek_device_error_async.argtypes = [c_void_p, c_void_p]
    lib.tsg_batch_packed_workspace_bytes.restype = c_int32
    lib.tsg_batch_packed_workspace_bytes.argtypes = [c_int32, POINTER(c_void_p), c_int32, c_int32,
                                                     _i64p, c_int32, _i64p]
    lib.tsg_batch_run_packed.restype = c_int32
    lib.tsg_batch_run_packed.argtypes = [c_int32, POINTER(c_void_p), c_int32, c_int32,
                                         POINTER(c_uint32), POINTER(c_void_p), _i64p, c_int32,
                                         c_void_p, c_int64, POINTER(c_void_p), c_void_p, _i64p]
    lib.tsg_cm_set_gemm_mode.restype = c_int32
    lib.tsg_cm_set_gemm_mode.argtypes = [c_int32]
    lib.tsg_plan_variants_workspace_bytes.restype = c_int32
    lib.tsg_plan_variants_workspace_bytes.argtypes = [c_void_p, c_int32, c_int32, c_int64,
                                                      c_int64, _i64p]
    lib.tsg_plan_run_variants.restype = c_int32
    lib.tsg_plan_run_variants.argtypes = [c_void_p, c_int32, c_int32, POINTER(c_uint32),
                                          c_void_p, c_int64, c_int64, c_int64, c_void_p,
                                          c_int64, c_void_p, c_int32, c_void_p]
    lib.tsg_cm_gemm_bf16.restype = c_int32
    lib.tsg_cm_gemm_bf16.argtypes = [c_int64, c_int64, c_int64, c_void_p, c_void_p, c_void_p,
                                     c_int32, c_void_p, c_int64, c_int32, c_void_p]
    lib.tsg_cm_child_sum.restype = c_int32
    lib.tsg_cm_child_sum.argtypes = [c_void_p, c_void_p, c_void_p, c_void_p, c_int64, c_int32,
                                     c_int32, c_void_p]
    lib.tsg_cm_parent_add.restype = c_int32
    lib.tsg_cm_parent_add.argtypes = [c_void_p, c_int32, c_void_p, c_void_p, c_int64, c_int32,
                                      c_void_p]
    lib.tsg_cm_gemm_at_b.restype = c_int32
    lib.tsg_cm_gemm_at_b.argtypes = [c_void_p, c_int32, c_void_p, c_int32, c_int64, c_void_p,
                                     c_void_p]
    lib.tsg_cm_adam.restype = c_int32
    lib.tsg_cm_adam.argtypes = [c_void_p, c_void_p, c_void_p, c_void_p, c_int64, ctypes.c_float,
                                ctypes.c_float, ctypes.c_float, ctypes.c_float, c_int32, c_void_p]
    lib.tsg_cm_take_error.restype = c_int32
    lib.tsg_cm_take_error.argtypes = [c_void_p]
    lib.tsg_plan_set_step_options.restype = c_int32
    lib.tsg_plan_set_step_options.argtypes = [c_void_p, c_int32, _i32p]
    lib.tsg_plan_launches.restype = c_int32
    lib.tsg_plan_launches.argtypes = [c_void_p, c_int32, c_int32, c_int64, c_int64, c_int64,
                                      _i64p]
    lib.tsg_set_fusion.restype = c_int32
    lib.tsg_set_fusion.argtypes = [c_int32]
    lib.tsg_fusion_enabled.restype = c_int32
    lib.tsg_fusion_enabled.argtypes = []
    lib.tsg_set_wait_limit_ns.restype = c_int32
    lib.tsg_set_wait_limit_ns.argtypes = [ctypes.c_uint64]
    lib.tsg_wait_limit_ns.restype = ctypes.c_uint64
    lib.tsg_wait_limit_ns.argtypes = []
    lib.tsg_debug_stall_producer.restype = c_int32
    lib.tsg_debug_stall_producer.argtypes = [c_int64]
    u64p = POINTER(ctypes.c_uint64)
    lib.tsg_plan_subset_dp.restype = c_int32
    lib.tsg_plan_subset_dp.argtypes = [c_int32, c_int32, u64p, u64p, u64p, c_int32,
                                       POINTER(ctypes.c_double), POINTER(c_uint32), u64p]


def library_path() -> str:
    return str(_build.LIB_PATH)


def lib(build_if_missing: bool = True) -> ctypes.CDLL:
    """Loads (building first if needed) and returns the native library."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        path = _build.LIB_PATH
        if build_if_missing and (not path.exists() or _build.needs_build()):
            try:
                _build.build_library()
            except Exception as exc:  # pragma: no cover - exercised only without nvcc
                if not path.exists():
                    raise NativeLibraryError(
                        f"libtensorsat_gb300.so is missing and could not be built: {exc}"
                    ) from exc
        if not path.exists():
            raise NativeLibraryError(f"native library not found at {path}")
        try:
            handle = ctypes.CDLL(os.fspath(path))
        except OSError as exc:
            raise NativeLibraryError(f"cannot load {path}: {exc}") from exc
        _declare(handle)
        _lib = handle
        return handle


def check(status: int) -> None:
    """Raises the exception matching a non-OK status."""
    if status == TSG_OK:
        return
    msg = lib().tsg_last_error().decode(errors="replace")
    if status in (TSG_ERR_INVALID_ARGUMENT, TSG_ERR_TOO_LARGE):
        raise TsgValueError(status, msg)
    raise TsgError(status, msg)


def i64_array(values) -> ctypes.Array:
    vals = list(values)
    return (c_int64 * max(1, len(vals)))(*vals)


def i32_array(values) -> ctypes.Array:
    vals = list(values)
    return (c_int32 * max(1, len(vals)))(*vals)


def ptr_i32(a) -> ctypes._Pointer:
    """Pointer to a contiguous numpy int32 array."""
    return a.ctypes.data_as(_i32p)


def ptr_i64(a) -> ctypes._Pointer:
    return a.ctypes.data_as(_i64p)


__all__ = [name for name in dir() if name.startswith("TSG_")] + [
    "NativeLibraryError",
    "TsgError",
    "TsgValueError",
    "lib",
    "check",
    "library_path",
    "EXPORTED_SYMBOLS",
]
