// Shared host/device helpers of the tensorsat_gb300 library: status handling and the
// device-side arithmetic of the three rings (OR-AND bits, residues mod p, uint64).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <cstdio>
#include <string>

#include "tensorsat_gb300.h"

namespace tsg {

// Records `msg` as the calling thread's last error and returns `code`.
tsg_status fail(tsg_status code, const std::string& msg);

// Maps a CUDA error (if any) to TSG_ERR_CUDA with the CUDA message appended.
tsg_status cuda_status(cudaError_t err, const char* what);

#define TSG_CUDA_TRY(expr)                                   \
  do {                                                      \
    cudaError_t tsg_err_ = (expr);                          \
    if (tsg_err_ != cudaSuccess) return ::tsg::cuda_status(tsg_err_, #expr); \
  } while (0)

#define TSG_TRY(expr)                   \
  do {                                 \
    tsg_status tsg_st_ = (expr);       \
    if (tsg_st_ != TSG_OK) return tsg_st_; \
  } while (0)

// Number of SMs of the current device (cached per device ordinal).
int device_sm_count();

// Grid size for a grid-stride loop over `work` items with `threads` per block:
// enough blocks to cover the work, capped at `per_sm` resident blocks on every SM.
inline unsigned grid_for(uint64_t work, unsigned threads, int per_sm = 16) {
  uint64_t blocks = (work + threads - 1) / threads;
  uint64_t cap = (uint64_t)device_sm_count() * (uint64_t)per_sm;
  if (blocks > cap) blocks = cap;
  if (blocks == 0) blocks = 1;
  return (unsigned)blocks;
}

// Barrett reduction (P. Barrett, CRYPTO '86) of x < 2^63 modulo an odd p < 2^31, with
// m = floor((2^64 - 1) / p) precomputed on the host. The quotient estimate
// q = floor(x * m / 2^64) is q_true or q_true - 1, so one conditional subtraction
// finishes the reduction.
__device__ __forceinline__ uint32_t barrett_reduce(uint64_t x, uint32_t p, uint64_t m) {
  uint64_t q = __umul64hi(x, m);
  uint64_t r = x - q * (uint64_t)p;
  return (uint32_t)(r >= p ? r - p : r);
}

// Montgomery reduction (P. L. Montgomery, Math. Comp. 44, 1985) with R = 2^32 for an odd
// p < 2^31: returns T * R^-1 mod p for T < p * 2^32, given pinv = -p^-1 mod 2^32.
// m = T * pinv (mod 2^32) makes T + m * p divisible by 2^32; the quotient is < 2p.
__device__ __forceinline__ uint32_t mont_redc(uint64_t T, uint32_t p, uint32_t pinv) {
  const uint32_t m = (uint32_t)T * pinv;
  const uint32_t t = (uint32_t)((T + (uint64_t)m * p) >> 32);
  return t >= p ? t - p : t;
}

// x mod p for x < 32 * 2^31 and p = 2^31 - d with d < 2^10: x = q * 2^31 + s gives
// x - q * p = q * d + s < 2p, so one conditional subtraction finishes.
__device__ __forceinline__ uint32_t small_mod(uint64_t x, uint32_t p) {
  const uint64_t q = x >> 31;
  const uint64_t r = x - q * (uint64_t)p;
  return (uint32_t)(r >= p ? r - p : r);
}

__device__ __forceinline__ uint32_t add_mod(uint32_t a, uint32_t b, uint32_t p) {
  const uint32_t s = a + b;  // a, b < p < 2^31: no wrap
  return s >= p ? s - p : s;
}

}  // namespace tsg
