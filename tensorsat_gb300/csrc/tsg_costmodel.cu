// Kernels of the learned cost model (tensorsat_gb300/costmodel.py): a message-passing
// network over contraction trees that predicts a tree's device time, used to rank the
// planner's candidate trees. None of this touches the answers of a contraction.
//
// The dense layers run on the 5th-generation tensor cores: tcgen05.mma (kind::f16, BF16
// operands, FP32 accumulation in tensor memory), one elected thread issuing the MMAs of a
// 128-row tile, operands staged in shared memory in the canonical K-major layout without
// swizzling (8-row x 16-byte core matrices), the accumulator read back with tcgen05.ld
// for a fused epilogue (bias, ReLU, BF16 or FP32 store). The remaining training kernels
// (child aggregation and its transpose, weight gradients, Adam) are plain CUDA.
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_bf16.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <atomic>
#include <mutex>
#include <string>

#include "tsg_common.cuh"

namespace tsg {
namespace cm {

constexpr int kTileM = 128;  // rows of one CTA tile = TMEM lanes
constexpr int kTileK = 64;   // K staged per round (4 MMAs of K = 16)
constexpr int kThreads = 128;
constexpr unsigned long long kWaitNs = 2000000000ull;
constexpr int kStagePerWarp = 32 * (32 * 4 + 16);  // epilogue stage: 32 rows of 32 FP32 + pad

__device__ int g_cm_error = 0;  // set when a bounded wait for the MMAs gives up

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

// Shared-memory matrix descriptor (tcgen05): start address, leading-dimension byte offset
// (between core matrices adjacent in K), stride byte offset (between 8-row groups),
// descriptor version 1, no swizzling.
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
  uint64_t d = 0;
  d |= (uint64_t)((addr >> 4) & 0x3FFF);
  d |= (uint64_t)((lbo >> 4) & 0x3FFF) << 16;
  d |= (uint64_t)((sbo >> 4) & 0x3FFF) << 32;
  d |= (uint64_t)1 << 46;  // version
  return d;                // base offset 0, layout type 0 (no swizzle)
}

// Instruction descriptor of kind::f16: FP32 accumulator, BF16 A and B, both K-major,
// N columns, M = 128 rows.
__host__ __device__ constexpr uint32_t instr_desc(int n) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(n >> 3) << 17) |
         ((uint32_t)(kTileM >> 4) << 24);
}

// Byte offset of element (r, k) of a rows x kTileK tile in the canonical K-major layout:
// core matrix (r / 8, k / 8) of 8 rows x 16 bytes, K-adjacent core matrices 128 bytes
// apart (LBO), 8-row groups kTileK / 8 * 128 bytes apart (SBO).
__device__ __forceinline__ uint32_t tile_offset(int r, int k) {
  return (uint32_t)((r >> 3) * (kTileK / 8) * 128 + (k >> 3) * 128 + (r & 7) * 16 + (k & 7) * 2);
}

__device__ __forceinline__ uint32_t pack_bf16x2(float lo, float hi) {
  const __nv_bfloat162 p = __floats2bfloat162_rn(lo, hi);
  return *reinterpret_cast<const uint32_t*>(&p);
}

__device__ __forceinline__ bool wait_mbar(uint64_t* bar, uint32_t parity) {
  const uint32_t addr = smem_u32(bar);
  uint64_t t0;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t0));
  for (;;) {
    uint32_t ok;
    asm volatile(
        "{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n"
        "selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(addr), "r"(parity), "r"(20000u)
        : "memory");
    if (ok) return true;
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    if (t - t0 > kWaitNs) return false;
  }
}

// Epilogue of a 128-row tile: warp w reads TMEM lanes 32w..32w+31 (rows), 32 columns per
// load; each thread puts its row's 32 results (bias, ReLU, conversion applied) into the
// warp's stage in shared memory (`smem`, free once the MMAs are done), then the warp writes
// the 32 x 32 block out in 16-byte pieces, whole rows per group of lanes.
template <int N>
__device__ __forceinline__ void epilogue(uint32_t tmem, uint8_t* smem, void* out, int m0, int ldo,
                                         const float* __restrict__ bias, int relu, int out_f32) {
  const int tid = threadIdx.x;
  const int warp = tid >> 5;
  const int lane = tid & 31;
  const int eb = out_f32 ? 4 : 2;
  const int pitch = 32 * eb + 16;  // bytes per staged row (16-byte groups spread over banks)
  uint8_t* stage = smem + warp * kStagePerWarp;
  const int lpr = 2 * eb;          // lanes per row of 32 results
  const int rpi = 32 / lpr;        // rows per warp-wide copy
#pragma unroll 1
  for (int c0 = 0; c0 < N; c0 += 32) {
    uint32_t v[32];
    const uint32_t taddr = tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0;
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,"
        "%13,%14,%15,%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
        : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]),
          "=r"(v[6]), "=r"(v[7]), "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]),
          "=r"(v[12]), "=r"(v[13]), "=r"(v[14]), "=r"(v[15]), "=r"(v[16]), "=r"(v[17]),
          "=r"(v[18]), "=r"(v[19]), "=r"(v[20]), "=r"(v[21]), "=r"(v[22]), "=r"(v[23]),
          "=r"(v[24]), "=r"(v[25]), "=r"(v[26]), "=r"(v[27]), "=r"(v[28]), "=r"(v[29]),
          "=r"(v[30]), "=r"(v[31])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
    float x[32];
#pragma unroll
    for (int j = 0; j < 32; ++j) {
      x[j] = __uint_as_float(v[j]) + (bias ? bias[c0 + j] : 0.f);
      if (relu) x[j] = fmaxf(x[j], 0.f);
    }
    uint8_t* my = stage + lane * pitch;
    if (out_f32) {
#pragma unroll
      for (int j = 0; j < 32; j += 4)
        *reinterpret_cast<float4*>(my + j * 4) = make_float4(x[j], x[j + 1], x[j + 2], x[j + 3]);
    } else {
#pragma unroll
      for (int j = 0; j < 32; j += 8) {
        uint4 u;
        u.x = pack_bf16x2(x[j], x[j + 1]);
        u.y = pack_bf16x2(x[j + 2], x[j + 3]);
        u.z = pack_bf16x2(x[j + 4], x[j + 5]);
        u.w = pack_bf16x2(x[j + 6], x[j + 7]);
        *reinterpret_cast<uint4*>(my + j * 2) = u;
      }
    }
    __syncwarp();
    for (int r0 = 0; r0 < 32; r0 += rpi) {
      const int r = r0 + lane / lpr, part = lane % lpr;
      const uint4 u = *reinterpret_cast<const uint4*>(stage + r * pitch + part * 16);
      uint8_t* dst = reinterpret_cast<uint8_t*>(out) +
                     ((size_t)(m0 + warp * 32 + r) * ldo + c0) * eb + part * 16;
      *reinterpret_cast<uint4*>(dst) = u;
    }
    __syncwarp();
  }
}

// D[M x N] = A[M x K] * B[N x K]^T (+ bias[N], ReLU): A and B row-major BF16 (K
// contiguous), K a multiple of 64, M a multiple of 128, N in {64, 128}. One CTA per
// 128-row tile, all N columns in tensor memory.
template <int N>
__global__ void __launch_bounds__(kThreads, 1)
    gemm_bf16_tn_kernel(const __nv_bfloat16* __restrict__ A, const __nv_bfloat16* __restrict__ B,
                        const float* __restrict__ bias, void* out, int K, int ldo, int relu,
                        int out_f32) {
  // the A and B tiles; after the last MMA the same bytes stage the epilogue's rows
  __shared__ __align__(1024) uint8_t smem[(kTileM + N) * kTileK * 2];
  static_assert((kTileM + N) * kTileK * 2 >= 4 * kStagePerWarp, "epilogue stage does not fit");
  uint8_t* sa = smem;
  uint8_t* sb = smem + kTileM * kTileK * 2;
  __shared__ __align__(8) uint64_t mbar;
  __shared__ uint32_t tmem_base;
  const int tid = threadIdx.x;
  const int warp = tid >> 5;
  const int m0 = blockIdx.x * kTileM;
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_u32(&tmem_base)),
                 "r"((uint32_t)N)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  if (tid == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&mbar)) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = tmem_base;
  constexpr uint32_t idesc = instr_desc(N);
  const int ktiles = K / kTileK;
  bool ok = true;
  for (int kt = 0; kt < ktiles && ok; ++kt) {
    // stage the A and B tiles: 16-byte chunks (8 consecutive K values) per thread. Each
    // group of 8 threads takes the 8 rows of one core matrix (distinct shared-memory
    // banks); a warp reads 64 contiguous bytes of each of 8 rows.
    const int k0 = kt * kTileK;
    for (int c = tid; c < kTileM * (kTileK / 8); c += kThreads) {
      const int q = c >> 3;
      const int r = (q / (kTileK / 8)) * 8 + (c & 7), kc = (q % (kTileK / 8)) * 8;
      const uint4 v = *reinterpret_cast<const uint4*>(A + (size_t)(m0 + r) * K + k0 + kc);
      *reinterpret_cast<uint4*>(sa + tile_offset(r, kc)) = v;
    }
    for (int c = tid; c < N * (kTileK / 8); c += kThreads) {
      const int q = c >> 3;
      const int r = (q / (kTileK / 8)) * 8 + (c & 7), kc = (q % (kTileK / 8)) * 8;
      const uint4 v = *reinterpret_cast<const uint4*>(B + (size_t)r * K + k0 + kc);
      *reinterpret_cast<uint4*>(sb + tile_offset(r, kc)) = v;
    }
    // the generic-proxy stores must be visible to the tensor cores' async proxy
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    __syncthreads();
    if (tid == 0) {
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
#pragma unroll
      for (int kk = 0; kk < kTileK / 16; ++kk) {
        // K = 16 per MMA: two core matrices along K (2 x 128 bytes) further each time
        const uint64_t ad = smem_desc(smem_u32(sa) + kk * 256, 128, (kTileK / 8) * 128);
        const uint64_t bd = smem_desc(smem_u32(sb) + kk * 256, 128, (kTileK / 8) * 128);
        const uint32_t acc = (kt > 0 || kk > 0) ? 1u : 0u;
        asm volatile(
            "{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\n"
            "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem),
            "l"(ad), "l"(bd), "r"(idesc), "r"(acc)
            : "memory");
      }
      asm volatile(
          "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
              smem_u32(&mbar))
          : "memory");
    }
    // the MMAs read the staged tiles: wait before the next round overwrites them
    if (!wait_mbar(&mbar, (uint32_t)(kt & 1))) {
      if (tid == 0) atomicExch(&g_cm_error, TSG_ERR_TIMEOUT);
      ok = false;
    }
    __syncthreads();
  }
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  if (ok) epilogue<N>(tmem, smem, out, m0, ldo, bias, relu, out_f32);
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem),
                 "r"((uint32_t)N)
                 : "memory");
}

// The same product with the operand tiles loaded by the tensor memory accelerator:
// cp.async.bulk.tensor 2D boxes of 64 K x rows (128 bytes per row) written into shared
// memory in the 128-byte swizzled K-major layout, completion counted in bytes on an
// mbarrier; one thread issues the copies and the MMAs. K is staged 128 at a time (two
// boxes per operand).
constexpr int kTmaBoxK = 64;     // K per box: one 128-byte line per row
constexpr int kTmaRoundK = 128;  // K per round (two boxes per operand)

// Shared-memory descriptor of a K-major tile in the 128-byte swizzled layout TMA writes:
// 8-row groups 1024 bytes apart (SBO), leading offset unused (1), version 1, layout type
// 2 (128-byte swizzle, bits 61-63). A K step of 16 values moves the start by 32 bytes
// within the swizzled line; tiles are 1024-byte aligned (base offset 0).
__device__ __forceinline__ uint64_t smem_desc_sw128(uint32_t addr) {
  uint64_t d = 0;
  d |= (uint64_t)((addr >> 4) & 0x3FFF);
  d |= (uint64_t)1 << 16;
  d |= (uint64_t)(1024 >> 4) << 32;
  d |= (uint64_t)1 << 46;
  d |= (uint64_t)2 << 61;
  return d;
}

__device__ __forceinline__ void tma_load_2d(void* dst, const CUtensorMap* map, int x, int y,
                                            uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes "
      "[%0], [%1, {%2, %3}], [%4];" ::"r"(smem_u32(dst)),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(smem_u32(bar))
      : "memory");
}

template <int N>
constexpr int tma_smem_bytes() {
  return 1024 + (kTmaRoundK / kTmaBoxK) * (kTileM + N) * kTmaBoxK * 2;
}

template <int N>
__global__ void __launch_bounds__(kThreads, 1)
    gemm_bf16_tma_kernel(const __grid_constant__ CUtensorMap tma_a,
                         const __grid_constant__ CUtensorMap tma_b,
                         const float* __restrict__ bias, void* out, int K, int ldo, int relu,
                         int out_f32) {
  extern __shared__ uint8_t dyn_smem[];
  // 1024-byte aligned tiles: the round's A boxes, then its B boxes; afterwards the same
  // bytes stage the epilogue
  uint8_t* smem = reinterpret_cast<uint8_t*>(
      (reinterpret_cast<uintptr_t>(dyn_smem) + 1023) & ~static_cast<uintptr_t>(1023));
  constexpr int kABox = kTileM * kTmaBoxK * 2;
  constexpr int kBBox = N * kTmaBoxK * 2;
  static_assert((kTmaRoundK / kTmaBoxK) * kABox >= 4 * kStagePerWarp, "epilogue stage");
  uint8_t* sa = smem;
  uint8_t* sb = smem + (kTmaRoundK / kTmaBoxK) * kABox;
  __shared__ __align__(8) uint64_t full;
  __shared__ __align__(8) uint64_t mma_done;
  __shared__ uint32_t tmem_base;
  __shared__ int round_ok;
  const int tid = threadIdx.x;
  const int warp = tid >> 5;
  const int m0 = blockIdx.x * kTileM;
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_u32(&tmem_base)),
                 "r"((uint32_t)N)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  if (tid == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&full)) : "memory");
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&mma_done)) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = tmem_base;
  constexpr uint32_t idesc = instr_desc(N);
  const int rounds = (K + kTmaRoundK - 1) / kTmaRoundK;
  bool ok = true;
  for (int r = 0; r < rounds && ok; ++r) {
    const int k0 = r * kTmaRoundK;
    const int boxes = min(kTmaRoundK, K - k0) / kTmaBoxK;
    if (tid == 0) {
      const uint32_t bytes = (uint32_t)boxes * (kABox + kBBox);
      asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(
                       smem_u32(&full)),
                   "r"(bytes)
                   : "memory");
      for (int c = 0; c < boxes; ++c) {
        tma_load_2d(sa + c * kABox, &tma_a, k0 + c * kTmaBoxK, m0, &full);
        tma_load_2d(sb + c * kBBox, &tma_b, k0 + c * kTmaBoxK, 0, &full);
      }
      int good = wait_mbar(&full, (uint32_t)(r & 1)) ? 1 : 0;
      if (good) {
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        for (int c = 0; c < boxes; ++c) {
#pragma unroll
          for (int kk = 0; kk < kTmaBoxK / 16; ++kk) {
            const uint64_t ad = smem_desc_sw128(smem_u32(sa + c * kABox) + kk * 32);
            const uint64_t bd = smem_desc_sw128(smem_u32(sb + c * kBBox) + kk * 32);
            const uint32_t acc = (r > 0 || c > 0 || kk > 0) ? 1u : 0u;
            asm volatile(
                "{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\n"
                "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem),
                "l"(ad), "l"(bd), "r"(idesc), "r"(acc)
                : "memory");
          }
        }
        asm volatile(
            "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                smem_u32(&mma_done))
            : "memory");
      } else {
        atomicExch(&g_cm_error, TSG_ERR_TIMEOUT);
        wait_mbar(&full, (uint32_t)(r & 1));  // the copies in flight, once more (bounded)
      }
      round_ok = good;
    }
    __syncthreads();
    ok = round_ok != 0;
    // the MMAs read this round's tiles: wait before the next round or the epilogue
    if (ok && !wait_mbar(&mma_done, (uint32_t)(r & 1))) {
      if (tid == 0) atomicExch(&g_cm_error, TSG_ERR_TIMEOUT);
      ok = false;
    }
    __syncthreads();
  }
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  if (ok) epilogue<N>(tmem, smem, out, m0, ldo, bias, relu, out_f32);
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem),
                 "r"((uint32_t)N)
                 : "memory");
}

// Sum of each node's children's rows: out[v] = sum over children u of h[u] (BF16 rows of
// width w, FP32 sum; the tree's child lists in CSR form: child[cstart[v] .. cstart[v+1])).
__global__ void child_sum_kernel(const __nv_bfloat16* __restrict__ h, const int32_t* __restrict__ cstart,
                                 const int32_t* __restrict__ child, __nv_bfloat16* __restrict__ out,
                                 int64_t n, int w, int ldo) {
  const int64_t v = blockIdx.x;
  if (v >= n) return;
  for (int j = threadIdx.x; j < w; j += blockDim.x) {
    float acc = 0.f;
    for (int32_t e = cstart[v]; e < cstart[v + 1]; ++e) acc += __bfloat162float(h[(int64_t)child[e] * w + j]);
    out[v * ldo + j] = __float2bfloat16(acc);
  }
}

// Transpose of child_sum for the backward pass: dh[u] += dc[parent[u]] (FP32 rows), for
// every node u with a parent (parent[u] >= 0).
__global__ void parent_add_kernel(const float* __restrict__ dc, int ldc,
                                  const int32_t* __restrict__ parent, float* __restrict__ dh,
                                  int64_t n, int w) {
  const int64_t u = blockIdx.x;
  if (u >= n) return;
  const int32_t p = parent[u];
  if (p < 0) return;
  for (int j = threadIdx.x; j < w; j += blockDim.x) dh[u * w + j] += dc[(int64_t)p * ldc + j];
}

// out[i][j] = sum_n a[n][i] * b[n][j] (FP32; a: n x p, b: n x q, row-major): the weight
// gradients, a reduction over the nodes. 32 x 32 output tiles, the node range split over
// gridDim.z slabs accumulated with atomics (out cleared by the caller).
__global__ void __launch_bounds__(256)
    gemm_at_b_kernel(const float* __restrict__ a, int p, const float* __restrict__ b, int q,
                     int64_t n, float* __restrict__ out) {
  __shared__ float sa[32][33], sb[32][33];
  const int ti = threadIdx.x / 32, tj = threadIdx.x % 32;  // 8 x 32 threads
  const int i0 = blockIdx.y * 32, j0 = blockIdx.x * 32;
  const int64_t slab = (n + gridDim.z - 1) / gridDim.z;
  const int64_t n0 = blockIdx.z * slab, n1 = n0 + slab < n ? n0 + slab : n;
  float acc[4] = {0.f, 0.f, 0.f, 0.f};
  for (int64_t k0 = n0; k0 < n1; k0 += 32) {
    for (int r = ti; r < 32; r += 8) {
      const int64_t row = k0 + r;
      sa[r][tj] = (row < n1 && i0 + tj < p) ? a[row * p + i0 + tj] : 0.f;
      sb[r][tj] = (row < n1 && j0 + tj < q) ? b[row * q + j0 + tj] : 0.f;
    }
    __syncthreads();
#pragma unroll 8
    for (int r = 0; r < 32; ++r) {
      const float bv = sb[r][tj];
#pragma unroll
      for (int x = 0; x < 4; ++x) acc[x] += sa[r][ti + 8 * x] * bv;
    }
    __syncthreads();
  }
#pragma unroll
  for (int x = 0; x < 4; ++x) {
    const int i = i0 + ti + 8 * x, j = j0 + tj;
    if (i < p && j < q) atomicAdd(&out[(int64_t)i * q + j], acc[x]);
  }
}

// One Adam step (Kingma & Ba, 2015) on FP32 parameters with bias-corrected moments.
__global__ void adam_kernel(float* __restrict__ w, const float* __restrict__ g,
                            float* __restrict__ m, float* __restrict__ v, int64_t n, float lr,
                            float b1, float b2, float eps, float c1, float c2) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float gi = g[i];
  const float mi = b1 * m[i] + (1.f - b1) * gi;
  const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
  m[i] = mi;
  v[i] = vi;
  w[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
}

// Host side of the TMA form: the driver's tensor-map encoder, reached through the
// runtime's entry-point query (the library links only the runtime), and the maps of the
// two operands.
std::atomic<int> g_gemm_mode{0};  // 0: TMA-loaded tiles (default), 1: thread-staged tiles

PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder() {
  static std::once_flag once;
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  std::call_once(once, [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault,
                                         &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
  });
  return fn;
}

// Map of a row-major BF16 matrix (rows x k, k contiguous) read in boxes of 64 K x box_rows
// rows, 128-byte swizzle.
tsg_status operand_map(CUtensorMap* map, const void* ptr, uint64_t rows, uint64_t k,
                       uint32_t box_rows) {
  auto encode = tensor_map_encoder();
  if (!encode) return fail(TSG_ERR_UNSUPPORTED, "cm_gemm: cuTensorMapEncodeTiled unavailable");
  const cuuint64_t dims[2] = {k, rows};
  const cuuint64_t strides[1] = {k * 2};
  const cuuint32_t box[2] = {(cuuint32_t)kTmaBoxK, box_rows};
  const cuuint32_t estr[2] = {1, 1};
  const CUresult r = encode(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void*>(ptr), dims,
                            strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                            CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                            CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS)
    return fail(TSG_ERR_INVALID_ARGUMENT, "cm_gemm: tensor map rejected (" + std::to_string((int)r) + ")");
  return TSG_OK;
}

template <int N>
tsg_status launch_gemm_tma(const void* a, const void* b, int64_t m, int64_t k, const float* bias,
                           int32_t relu, void* out, int64_t ldo, int32_t out_f32,
                           cudaStream_t st) {
  CUtensorMap ma, mb;
  TSG_TRY(operand_map(&ma, a, (uint64_t)m, (uint64_t)k, kTileM));
  TSG_TRY(operand_map(&mb, b, (uint64_t)N, (uint64_t)k, N));
  constexpr int smem = tma_smem_bytes<N>();
  // the shared-memory opt-in is per device: set it once on each device that launches
  static std::atomic<uint64_t> attr_set{0};
  int dev = 0;
  TSG_CUDA_TRY(cudaGetDevice(&dev));
  const uint64_t bit = dev < 64 ? (uint64_t(1) << dev) : 0;
  if (!bit || !(attr_set.load(std::memory_order_acquire) & bit)) {
    TSG_CUDA_TRY(cudaFuncSetAttribute(gemm_bf16_tma_kernel<N>,
                                      cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
    attr_set.fetch_or(bit, std::memory_order_release);
  }
  gemm_bf16_tma_kernel<N><<<(unsigned)(m / kTileM), kThreads, smem, st>>>(
      ma, mb, bias, out, (int)k, (int)ldo, relu, out_f32);
  TSG_CUDA_TRY(cudaGetLastError());
  return TSG_OK;
}

}  // namespace cm
}  // namespace tsg

using namespace tsg;

extern "C" {

tsg_status tsg_cm_gemm_bf16(int64_t m, int64_t n, int64_t k, const void* a_dev,
                            const void* b_dev, const float* bias_dev, int32_t relu,
                            void* out_dev, int64_t ldo, int32_t out_f32, void* stream) {
  if (!a_dev || !b_dev || !out_dev) return fail(TSG_ERR_INVALID_ARGUMENT, "cm_gemm: null pointer");
  if (m <= 0 || m % cm::kTileM || k <= 0 || k % cm::kTileK || (n != 64 && n != 128) ||
      ldo < n || m / cm::kTileM > 0x7fffffff)
    return fail(TSG_ERR_INVALID_ARGUMENT,
                "cm_gemm: M must be a multiple of 128, K of 64, N 64 or 128, ldo >= N");
  if (((uintptr_t)a_dev | (uintptr_t)b_dev | (uintptr_t)out_dev) & 15)
    return fail(TSG_ERR_INVALID_ARGUMENT, "cm_gemm: operands and output must be 16-byte aligned");
  if ((ldo * (out_f32 ? 4 : 2)) % 16 != 0)
    return fail(TSG_ERR_INVALID_ARGUMENT, "cm_gemm: output rows must be a multiple of 16 bytes apart");
  const dim3 grid((unsigned)(m / cm::kTileM));
  cudaStream_t st = (cudaStream_t)stream;
  if (cm::g_gemm_mode.load(std::memory_order_relaxed) == 0) {
    if (n == 64)
      return cm::launch_gemm_tma<64>(a_dev, b_dev, m, k, bias_dev, relu, out_dev, ldo, out_f32, st);
    return cm::launch_gemm_tma<128>(a_dev, b_dev, m, k, bias_dev, relu, out_dev, ldo, out_f32, st);
  }
  const auto* a = (const __nv_bfloat16*)a_dev;
  const auto* b = (const __nv_bfloat16*)b_dev;
  switch (n) {
    case 64:
      cm::gemm_bf16_tn_kernel<64><<<grid, cm::kThreads, 0, st>>>(a, b, bias_dev, out_dev, (int)k,
                                                                 (int)ldo, relu, out_f32);
      break;
    default:
      cm::gemm_bf16_tn_kernel<128><<<grid, cm::kThreads, 0, st>>>(a, b, bias_dev, out_dev, (int)k,
                                                                  (int)ldo, relu, out_f32);
      break;
  }
  TSG_CUDA_TRY(cudaGetLastError());
  return TSG_OK;
}

tsg_status tsg_cm_set_gemm_mode(int32_t mode) {
  if (mode != 0 && mode != 1)
    return fail(TSG_ERR_INVALID_ARGUMENT, "cm_set_gemm_mode: 0 (TMA) or 1 (thread-staged)");
  cm::g_gemm_mode.store(mode, std::memory_order_relaxed);
  return TSG_OK;
}

tsg_status tsg_cm_child_sum(const void* h_dev, const int32_t* cstart_dev, const int32_t* child_dev,
                            void* out_dev, int64_t n, int32_t width, int32_t ldo, void* stream) {
  if (!h_dev || !cstart_dev || !child_dev || !out_dev || n < 0 || width <= 0 || ldo < width)
    return fail(TSG_ERR_INVALID_ARGUMENT, "cm_child_sum: bad arguments");
  if (n == 0) return TSG_OK;
  cm::child_sum_kernel<<<(unsigned)n, 128, 0, (cudaStream_t)stream>>>(
      (const __nv_bfloat16*)h_dev, cstart_dev, child_dev, (__nv_bfloat16*)out_dev, n, width, ldo);
  TSG_CUDA_TRY(cudaGetLastError());
  return TSG_OK;
}

tsg_status tsg_cm_parent_add(const float* dc_dev, int32_t ldc, const int32_t* parent_dev,
                             float* dh_dev, int64_t n, int32_t width, void* stream) {
  if (!dc_dev || !parent_dev || !dh_dev || n < 0 || width <= 0 || ldc < width)
    return fail(TSG_ERR_INVALID_ARGUMENT, "cm_parent_add: bad arguments");
  if (n == 0) return TSG_OK;
  cm::parent_add_kernel<<<(unsigned)n, 128, 0, (cudaStream_t)stream>>>(dc_dev, ldc, parent_dev,
                                                                       dh_dev, n, width);
  TSG_CUDA_TRY(cudaGetLastError());
  return TSG_OK;
}

tsg_status tsg_cm_gemm_at_b(const float* a_dev, int32_t p, const float* b_dev, int32_t q,
                            int64_t n, float* out_dev, void* stream) {
  if (!a_dev || !b_dev || !out_dev || p <= 0 || q <= 0 || n < 0)
    return fail(TSG_ERR_INVALID_ARGUMENT, "cm_gemm_at_b: bad arguments");
  cudaStream_t st = (cudaStream_t)stream;
  TSG_CUDA_TRY(cudaMemsetAsync(out_dev, 0, sizeof(float) * (size_t)p * q, st));
  if (n == 0) return TSG_OK;
  const unsigned slabs = (unsigned)std::max<int64_t>(1, std::min<int64_t>(64, n / 4096));
  const dim3 grid((unsigned)((q + 31) / 32), (unsigned)((p + 31) / 32), slabs);
  cm::gemm_at_b_kernel<<<grid, 256, 0, st>>>(a_dev, p, b_dev, q, n, out_dev);
  TSG_CUDA_TRY(cudaGetLastError());
  return TSG_OK;
}

tsg_status tsg_cm_adam(float* w_dev, const float* g_dev, float* m_dev, float* v_dev, int64_t n,
                       float lr, float beta1, float beta2, float eps, int32_t step, void* stream) {
  if (!w_dev || !g_dev || !m_dev || !v_dev || n < 0 || step < 1)
    return fail(TSG_ERR_INVALID_ARGUMENT, "cm_adam: bad arguments");
  if (n == 0) return TSG_OK;
  const float c1 = 1.f - powf(beta1, (float)step), c2 = 1.f - powf(beta2, (float)step);
  cm::adam_kernel<<<(unsigned)((n + 255) / 256), 256, 0, (cudaStream_t)stream>>>(
      w_dev, g_dev, m_dev, v_dev, n, lr, beta1, beta2, eps, c1, c2);
  TSG_CUDA_TRY(cudaGetLastError());
  return TSG_OK;
}

tsg_status tsg_cm_take_error(void* stream) {
  int err = 0;
  const int zero = 0;
  cudaStream_t st = (cudaStream_t)stream;
  TSG_CUDA_TRY(cudaMemcpyFromSymbolAsync(&err, cm::g_cm_error, sizeof(int), 0,
                                         cudaMemcpyDeviceToHost, st));
  TSG_CUDA_TRY(cudaStreamSynchronize(st));
  if (err == 0) return TSG_OK;
  TSG_CUDA_TRY(cudaMemcpyToSymbolAsync(cm::g_cm_error, &zero, sizeof(int), 0,
                                       cudaMemcpyHostToDevice, st));
  TSG_CUDA_TRY(cudaStreamSynchronize(st));
  return fail(TSG_ERR_TIMEOUT, "cost model: a bounded wait for the tensor-core MMAs gave up");
}

}  // extern "C"
