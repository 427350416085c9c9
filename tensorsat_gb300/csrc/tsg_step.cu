// Box-level (per-step) operations of the tensorsat_gb300 C ABI: pairwise contraction of
// dense tensors with arbitrary port dimensions in the OR-AND semiring (FinRel._contract2,
// tensorsat/lang/fin_rel.py:255-288) or over uint64 counts, port rewiring
// (FinRel._rewire, tensorsat/lang/fin_rel.py:379-393), union and spider tensors.
//
// These calls serve the drop-in box class one step at a time; the hot loop over a whole
// contraction tree lives in tsg_tree.cu.

#include <algorithm>
#include <cstring>
#include <map>
#include <vector>

#include "tsg_common.cuh"

namespace tsg {

static thread_local std::string g_last_error;

tsg_status fail(tsg_status code, const std::string& msg) {
  g_last_error = msg;
  return code;
}

tsg_status cuda_status(cudaError_t err, const char* what) {
  (void)cudaGetLastError();  // clear a sticky launch error so later calls start clean
  return fail(TSG_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(err));
}

int device_sm_count() {
  static int cached[64] = {0};
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return 148;
  if (cached[dev] == 0) {
    int n = 0;
    if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n <= 0)
      n = 148;
    cached[dev] = n;
  }
  return cached[dev];
}

namespace {

constexpr int kMaxWires = 2 * TSG_MAX_PORTS;  // distinct wires of one contraction

// Index description of one generic contraction. Output ports are decoded from the output
// linear index (last port fastest). Each distinct wire among the output ports contributes
// its coordinate times its summed strides in lhs / rhs once ("owner" port); further ports
// carrying the same wire only check that their coordinate agrees (diagonal), else the
// entry is zero. Summed wires are walked by an odometer.
struct GenericArgs {
  int32_t n_out;
  int32_t n_sum;
  int32_t n_wires;        // distinct wires on output ports
  int32_t rhs_is_one;     // rhs is the scalar 1 (used by rewire)
  int64_t total;          // output entries
  int64_t ksize;          // size of the summed index space
  int64_t out_dim[TSG_MAX_PORTS];
  int32_t out_wire[TSG_MAX_PORTS];   // distinct-wire id of each output port
  int64_t wire_ls[kMaxWires];        // lhs stride of each distinct output wire
  int64_t wire_rs[kMaxWires];
  int64_t sum_dim[kMaxWires];
  int64_t sum_ls[kMaxWires];
  int64_t sum_rs[kMaxWires];
  int64_t lhs_numel, rhs_numel;  // plane strides of the modular form
  uint32_t mod[TSG_MAX_PRIMES];  // moduli of the modular form, one per plane
};

// lhs / rhs offsets of output entry t; false off the diagonal of repeated output wires
// (the entry is then zero).
__device__ __forceinline__ bool decode_output(const GenericArgs& a, int64_t t, int64_t* lo_out,
                                              int64_t* ro_out) {
  int64_t coord[kMaxWires];
  for (int w = 0; w < a.n_wires; ++w) coord[w] = -1;
  int64_t rem = t, lo = 0, ro = 0;
  bool on_diagonal = true;
  for (int p = a.n_out - 1; p >= 0; --p) {
    const int64_t d = a.out_dim[p];
    const int64_t c = rem % d;
    rem /= d;
    const int w = a.out_wire[p];
    if (coord[w] < 0) {
      coord[w] = c;
      lo += c * a.wire_ls[w];
      ro += c * a.wire_rs[w];
    } else if (coord[w] != c) {
      on_diagonal = false;
    }
  }
  *lo_out = lo;
  *ro_out = ro;
  return on_diagonal;
}

// Modulus of plane q, selected without dynamic indexing of the parameter block.
__device__ __forceinline__ uint32_t plane_mod(const GenericArgs& a, int q) {
  uint32_t m = a.mod[0];
#pragma unroll
  for (int i = 1; i < TSG_MAX_PRIMES; ++i)
    if (q == i) m = a.mod[i];
  return m;
}

// Residues mod p (plain, 0 <= x < p) of every plane (blockIdx.y): out = sum of lhs * rhs
// over the summed wires, each product reduced mod p and the sum once more at the end.
__global__ void generic_modp_kernel(const uint32_t* __restrict__ lhs,
                                    const uint32_t* __restrict__ rhs, uint32_t* __restrict__ out,
                                    GenericArgs a) {
  const int q = blockIdx.y;
  const uint64_t p = plane_mod(a, q);
  const uint32_t* L = lhs + q * a.lhs_numel;
  const uint32_t* R = rhs + q * a.rhs_numel;
  uint32_t* O = out + q * a.total;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < a.total; t += stride) {
    int64_t lo, ro;
    uint64_t acc = 0;
    if (decode_output(a, t, &lo, &ro)) {
      int64_t kc[kMaxWires];
      for (int i = 0; i < a.n_sum; ++i) kc[i] = 0;
      int64_t klo = 0, kro = 0;
      int64_t terms = 0;
      while (true) {
        acc += ((uint64_t)L[lo + klo] * R[ro + kro]) % p;
        if (++terms == (int64_t(1) << 30)) {  // sums of reduced products stay below 2^62
          acc %= p;
          terms = 0;
        }
        int i = a.n_sum - 1;
        for (; i >= 0; --i) {
          if (++kc[i] < a.sum_dim[i]) {
            klo += a.sum_ls[i];
            kro += a.sum_rs[i];
            break;
          }
          klo -= (a.sum_dim[i] - 1) * a.sum_ls[i];
          kro -= (a.sum_dim[i] - 1) * a.sum_rs[i];
          kc[i] = 0;
        }
        if (i < 0) break;
      }
    }
    O[t] = (uint32_t)(acc % p);
  }
}

// Split-K form of the modular contraction: one block per output entry and plane.
__global__ void generic_modp_splitk_kernel(const uint32_t* __restrict__ lhs,
                                           const uint32_t* __restrict__ rhs,
                                           uint32_t* __restrict__ out, GenericArgs a) {
  __shared__ uint64_t red[128];
  const int q = blockIdx.y;
  const uint64_t p = plane_mod(a, q);
  const uint32_t* L = lhs + q * a.lhs_numel;
  const uint32_t* R = rhs + q * a.rhs_numel;
  uint32_t* O = out + q * a.total;
  for (int64_t t = blockIdx.x; t < a.total; t += gridDim.x) {
    int64_t lo, ro;
    uint64_t acc = 0;
    if (decode_output(a, t, &lo, &ro)) {
      for (int64_t kk = threadIdx.x; kk < a.ksize; kk += blockDim.x) {
        int64_t r2 = kk, klo = 0, kro = 0;
        for (int i = a.n_sum - 1; i >= 0; --i) {
          const int64_t c = r2 % a.sum_dim[i];
          r2 /= a.sum_dim[i];
          klo += c * a.sum_ls[i];
          kro += c * a.sum_rs[i];
        }
        acc = (acc + ((uint64_t)L[lo + klo] * R[ro + kro]) % p) % p;
      }
    }
    red[threadIdx.x] = acc;
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1) {
      if ((int)threadIdx.x < s) red[threadIdx.x] = (red[threadIdx.x] + red[threadIdx.x + s]) % p;
      __syncthreads();
    }
    if (threadIdx.x == 0) O[t] = (uint32_t)red[0];
    __syncthreads();
  }
}

template <typename T, bool kOrAnd>
__global__ void generic_contract_kernel(const T* __restrict__ lhs, const T* __restrict__ rhs,
                                        T* __restrict__ out, GenericArgs a) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < a.total; t += stride) {
    int64_t coord[kMaxWires];
    for (int w = 0; w < a.n_wires; ++w) coord[w] = -1;
    int64_t rem = t, lo = 0, ro = 0;
    bool on_diagonal = true;
    for (int p = a.n_out - 1; p >= 0; --p) {
      const int64_t d = a.out_dim[p];
      const int64_t c = rem % d;
      rem /= d;
      const int w = a.out_wire[p];
      if (coord[w] < 0) {
        coord[w] = c;
        lo += c * a.wire_ls[w];
        ro += c * a.wire_rs[w];
      } else if (coord[w] != c) {
        on_diagonal = false;
      }
    }
    T acc = 0;
    if (on_diagonal) {
      int64_t kc[kMaxWires];
      for (int i = 0; i < a.n_sum; ++i) kc[i] = 0;
      int64_t klo = 0, kro = 0;
      while (true) {
        const T l = lhs[lo + klo];
        const T r = a.rhs_is_one ? (T)1 : rhs[ro + kro];
        if (kOrAnd) {
          acc |= (T)(l & r);
        } else {
          acc += l * r;
        }
        // odometer over the summed wires, last wire fastest
        int i = a.n_sum - 1;
        for (; i >= 0; --i) {
          if (++kc[i] < a.sum_dim[i]) {
            klo += a.sum_ls[i];
            kro += a.sum_rs[i];
            break;
          }
          klo -= (a.sum_dim[i] - 1) * a.sum_ls[i];
          kro -= (a.sum_dim[i] - 1) * a.sum_rs[i];
          kc[i] = 0;
        }
        if (i < 0) break;
      }
      if (kOrAnd) acc = acc ? (T)1 : (T)0;
    }
    out[t] = acc;
  }
}

// Split-K form for few outputs over a large summed space: one block per output entry,
// threads stride over the summed index (decoded per thread), then a block reduction.
template <typename T, bool kOrAnd>
__global__ void generic_contract_splitk_kernel(const T* __restrict__ lhs,
                                               const T* __restrict__ rhs, T* __restrict__ out,
                                               GenericArgs a, int64_t ksize) {
  __shared__ T red[128];
  for (int64_t t = blockIdx.x; t < a.total; t += gridDim.x) {
    int64_t coord[kMaxWires];
    for (int w = 0; w < a.n_wires; ++w) coord[w] = -1;
    int64_t rem = t, lo = 0, ro = 0;
    bool on_diagonal = true;
    for (int p = a.n_out - 1; p >= 0; --p) {
      const int64_t d = a.out_dim[p];
      const int64_t c = rem % d;
      rem /= d;
      const int w = a.out_wire[p];
      if (coord[w] < 0) {
        coord[w] = c;
        lo += c * a.wire_ls[w];
        ro += c * a.wire_rs[w];
      } else if (coord[w] != c) {
        on_diagonal = false;
      }
    }
    T acc = 0;
    if (on_diagonal) {
      for (int64_t kk = threadIdx.x; kk < ksize; kk += blockDim.x) {
        int64_t r2 = kk, klo = 0, kro = 0;
        for (int i = a.n_sum - 1; i >= 0; --i) {
          const int64_t c = r2 % a.sum_dim[i];
          r2 /= a.sum_dim[i];
          klo += c * a.sum_ls[i];
          kro += c * a.sum_rs[i];
        }
        const T l = lhs[lo + klo];
        const T r = a.rhs_is_one ? (T)1 : rhs[ro + kro];
        if (kOrAnd) {
          acc |= (T)(l & r);
        } else {
          acc += l * r;
        }
      }
    }
    red[threadIdx.x] = acc;
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1) {
      if ((int)threadIdx.x < s) {
        if (kOrAnd) {
          red[threadIdx.x] |= red[threadIdx.x + s];
        } else {
          red[threadIdx.x] += red[threadIdx.x + s];
        }
      }
      __syncthreads();
    }
    if (threadIdx.x == 0) out[t] = kOrAnd ? (red[0] ? (T)1 : (T)0) : red[0];
    __syncthreads();
  }
}

bool mul_overflows(int64_t a, int64_t b, int64_t* out) {
  if (a < 0 || b < 0) return true;
  if (a != 0 && b > INT64_MAX / a) return true;
  *out = a * b;
  return false;
}

// Builds GenericArgs from the einsum-style description; validates everything the kernel
// relies on. `rhs_rank < 0` means "rhs is the scalar 1".
tsg_status build_generic(int32_t lhs_rank, const int64_t* lhs_wires, const int64_t* lhs_dims,
                         int32_t rhs_rank, const int64_t* rhs_wires, const int64_t* rhs_dims,
                         int32_t out_rank, const int64_t* out_wires, GenericArgs* a) {
  const bool rhs_one = rhs_rank < 0;
  if (rhs_one) rhs_rank = 0;
  if (lhs_rank < 0 || lhs_rank > TSG_MAX_PORTS || rhs_rank > TSG_MAX_PORTS || out_rank < 0 ||
      out_rank > TSG_MAX_PORTS)
    return fail(TSG_ERR_INVALID_ARGUMENT, "contract2: ranks must lie in [0, 64]");
  if ((lhs_rank > 0 && (!lhs_wires || !lhs_dims)) || (rhs_rank > 0 && (!rhs_wires || !rhs_dims)) ||
      (out_rank > 0 && !out_wires))
    return fail(TSG_ERR_INVALID_ARGUMENT, "contract2: missing wire or dim array");
  std::map<int64_t, int64_t> dim_of;
  auto note = [&](int64_t w, int64_t d) -> bool {
    if (d <= 0) return false;
    auto it = dim_of.find(w);
    if (it == dim_of.end()) {
      dim_of[w] = d;
      return true;
    }
    return it->second == d;
  };
  for (int i = 0; i < lhs_rank; ++i)
    if (!note(lhs_wires[i], lhs_dims[i]))
      return fail(TSG_ERR_INVALID_ARGUMENT, "contract2: inconsistent or non-positive lhs dims");
  for (int i = 0; i < rhs_rank; ++i)
    if (!note(rhs_wires[i], rhs_dims[i]))
      return fail(TSG_ERR_INVALID_ARGUMENT, "contract2: inconsistent or non-positive rhs dims");
  for (int i = 0; i < out_rank; ++i)
    if (dim_of.find(out_wires[i]) == dim_of.end())
      return fail(TSG_ERR_INVALID_ARGUMENT, "contract2: every output wire must appear in lhs or rhs");
  // strides of the operands (C order) summed per wire
  auto strides = [](int32_t rank, const int64_t* wires, const int64_t* dims,
                    std::map<int64_t, int64_t>* acc) -> bool {
    int64_t s = 1;
    for (int i = rank - 1; i >= 0; --i) {
      (*acc)[wires[i]] += s;
      if (mul_overflows(s, dims[i], &s)) return false;
    }
    return true;
  };
  std::map<int64_t, int64_t> ls, rs;
  if (!strides(lhs_rank, lhs_wires, lhs_dims, &ls) || !strides(rhs_rank, rhs_wires, rhs_dims, &rs))
    return fail(TSG_ERR_TOO_LARGE, "contract2: operand size overflows int64");
  std::memset(a, 0, sizeof(*a));
  a->n_out = out_rank;
  a->rhs_is_one = rhs_one ? 1 : 0;
  a->lhs_numel = a->rhs_numel = 1;
  for (int i = 0; i < lhs_rank; ++i)
    if (mul_overflows(a->lhs_numel, lhs_dims[i], &a->lhs_numel))
      return fail(TSG_ERR_TOO_LARGE, "contract2: operand size overflows int64");
  for (int i = 0; i < rhs_rank; ++i)
    if (mul_overflows(a->rhs_numel, rhs_dims[i], &a->rhs_numel))
      return fail(TSG_ERR_TOO_LARGE, "contract2: operand size overflows int64");
  std::map<int64_t, int> out_id;
  int64_t total = 1;
  for (int p = 0; p < out_rank; ++p) {
    const int64_t w = out_wires[p];
    auto it = out_id.find(w);
    int id;
    if (it == out_id.end()) {
      id = (int)out_id.size();
      out_id[w] = id;
      a->wire_ls[id] = ls.count(w) ? ls[w] : 0;
      a->wire_rs[id] = rs.count(w) ? rs[w] : 0;
    } else {
      id = it->second;
    }
    a->out_wire[p] = id;
    a->out_dim[p] = dim_of[w];
    if (mul_overflows(total, dim_of[w], &total))
      return fail(TSG_ERR_TOO_LARGE, "contract2: output size overflows int64");
  }
  a->n_wires = (int)out_id.size();
  a->total = total;
  int ns = 0;
  int64_t ksize = 1;
  for (auto& kv : dim_of) {
    if (out_id.count(kv.first)) continue;
    if (ns >= kMaxWires) return fail(TSG_ERR_UNSUPPORTED, "contract2: too many summed wires");
    a->sum_dim[ns] = kv.second;
    a->sum_ls[ns] = ls.count(kv.first) ? ls[kv.first] : 0;
    a->sum_rs[ns] = rs.count(kv.first) ? rs[kv.first] : 0;
    if (mul_overflows(ksize, kv.second, &ksize))
      return fail(TSG_ERR_TOO_LARGE, "contract2: summed index space overflows int64");
    ++ns;
  }
  a->n_sum = ns;
  a->ksize = ksize;
  return TSG_OK;
}

template <typename T, bool kOrAnd>
tsg_status launch_generic(const T* lhs, const T* rhs, T* out, const GenericArgs& a,
                          cudaStream_t stream) {
  if (a.total == 0) return TSG_OK;
  const unsigned threads = 128;
  if (a.ksize > 256 && a.total < 4096) {
    // few outputs over a large summed space: spread each output's sum over a block
    const unsigned blocks = (unsigned)std::min<int64_t>(a.total, (int64_t)device_sm_count() * 8);
    generic_contract_splitk_kernel<T, kOrAnd>
        <<<blocks, threads, 0, stream>>>(lhs, rhs, out, a, a.ksize);
  } else {
    generic_contract_kernel<T, kOrAnd>
        <<<grid_for((uint64_t)a.total, threads, 8), threads, 0, stream>>>(lhs, rhs, out, a);
  }
  TSG_CUDA_TRY(cudaGetLastError());
  return TSG_OK;
}

__global__ void union_or_kernel(const uint8_t* __restrict__ a, const uint8_t* __restrict__ b,
                                uint8_t* __restrict__ out, int64_t n) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride)
    out[i] = a[i] | b[i];
}

__global__ void spider_kernel(uint8_t* __restrict__ out, int64_t n, int64_t diag_step) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride)
    out[i] = (i % diag_step == 0) ? 1 : 0;
}

}  // namespace
}  // namespace tsg

using namespace tsg;

extern "C" {

const char* tsg_last_error(void) { return g_last_error.c_str(); }

int32_t tsg_abi_version(void) { return 1; }

tsg_status tsg_contract2_or_and(const uint8_t* lhs_dev, int32_t lhs_rank,
                                const int64_t* lhs_wires, const int64_t* lhs_dims,
                                const uint8_t* rhs_dev, int32_t rhs_rank,
                                const int64_t* rhs_wires, const int64_t* rhs_dims,
                                int32_t out_rank, const int64_t* out_wires, uint8_t* out_dev,
                                void* stream) {
  if (!lhs_dev || !rhs_dev || !out_dev)
    return fail(TSG_ERR_INVALID_ARGUMENT, "contract2: null tensor pointer");
  if (rhs_rank < 0) return fail(TSG_ERR_INVALID_ARGUMENT, "contract2: negative rhs rank");
  GenericArgs a;
  TSG_TRY(build_generic(lhs_rank, lhs_wires, lhs_dims, rhs_rank, rhs_wires, rhs_dims, out_rank,
                        out_wires, &a));
  return launch_generic<uint8_t, true>(lhs_dev, rhs_dev, out_dev, a, (cudaStream_t)stream);
}

tsg_status tsg_contract2_count_u64(const uint64_t* lhs_dev, int32_t lhs_rank,
                                   const int64_t* lhs_wires, const int64_t* lhs_dims,
                                   const uint64_t* rhs_dev, int32_t rhs_rank,
                                   const int64_t* rhs_wires, const int64_t* rhs_dims,
                                   int32_t out_rank, const int64_t* out_wires, uint64_t* out_dev,
                                   void* stream) {
  if (!lhs_dev || !rhs_dev || !out_dev)
    return fail(TSG_ERR_INVALID_ARGUMENT, "contract2: null tensor pointer");
  if (rhs_rank < 0) return fail(TSG_ERR_INVALID_ARGUMENT, "contract2: negative rhs rank");
  GenericArgs a;
  TSG_TRY(build_generic(lhs_rank, lhs_wires, lhs_dims, rhs_rank, rhs_wires, rhs_dims, out_rank,
                        out_wires, &a));
  return launch_generic<uint64_t, false>(lhs_dev, rhs_dev, out_dev, a, (cudaStream_t)stream);
}

tsg_status tsg_contract2_modp(const uint32_t* lhs_dev, int32_t lhs_rank,
                              const int64_t* lhs_wires, const int64_t* lhs_dims,
                              const uint32_t* rhs_dev, int32_t rhs_rank,
                              const int64_t* rhs_wires, const int64_t* rhs_dims,
                              int32_t out_rank, const int64_t* out_wires, int32_t num_primes,
                              const uint32_t* primes, uint32_t* out_dev, void* stream) {
  if (!lhs_dev || !rhs_dev || !out_dev)
    return fail(TSG_ERR_INVALID_ARGUMENT, "contract2: null tensor pointer");
  if (rhs_rank < 0) return fail(TSG_ERR_INVALID_ARGUMENT, "contract2: negative rhs rank");
  if (num_primes < 1 || num_primes > TSG_MAX_PRIMES || !primes)
    return fail(TSG_ERR_INVALID_ARGUMENT, "contract2_modp: 1..4 moduli expected");
  GenericArgs a;
  TSG_TRY(build_generic(lhs_rank, lhs_wires, lhs_dims, rhs_rank, rhs_wires, rhs_dims, out_rank,
                        out_wires, &a));
  for (int q = 0; q < num_primes; ++q) {
    if (primes[q] < 2) return fail(TSG_ERR_INVALID_ARGUMENT, "contract2_modp: moduli must be >= 2");
    a.mod[q] = primes[q];
  }
  if (a.total == 0) return TSG_OK;
  cudaStream_t st = (cudaStream_t)stream;
  const unsigned threads = 128;
  if (a.ksize > 256 && a.total < 4096) {
    const unsigned blocks = (unsigned)std::min<int64_t>(a.total, (int64_t)device_sm_count() * 8);
    generic_modp_splitk_kernel<<<dim3(blocks, (unsigned)num_primes), threads, 0, st>>>(
        lhs_dev, rhs_dev, out_dev, a);
  } else {
    generic_modp_kernel<<<dim3(grid_for((uint64_t)a.total, threads, 8), (unsigned)num_primes),
                          threads, 0, st>>>(lhs_dev, rhs_dev, out_dev, a);
  }
  TSG_CUDA_TRY(cudaGetLastError());
  return TSG_OK;
}

tsg_status tsg_rewire_or_and(const uint8_t* in_dev, int32_t rank, const int64_t* dims,
                             int32_t out_rank, const int32_t* out_ports, uint8_t* out_dev,
                             void* stream) {
  if (!in_dev || !out_dev) return fail(TSG_ERR_INVALID_ARGUMENT, "rewire: null tensor pointer");
  if (rank < 0 || rank > TSG_MAX_PORTS || out_rank < 0 || out_rank > TSG_MAX_PORTS)
    return fail(TSG_ERR_INVALID_ARGUMENT, "rewire: ranks must lie in [0, 64]");
  if ((rank > 0 && !dims) || (out_rank > 0 && !out_ports))
    return fail(TSG_ERR_INVALID_ARGUMENT, "rewire: missing dims or ports");
  std::vector<int64_t> wires(rank), outw(out_rank);
  for (int i = 0; i < rank; ++i) wires[i] = i;
  for (int i = 0; i < out_rank; ++i) {
    if (out_ports[i] < 0 || out_ports[i] >= rank)
      return fail(TSG_ERR_INVALID_ARGUMENT, "rewire: output ports must be valid for the box");
    outw[i] = out_ports[i];
  }
  GenericArgs a;
  TSG_TRY(build_generic(rank, wires.data(), dims, -1, nullptr, nullptr, out_rank, outw.data(), &a));
  return launch_generic<uint8_t, true>(in_dev, in_dev, out_dev, a, (cudaStream_t)stream);
}

tsg_status tsg_union_or(const uint8_t* a_dev, const uint8_t* b_dev, uint8_t* out_dev, int64_t n,
                        void* stream) {
  if (n < 0) return fail(TSG_ERR_INVALID_ARGUMENT, "union: negative size");
  if (n == 0) return TSG_OK;
  if (!a_dev || !b_dev || !out_dev) return fail(TSG_ERR_INVALID_ARGUMENT, "union: null pointer");
  const unsigned threads = 256;
  union_or_kernel<<<grid_for((uint64_t)n, threads, 8), threads, 0, (cudaStream_t)stream>>>(
      a_dev, b_dev, out_dev, n);
  TSG_CUDA_TRY(cudaGetLastError());
  return TSG_OK;
}

tsg_status tsg_spider_fill(uint8_t* out_dev, int64_t dim, int32_t num_ports, void* stream) {
  if (!out_dev) return fail(TSG_ERR_INVALID_ARGUMENT, "spider: null pointer");
  if (dim <= 0 || num_ports <= 0 || num_ports > TSG_MAX_PORTS)
    return fail(TSG_ERR_INVALID_ARGUMENT, "spider: dim and number of ports must be positive");
  int64_t n = 1, diag = 0, pw = 1;
  for (int p = 0; p < num_ports; ++p) {
    diag += pw;  // diagonal step = 1 + dim + dim^2 + ... + dim^(ports-1)
    if (mul_overflows(n, dim, &n)) return fail(TSG_ERR_TOO_LARGE, "spider: size overflows int64");
    if (p + 1 < num_ports && mul_overflows(pw, dim, &pw))
      return fail(TSG_ERR_TOO_LARGE, "spider: size overflows int64");
  }
  const unsigned threads = 256;
  spider_kernel<<<grid_for((uint64_t)n, threads, 8), threads, 0, (cudaStream_t)stream>>>(
      out_dev, n, diag);
  TSG_CUDA_TRY(cudaGetLastError());
  return TSG_OK;
}

}  // extern "C"
