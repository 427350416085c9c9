// Device side of the tree executor, shared by its translation units: argument structs,
// the tree-step kernels (general, tile, streaming, root reduction) and the per-ring
// launch entry points. Each kernel instantiation is launched from exactly one translation
// unit (tsg_tree.cu: general and reduction kernels; tsg_tile_*.cu / tsg_stream_*.cu: tile
// and streaming kernels per ring), which compile in parallel.
#pragma once

#include <algorithm>
#include <cstring>
#include <type_traits>

#include "tsg_common.cuh"

namespace tsg {
namespace dev {


constexpr int kMaxRuns = 64;
constexpr int kThreads = 256;

struct BitMap {
  int32_t n;
  uint8_t src[kMaxRuns];
  uint8_t len[kMaxRuns];
  uint8_t dst[kMaxRuns];
};

struct StepArgs {
  const uint8_t* lhs;
  const uint8_t* rhs;
  uint8_t* out;
  uint64_t l_base, r_base;             // constant element offsets
  uint64_t l_plane, r_plane, o_plane;  // residue-plane strides (elements)
  uint64_t total;                      // output entries of this launch
  int32_t k_bits;
  BitMap lt, lk, rt, rk;
};

// Residues mod p are kept in Montgomery form (x * 2^32 mod p) in every intermediate; the
// root reduction converts back, so results are plain residues.
struct RingArgs {
  int32_t np;
  uint32_t p[TSG_MAX_PRIMES];
  uint64_t m[TSG_MAX_PRIMES];     // Barrett constants floor((2^64-1)/p)
  uint32_t pinv[TSG_MAX_PRIMES];  // -p^-1 mod 2^32
  uint32_t r1[TSG_MAX_PRIMES];    // 2^32 mod p (Montgomery form of 1)
};

// Montgomery-form value of sum_k L*R for one output and prime, from the 64-bit sum of
// products `acc` (operands: plain 0/1 for leaves, Montgomery residues otherwise):
//   both leaves:   acc is a plain count <= 16      -> acc * (2^32 mod p) mod p
//   one leaf:      acc is a sum of <= 16 residues  -> reduce the small multiple
//   no leaf:       acc < 2 p^2 (two products)      -> Montgomery reduction
__device__ __forceinline__ uint32_t mont_finish(uint64_t acc, int leaves, const RingArgs& ring,
                                                int p) {
  if (leaves == 2) return small_mod(acc * ring.r1[p], ring.p[p]);
  if (leaves == 1) return small_mod(acc, ring.p[p]);
  return mont_redc(acc, ring.p[p], ring.pinv[p]);
}

// One plane's constants, selected from the kernel parameters without dynamic indexing
// (which would copy the parameter block to local memory).
struct PlaneConst {
  uint32_t p, pinv, r1;
};

__device__ __forceinline__ PlaneConst plane_const(const RingArgs& ring, int p) {
  PlaneConst c{ring.p[0], ring.pinv[0], ring.r1[0]};
#pragma unroll
  for (int i = 1; i < TSG_MAX_PRIMES; ++i)
    if (p == i) c = PlaneConst{ring.p[i], ring.pinv[i], ring.r1[i]};
  return c;
}

// mont_finish with the plane's constants in registers.
__device__ __forceinline__ uint32_t mont_finish_c(uint64_t acc, int leaves, const PlaneConst& c) {
  if (leaves == 2) return small_mod(acc * c.r1, c.p);
  if (leaves == 1) return small_mod(acc, c.p);
  return mont_redc(acc, c.p, c.pinv);
}

__device__ __forceinline__ uint64_t scatter_bits(const BitMap& m, uint64_t x) {
  uint64_t r = 0;
#pragma unroll 1
  for (int i = 0; i < m.n; ++i)
    r |= ((x >> m.src[i]) & ((1ull << m.len[i]) - 1ull)) << m.dst[i];
  return r;
}

template <bool kLeaf, typename T>
__device__ __forceinline__ T load_elem(const uint8_t* base, uint64_t off) {
  if constexpr (kLeaf) {
    return (T)base[off];
  } else {
    return reinterpret_cast<const T*>(base)[off];
  }
}

// One pairwise contraction step: out[t] = sum_k lhs[scatter(t,k)] * rhs[scatter(t,k)] in
// the ring kRing. kLLeaf / kRLeaf mark uint8 leaf operands (widened on load).
template <int kRing, bool kLLeaf, bool kRLeaf>
__global__ void __launch_bounds__(kThreads) tree_step_kernel(StepArgs a, RingArgs ring) {
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  const uint64_t nk = 1ull << a.k_bits;
  for (uint64_t t = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; t < a.total; t += stride) {
    const uint64_t lo = a.l_base + scatter_bits(a.lt, t);
    const uint64_t ro = a.r_base + scatter_bits(a.rt, t);
    if constexpr (kRing == TSG_RING_OR_AND) {
      uint32_t acc = 0;
      for (uint64_t kk = 0; kk < nk; ++kk) {
        acc |= (uint32_t)a.lhs[lo + scatter_bits(a.lk, kk)] &
               (uint32_t)a.rhs[ro + scatter_bits(a.rk, kk)];
      }
      a.out[t] = acc ? 1 : 0;
    } else if constexpr (kRing == TSG_RING_U64) {
      uint64_t acc = 0;
      for (uint64_t kk = 0; kk < nk; ++kk) {
        acc += load_elem<kLLeaf, uint64_t>(a.lhs, lo + scatter_bits(a.lk, kk)) *
               load_elem<kRLeaf, uint64_t>(a.rhs, ro + scatter_bits(a.rk, kk));
      }
      reinterpret_cast<uint64_t*>(a.out)[t] = acc;
    } else {
      // Montgomery residues; products of two residues are reduced pairwise (2 p^2 < p 2^32)
      constexpr int leaves = (kLLeaf ? 1 : 0) + (kRLeaf ? 1 : 0);
      uint32_t acc[TSG_MAX_PRIMES] = {0, 0, 0, 0};
      uint64_t part[TSG_MAX_PRIMES] = {0, 0, 0, 0};
      for (uint64_t kk = 0; kk < nk; ++kk) {
        const uint64_t lko = lo + scatter_bits(a.lk, kk);
        const uint64_t rko = ro + scatter_bits(a.rk, kk);
#pragma unroll
        for (int p = 0; p < TSG_MAX_PRIMES; ++p) {
          if (p < ring.np) {
            const uint32_t l = load_elem<kLLeaf, uint32_t>(a.lhs, lko + (kLLeaf ? 0 : p * a.l_plane));
            const uint32_t r = load_elem<kRLeaf, uint32_t>(a.rhs, rko + (kRLeaf ? 0 : p * a.r_plane));
            part[p] += (uint64_t)l * r;
            if (leaves == 0 ? (kk & 1) : ((kk & 15) == 15)) {
              acc[p] = add_mod(acc[p], mont_finish(part[p], leaves, ring, p), ring.p[p]);
              part[p] = 0;
            }
          }
        }
      }
      uint32_t* out = reinterpret_cast<uint32_t*>(a.out);
#pragma unroll
      for (int p = 0; p < TSG_MAX_PRIMES; ++p) {
        if (p < ring.np)
          out[t + p * a.o_plane] = add_mod(acc[p], mont_finish(part[p], leaves, ring, p), ring.p[p]);
      }
    }
  }
}

// Steps with few output entries and many summed combinations (the last steps of a small
// network sum every wire nothing else needs): one block per output entry, the block's
// threads split the summed combinations and combine them in shared memory, instead of one
// thread looping over all of them. MODP terms are kept as residues (Montgomery products
// reduced one by one, sums reduced before they pass 2^62); counts of two leaves are
// brought into Montgomery form at the end.
template <int kRing, bool kLLeaf, bool kRLeaf>
__global__ void __launch_bounds__(kThreads) tree_step_sum_kernel(StepArgs a, RingArgs ring) {
  constexpr int PP = kRing == TSG_RING_MODP ? TSG_MAX_PRIMES : 1;
  constexpr int leaves = (kLLeaf ? 1 : 0) + (kRLeaf ? 1 : 0);
  __shared__ uint64_t red[PP][kThreads];
  const uint64_t nk = 1ull << a.k_bits;
  for (uint64_t t = blockIdx.x; t < a.total; t += gridDim.x) {
    const uint64_t lo = a.l_base + scatter_bits(a.lt, t);
    const uint64_t ro = a.r_base + scatter_bits(a.rt, t);
    uint64_t part[PP];
#pragma unroll
    for (int p = 0; p < PP; ++p) part[p] = 0;
    for (uint64_t kk = threadIdx.x; kk < nk; kk += blockDim.x) {
      const uint64_t lko = lo + scatter_bits(a.lk, kk);
      const uint64_t rko = ro + scatter_bits(a.rk, kk);
      if constexpr (kRing == TSG_RING_OR_AND) {
        part[0] |= (uint64_t)(a.lhs[lko] & a.rhs[rko]);
      } else if constexpr (kRing == TSG_RING_U64) {
        part[0] += load_elem<kLLeaf, uint64_t>(a.lhs, lko) * load_elem<kRLeaf, uint64_t>(a.rhs, rko);
      } else {
#pragma unroll
        for (int p = 0; p < PP; ++p) {
          if (p < ring.np) {
            const uint64_t l = load_elem<kLLeaf, uint32_t>(a.lhs, lko + (kLLeaf ? 0 : p * a.l_plane));
            const uint64_t r = load_elem<kRLeaf, uint32_t>(a.rhs, rko + (kRLeaf ? 0 : p * a.r_plane));
            const uint64_t prod = l * r;
            part[p] += leaves == 0 ? (uint64_t)mont_redc(prod, ring.p[p], ring.pinv[p]) : prod;
            if (part[p] >> 62) part[p] = barrett_reduce(part[p], ring.p[p], ring.m[p]);
          }
        }
      }
    }
#pragma unroll
    for (int p = 0; p < PP; ++p) {
      if constexpr (kRing == TSG_RING_MODP) {
        if (p < ring.np) part[p] = barrett_reduce(part[p], ring.p[p], ring.m[p]);
      }
      red[p][threadIdx.x] = part[p];
    }
    __syncthreads();
    for (int half = blockDim.x / 2; half > 0; half >>= 1) {
      if ((int)threadIdx.x < half) {
#pragma unroll
        for (int p = 0; p < PP; ++p) {
          if constexpr (kRing == TSG_RING_OR_AND) red[p][threadIdx.x] |= red[p][threadIdx.x + half];
          else red[p][threadIdx.x] += red[p][threadIdx.x + half];  // MODP: 256 terms < 2^31
        }
      }
      __syncthreads();
    }
    if (threadIdx.x == 0) {
      if constexpr (kRing == TSG_RING_OR_AND) {
        a.out[t] = red[0][0] ? 1 : 0;
      } else if constexpr (kRing == TSG_RING_U64) {
        reinterpret_cast<uint64_t*>(a.out)[t] = red[0][0];
      } else {
        uint32_t* out = reinterpret_cast<uint32_t*>(a.out);
#pragma unroll
        for (int p = 0; p < PP; ++p) {
          if (p < ring.np) {
            uint64_t v = barrett_reduce(red[p][0], ring.p[p], ring.m[p]);
            if (leaves == 2) v = barrett_reduce(v * ring.r1[p], ring.p[p], ring.m[p]);
            out[t + p * a.o_plane] = (uint32_t)v;
          }
        }
      }
    }
    __syncthreads();
  }
}

// ------------------------------------------------------------------------------------
// Tile kernel: the common case where a slice's tensors have < 2^32 entries and at most
// 4 wires are summed. Output bits split into three groups:
//   E  up to 2 "enumerated" bits, looped over inside a thread: the output bits the larger
//      operand does not carry, so that operand is read once and reused for every E value;
//   F  the remaining output bits; the low `tile_bits` of them index threads (V consecutive
//      positions per thread), the rest index blocks (blockIdx.x);
//   g  the slice slot (blockIdx.y).
// Every operand offset is base + scatter(g) + scatter(F high) [uniform per block] +
// scatter(F low) [once per thread] + tables for the V positions, E values and summed
// combinations, so the per-output index work is a few table adds.

constexpr int kMaxNarrowRuns = 32;
constexpr int kModeGather = 0;
constexpr int kModeContig = 1;
constexpr int kModeBcast = 2;
constexpr int kModePair = 3;  // two distinct offsets: 0 and tab[3]; pair_sel picks per position
// OR-AND, 16 byte positions of which the operand carries c <= 3 of the 4 index bits: the
// 2^c distinct bytes (offsets dtab) are packed into two words and spread over the four
// output words with byte permutes (selectors psel)
constexpr int kModePerm = 4;
// V = 4, count rings: positions at offsets {0, 1, d, d + 1} (two adjacent pairs), read as
// two 2-element vector loads
constexpr int kModeDual = 5;
// OR-AND, V = 16: the operand carries all four fastest positions, two of them as its own
// bits 0 and 1 (one aligned 4-byte word) and two elsewhere; four word loads at dtab[0..3]
// and, per output word i, one __byte_perm of words qsrc[i] & 3 and qsrc[i] >> 2 with
// selector psel[i]
constexpr int kModeQuad = 6;
constexpr int kMaxE = 4;   // enumerated output combinations per thread (|E| <= 2)
constexpr int kMaxK = 64;  // summed combinations kept in tables (k <= 6)

struct NarrowMap {
  int32_t n;
  uint8_t src[kMaxNarrowRuns];
  uint8_t len[kMaxNarrowRuns];
  uint8_t dst[kMaxNarrowRuns];
};

struct TileOperand {
  const uint8_t* ptr;
  uint64_t base;          // constant element offset
  uint64_t plane;         // residue-plane stride (elements); 0 for leaves
  NarrowMap f_lo, f_hi;   // F bits below / at or above tile_bits -> operand bits
  BitMap g;               // slice-slot bits -> operand bits
  uint32_t tab[16];       // offsets of the V consecutive F positions
  uint32_t e_off[kMaxE];  // offsets of the E combinations
  uint32_t k_off[kMaxK];  // offsets of the summed combinations
  int32_t mode;           // kModeContig / kModeBcast / kModePair / kModeGather / kModePerm
  int32_t pair_sel;       // kModePair: bit j set when position j reads offset tab[3]
  int32_t has_e;          // carries E bits (reloaded per E combination)
  int32_t leaf;           // uint8 leaf (widened on load)
  int32_t pn;             // kModePerm: distinct values (2, 4 or 8)
  uint32_t dtab[8];       // kModePerm: their offsets
  uint32_t psel[4];       // kModePerm / kModeQuad: __byte_perm selector of each output word
  uint32_t qsrc[4];       // kModeQuad: source words of each output word (2 bits each)
};

struct TileArgs {
  TileOperand op[2];
  uint8_t* out;
  uint64_t o_plane;
  uint32_t n_out;          // outputs per slice
  NarrowMap of_lo, of_hi;  // F bits -> output bit positions
  uint32_t o_tab[16];
  uint32_t o_e[kMaxE];
  int32_t tile_bits;
  int32_t n_k;             // summed combinations (2^k)
  int32_t o_contig;        // the V positions are consecutive outputs
  int32_t plane_split;     // MODP: one residue plane per block (blockIdx.z), not all per thread
};

__device__ __forceinline__ uint32_t scatter32(const NarrowMap& m, uint32_t x) {
  uint32_t r = 0;
#pragma unroll 1
  for (int i = 0; i < m.n; ++i) r |= ((x >> m.src[i]) & ((1u << m.len[i]) - 1u)) << m.dst[i];
  return r;
}

// Loads the V values of one operand (residue plane already folded into `off`).
template <typename T, typename VT, int V>
__device__ __forceinline__ void tile_load(const TileOperand& op, uint64_t off, VT (&out)[V]) {
  const uint8_t* base = op.ptr;
  if (op.leaf) {
    if (V == 16 && op.mode == kModeContig) {
      const uint4 w = *reinterpret_cast<const uint4*>(base + off);
      const uint32_t ws[4] = {w.x, w.y, w.z, w.w};
#pragma unroll
      for (int j = 0; j < V; ++j) out[j] = (VT)((ws[j / 4] >> (8 * (j % 4))) & 0xff);
    } else if (V == 4 && op.mode == kModeContig) {
      const uint32_t w = *reinterpret_cast<const uint32_t*>(base + off);
#pragma unroll
      for (int j = 0; j < V; ++j) out[j] = (VT)((w >> (8 * j)) & 0xff);
    } else if (op.mode == kModeBcast) {
      const VT x = (VT)base[off];
#pragma unroll
      for (int j = 0; j < V; ++j) out[j] = x;
    } else if (V == 4 && op.mode == kModePair) {
      const VT x0 = (VT)base[off], x1 = (VT)base[off + op.tab[3]];
#pragma unroll
      for (int j = 0; j < V; ++j) out[j] = ((op.pair_sel >> j) & 1) ? x1 : x0;
    } else {
#pragma unroll
      for (int j = 0; j < V; ++j) out[j] = (VT)base[off + op.tab[j]];
    }
    return;
  }
  const T* p = reinterpret_cast<const T*>(base);
  if (V == 16 && op.mode == kModeContig) {
    if constexpr (sizeof(T) == 1) {
      const uint4 w = *reinterpret_cast<const uint4*>(p + off);
      const uint32_t ws[4] = {w.x, w.y, w.z, w.w};
#pragma unroll
      for (int j = 0; j < V; ++j) out[j] = (VT)((ws[j / 4] >> (8 * (j % 4))) & 0xff);
    }
  } else if (V == 4 && op.mode == kModeContig) {
    if constexpr (sizeof(T) == 1) {
      const uint32_t w = *reinterpret_cast<const uint32_t*>(p + off);
#pragma unroll
      for (int j = 0; j < V; ++j) out[j] = (VT)((w >> (8 * j)) & 0xff);
    } else if constexpr (sizeof(T) == 4) {
      const uint4 w = *reinterpret_cast<const uint4*>(p + off);
      out[0] = w.x;
      out[1 % V] = w.y;
      out[2 % V] = w.z;
      out[3 % V] = w.w;
    } else {
      const ulonglong2* q = reinterpret_cast<const ulonglong2*>(p + off);
      const ulonglong2 w0 = q[0], w1 = q[1];
      out[0] = w0.x;
      out[1 % V] = w0.y;
      out[2 % V] = w1.x;
      out[3 % V] = w1.y;
    }
  } else if (op.mode == kModeBcast) {
    const VT x = (VT)p[off];
#pragma unroll
    for (int j = 0; j < V; ++j) out[j] = x;
  } else if (V == 4 && sizeof(T) >= 4 && op.mode == kModeDual) {
    if constexpr (sizeof(T) == 4) {
      const uint2 x0 = *reinterpret_cast<const uint2*>(p + off);
      const uint2 x1 = *reinterpret_cast<const uint2*>(p + off + op.tab[2]);
      out[0] = x0.x;
      out[1 % V] = x0.y;
      out[2 % V] = x1.x;
      out[3 % V] = x1.y;
    } else if constexpr (sizeof(T) == 8) {
      const ulonglong2 x0 = *reinterpret_cast<const ulonglong2*>(p + off);
      const ulonglong2 x1 = *reinterpret_cast<const ulonglong2*>(p + off + op.tab[2]);
      out[0] = x0.x;
      out[1 % V] = x0.y;
      out[2 % V] = x1.x;
      out[3 % V] = x1.y;
    }
  } else if (V == 4 && op.mode == kModePair) {
    const VT x0 = (VT)p[off], x1 = (VT)p[off + op.tab[3]];
#pragma unroll
    for (int j = 0; j < V; ++j) out[j] = ((op.pair_sel >> j) & 1) ? x1 : x0;
  } else {
#pragma unroll
    for (int j = 0; j < V; ++j) out[j] = (VT)p[off + op.tab[j]];
  }
}

// OR-AND values are 0/1 bytes, so four positions packed in a 32-bit word combine with
// word-wide AND / OR. Loads `V` positions (V = 4 or 16) as V/4 packed words.
template <int V>
__device__ __forceinline__ void tile_load_packed(const TileOperand& op, uint64_t off,
                                                 uint32_t (&w)[V / 4]) {
  const uint8_t* base = op.ptr;
  if (op.mode == kModeContig) {
    if constexpr (V == 16) {
      const uint4 x = *reinterpret_cast<const uint4*>(base + off);
      w[0] = x.x;
      w[1 % (V / 4)] = x.y;
      w[2 % (V / 4)] = x.z;
      w[3 % (V / 4)] = x.w;
    } else {
      w[0] = *reinterpret_cast<const uint32_t*>(base + off);
    }
  } else if (op.mode == kModeBcast) {
    const uint32_t x = (uint32_t)base[off] * 0x01010101u;
#pragma unroll
    for (int i = 0; i < V / 4; ++i) w[i] = x;
  } else if (V == 4 && op.mode == kModeDual) {
    // positions {0, 1, d, d + 1}: two 2-byte loads (even offsets, proven on the host)
    const uint32_t lo = *reinterpret_cast<const uint16_t*>(base + off);
    const uint32_t hi = *reinterpret_cast<const uint16_t*>(base + off + op.tab[2]);
    w[0] = lo | (hi << 16);
  } else if (V == 4 && op.mode == kModePair) {
    const uint32_t x0 = base[off], x1 = base[off + op.tab[3]];
    uint32_t r = 0;
#pragma unroll
    for (int j = 0; j < 4; ++j) r |= (((op.pair_sel >> j) & 1) ? x1 : x0) << (8 * j);
    w[0] = r;
  } else if (V == 16 && op.mode == kModeQuad) {
    // four aligned words (alignment proven on the host); selects, not an indexed array
    const uint32_t q0 = *reinterpret_cast<const uint32_t*>(base + off);
    const uint32_t q1 = *reinterpret_cast<const uint32_t*>(base + off + op.dtab[1]);
    const uint32_t q2 = *reinterpret_cast<const uint32_t*>(base + off + op.dtab[2]);
    const uint32_t q3 = *reinterpret_cast<const uint32_t*>(base + off + op.dtab[3]);
    auto pick = [&](uint32_t q) { return q == 0 ? q0 : (q == 1 ? q1 : (q == 2 ? q2 : q3)); };
#pragma unroll
    for (int i = 0; i < V / 4; ++i)
      w[i] = __byte_perm(pick(op.qsrc[i] & 3u), pick((op.qsrc[i] >> 2) & 3u), op.psel[i]);
  } else if (V == 16 && op.mode == kModePerm) {
    uint32_t w0 = 0, w1 = 0;
#pragma unroll
    for (int d = 0; d < 8; ++d) {
      if (d < op.pn) {
        const uint32_t b = base[off + op.dtab[d]];
        if (d < 4) w0 |= b << (8 * d);
        else w1 |= b << (8 * (d - 4));
      }
    }
#pragma unroll
    for (int i = 0; i < V / 4; ++i) w[i] = __byte_perm(w0, w1, op.psel[i]);
  } else {
#pragma unroll
    for (int i = 0; i < V / 4; ++i) {
      uint32_t r = 0;
#pragma unroll
      for (int j = 0; j < 4; ++j) r |= (uint32_t)base[off + op.tab[4 * i + j]] << (8 * j);
      w[i] = r;
    }
  }
}

// One thread's work in the tile kernel. X is an operand without E bits (loaded once per
// residue plane and reused for every E value), Y the other one; the ring products commute,
// so the kernel passes (lhs, rhs) or (rhs, lhs). With a fixed summed count (NK > 0) the
// thread gathers all of Y's values of a plane before its first store: loads placed after
// a store to a possibly aliasing address would each wait out their own latency.
// kNoLeaf: neither operand is a leaf (the common large step), so every product is a
// product of two Montgomery residues and the arithmetic needs no per-thread leaf checks.
template <int kRing, int V, int NE, int NK, bool kNoLeaf = false>
__device__ __forceinline__ void tile_thread(const TileArgs& a, const RingArgs& ring,
                                            const TileOperand& X, const TileOperand& Y,
                                            uint64_t x0, uint64_t y0, uint64_t oo,
                                            int p_lo, int p_hi) {
  using T = typename std::conditional<kRing == TSG_RING_OR_AND, uint8_t,
            typename std::conditional<kRing == TSG_RING_U64, uint64_t, uint32_t>::type>::type;
  using VT = typename std::conditional<kRing == TSG_RING_U64, uint64_t, uint32_t>::type;
  using AT = uint64_t;
  constexpr bool kPacked = (kRing == TSG_RING_OR_AND) && (V % 4 == 0);
  constexpr int W = kPacked ? V / 4 : 1;  // packed words per operand (OR-AND)
  constexpr int KU = NK > 0 ? NK : 1;
  const int nk = NK > 0 ? NK : a.n_k;
  if constexpr (kPacked) {
    constexpr bool kHoist = NK > 0 && NE * KU * W <= 16;  // more spills registers
    uint32_t xw[KU][W];
    uint32_t yh[kHoist ? NE : 1][KU][W];
    if (NK > 0) {
#pragma unroll
      for (int ku = 0; ku < KU; ++ku) tile_load_packed<V>(X, x0 + X.k_off[ku], xw[ku]);
    }
    if constexpr (kHoist) {
#pragma unroll
      for (int e = 0; e < NE; ++e)
#pragma unroll
        for (int ku = 0; ku < KU; ++ku)
          tile_load_packed<V>(Y, y0 + Y.e_off[e] + Y.k_off[ku], yh[e][ku]);
    }
#pragma unroll
    for (int e = 0; e < NE; ++e) {
      uint32_t acc[W];
#pragma unroll
      for (int i = 0; i < W; ++i) acc[i] = 0;
      for (int kk0 = 0; kk0 < nk; kk0 += KU) {
#pragma unroll
        for (int ku = 0; ku < KU; ++ku) {
          const int kk = kk0 + ku;
          uint32_t xv[W], yv[W];
          if (NK > 0) {
#pragma unroll
            for (int i = 0; i < W; ++i) xv[i] = xw[ku][i];
          } else {
            tile_load_packed<V>(X, x0 + X.k_off[kk], xv);
          }
          if constexpr (kHoist) {
#pragma unroll
            for (int i = 0; i < W; ++i) yv[i] = yh[e][ku][i];
          } else {
            tile_load_packed<V>(Y, y0 + Y.e_off[e] + Y.k_off[kk], yv);
          }
#pragma unroll
          for (int i = 0; i < W; ++i) acc[i] |= xv[i] & yv[i];
        }
      }
      const uint64_t oe = oo + a.o_e[e];
      if (a.o_contig) {
        if constexpr (V == 16) {
          *reinterpret_cast<uint4*>(a.out + oe) =
              make_uint4(acc[0], acc[1 % W], acc[2 % W], acc[3 % W]);
        } else {
          *reinterpret_cast<uint32_t*>(a.out + oe) = acc[0];
        }
      } else {
#pragma unroll
        for (int j = 0; j < V; ++j) a.out[oe + a.o_tab[j]] = (acc[j / 4] >> (8 * (j % 4))) & 0xff;
      }
    }
  } else {
    // planes [p_lo, p_hi) outermost; X of plane p+1 is loaded while plane p is combined
    constexpr int PP = (kRing == TSG_RING_MODP) ? TSG_MAX_PRIMES : 1;
    constexpr bool kHoist = NK > 0 && NE * KU * V * sizeof(VT) <= 64;  // more spills registers
    const int np = p_hi;
    const int leaves = kNoLeaf ? 0 : X.leaf + Y.leaf;
    // partial sums are reduced pairwise only with more than two summed combinations
    constexpr bool kPairs = NK == 0 || NK > 2;
    VT xcur[KU][V], xnxt[KU][V];
    auto preload = [&](int p, VT (&xb)[KU][V]) {
      const uint64_t xp = x0 + (X.leaf ? 0 : p * X.plane);
#pragma unroll
      for (int ku = 0; ku < KU; ++ku) tile_load<T, VT, V>(X, xp + X.k_off[ku], xb[ku]);
    };
    if (NK > 0) preload(p_lo, xcur);
#pragma unroll
    for (int q = 0; q < PP; ++q) {
      const int p = p_lo + q;
      if (p >= np) break;
      const PlaneConst pc = plane_const(ring, p);
      if (NK > 0 && p + 1 < np) preload(p + 1, xnxt);
      const uint64_t xp = x0 + (X.leaf ? 0 : p * X.plane);
      const uint64_t yp = y0 + (Y.leaf ? 0 : p * Y.plane);
      VT yh[kHoist ? NE : 1][KU][V];
      if constexpr (kHoist) {
#pragma unroll
        for (int e = 0; e < NE; ++e)
#pragma unroll
          for (int ku = 0; ku < KU; ++ku)
            tile_load<T, VT, V>(Y, yp + Y.e_off[e] + Y.k_off[ku], yh[e][ku]);
      }
      // above the hoisting budget: double buffer over E (the next combination's values
      // are loaded before this one's stores)
      constexpr bool kDouble = !kHoist && NK > 0 && NE > 1;
      VT ycur[kDouble ? KU : 1][V], ynxt[kDouble ? KU : 1][V];
      if constexpr (kDouble) {
#pragma unroll
        for (int ku = 0; ku < KU; ++ku)
          tile_load<T, VT, V>(Y, yp + Y.e_off[0] + Y.k_off[ku], ycur[ku]);
      }
#pragma unroll
      for (int e = 0; e < NE; ++e) {
        if constexpr (kDouble) {
          if (e + 1 < NE) {
#pragma unroll
            for (int ku = 0; ku < KU; ++ku)
              tile_load<T, VT, V>(Y, yp + Y.e_off[e + 1] + Y.k_off[ku], ynxt[ku]);
          }
        }
        const uint64_t oe = oo + a.o_e[e];
        AT acc[V];
        uint32_t done[V];  // MODP: reduced chunks (Montgomery form) when more than 2 sums
#pragma unroll
        for (int j = 0; j < V; ++j) {
          acc[j] = 0;
          done[j] = 0;
        }
        for (int kk0 = 0; kk0 < nk; kk0 += KU) {
#pragma unroll
          for (int ku = 0; ku < KU; ++ku) {
            const int kk = kk0 + ku;
            VT xv[V], yv[V];
            if (NK > 0) {
#pragma unroll
              for (int j = 0; j < V; ++j) xv[j] = xcur[ku][j];
            } else {
              tile_load<T, VT, V>(X, xp + X.k_off[kk], xv);
            }
            if constexpr (kHoist) {
#pragma unroll
              for (int j = 0; j < V; ++j) yv[j] = yh[e][ku][j];
            } else if constexpr (kDouble) {
#pragma unroll
              for (int j = 0; j < V; ++j) yv[j] = ycur[ku][j];
            } else {
              tile_load<T, VT, V>(Y, yp + Y.e_off[e] + Y.k_off[kk], yv);
            }
#pragma unroll
            for (int j = 0; j < V; ++j) {
              if constexpr (kRing == TSG_RING_OR_AND) {
                acc[j] |= xv[j] & yv[j];
              } else {
                acc[j] += (AT)xv[j] * (AT)yv[j];
              }
            }
            if constexpr (kRing == TSG_RING_MODP && kPairs) {
              // two Montgomery products stay below p 2^32: reduce every pair of sums; sums
              // with a leaf factor are reduced every 16 terms (small_mod's range)
              if (leaves == 0 ? ((kk & 1) && kk + 1 < nk) : ((kk & 15) == 15 && kk + 1 < nk)) {
#pragma unroll
                for (int j = 0; j < V; ++j) {
                  done[j] = add_mod(done[j], mont_finish_c(acc[j], leaves, pc), pc.p);
                  acc[j] = 0;
                }
              }
            }
          }
        }
        if constexpr (kRing == TSG_RING_OR_AND) {
#pragma unroll
          for (int j = 0; j < V; ++j) a.out[oe + a.o_tab[j]] = acc[j] ? 1 : 0;
        } else if constexpr (kRing == TSG_RING_U64) {
          uint64_t* out = reinterpret_cast<uint64_t*>(a.out);
          if (V == 4 && a.o_contig) {
            reinterpret_cast<ulonglong2*>(out + oe)[0] = make_ulonglong2(acc[0], acc[1 % V]);
            reinterpret_cast<ulonglong2*>(out + oe)[1] = make_ulonglong2(acc[2 % V], acc[3 % V]);
          } else {
#pragma unroll
            for (int j = 0; j < V; ++j) out[oe + a.o_tab[j]] = acc[j];
          }
        } else {
          uint32_t* out = reinterpret_cast<uint32_t*>(a.out) + p * a.o_plane;
          uint32_t r[V];
#pragma unroll
          for (int j = 0; j < V; ++j)
            r[j] = kPairs ? add_mod(done[j], mont_finish_c(acc[j], leaves, pc), pc.p)
                          : mont_finish_c(acc[j], leaves, pc);
          if (V == 4 && a.o_contig) {
            *reinterpret_cast<uint4*>(out + oe) = make_uint4(r[0], r[1 % V], r[2 % V], r[3 % V]);
          } else {
#pragma unroll
            for (int j = 0; j < V; ++j) out[oe + a.o_tab[j]] = r[j];
          }
        }
        if constexpr (kDouble) {
#pragma unroll
          for (int ku = 0; ku < KU; ++ku)
#pragma unroll
            for (int j = 0; j < V; ++j) ycur[ku][j] = ynxt[ku][j];
        }
      }
      if (NK > 0) {
#pragma unroll
        for (int ku = 0; ku < KU; ++ku)
#pragma unroll
          for (int j = 0; j < V; ++j) xcur[ku][j] = xnxt[ku][j];
      }
    }
  }
}

template <int kRing, int V, int NE, int NK>
__global__ void __launch_bounds__(kThreads, 4) tree_step_tile_kernel(TileArgs a, RingArgs ring) {
  const uint32_t g = blockIdx.y;
  const uint32_t f_hi = blockIdx.x << a.tile_bits;
  const uint32_t f_lo = threadIdx.x * (uint32_t)V;
  uint64_t xo[2];
#pragma unroll
  for (int o = 0; o < 2; ++o) {
    const TileOperand& op = a.op[o];
    xo[o] = op.base + scatter_bits(op.g, g) + scatter32(op.f_hi, f_hi) + scatter32(op.f_lo, f_lo);
  }
  const uint64_t oo = (uint64_t)g * a.n_out + scatter32(a.of_hi, f_hi) + scatter32(a.of_lo, f_lo);
  const int np = kRing == TSG_RING_MODP ? ring.np : 1;
  const int p_lo = a.plane_split ? (int)blockIdx.z : 0;
  const int p_hi = a.plane_split ? p_lo + 1 : np;
  // at most one operand carries E bits (the other is the one E was chosen against); the
  // count rings take a leaf-free path when neither operand is a leaf
  const bool no_leaf = kRing == TSG_RING_MODP && !a.op[0].leaf && !a.op[1].leaf;
  if (!a.op[0].has_e) {
    if (no_leaf)
      tile_thread<kRing, V, NE, NK, true>(a, ring, a.op[0], a.op[1], xo[0], xo[1], oo, p_lo, p_hi);
    else
      tile_thread<kRing, V, NE, NK>(a, ring, a.op[0], a.op[1], xo[0], xo[1], oo, p_lo, p_hi);
  } else {
    if (no_leaf)
      tile_thread<kRing, V, NE, NK, true>(a, ring, a.op[1], a.op[0], xo[1], xo[0], oo, p_lo, p_hi);
    else
      tile_thread<kRing, V, NE, NK>(a, ring, a.op[1], a.op[0], xo[1], xo[0], oo, p_lo, p_hi);
  }
}

// ------------------------------------------------------------------------------------
// Fused steps. A step P = A x B whose large result is read by exactly one consumer step
// C x P as that step's E-free operand is not launched: the consumer computes each entry
// of P it needs from A and B, and P never exists in HBM. For the consumer's index x and
// summed combination k,
//   P[y(x, k)] = sum over the producer's summed combinations kp of A[a(x, k, kp)] B[b(x, k, kp)]
// where the offset maps a, b compose the consumer's map onto P with the producer's maps
// onto A and B (the host builds them as tile operands in the consumer's index space).
// Every P entry the consumer reads is computed once per (position, summed combination):
// P carries every output bit but the enumerated ones, so no two threads share an entry.
// All rings: residues and counts per position, OR-AND as packed words of 0/1 bytes.

struct FusedArgs {
  TileOperand op[2];      // A and B: producer operands, mapped in the consumer's index
  uint32_t kp_off[2][2];  // per operand, offset of each producer summed combination
  int32_t fx;             // consumer operand that is computed (never read from memory)
};

// The V values of P for summed combination `ku` of plane p (offsets a_p, b_p already
// include the plane): MODP residues in Montgomery form, U64 plain counts.
template <int kRing, int V, int NKP, typename VT>
__device__ __forceinline__ void fused_x(const FusedArgs& f, uint64_t a_p, uint64_t b_p, int ku,
                                        const PlaneConst& pc, VT (&x)[V]) {
  using T = typename std::conditional<kRing == TSG_RING_U64, uint64_t, uint32_t>::type;
  const TileOperand& A = f.op[0];
  const TileOperand& B = f.op[1];
  uint64_t acc[V];
#pragma unroll
  for (int j = 0; j < V; ++j) acc[j] = 0;
#pragma unroll
  for (int kp = 0; kp < NKP; ++kp) {
    VT av[V], bv[V];
    tile_load<T, VT, V>(A, a_p + A.k_off[ku] + f.kp_off[0][kp], av);
    tile_load<T, VT, V>(B, b_p + B.k_off[ku] + f.kp_off[1][kp], bv);
#pragma unroll
    for (int j = 0; j < V; ++j) acc[j] += (uint64_t)av[j] * (uint64_t)bv[j];
  }
  if constexpr (kRing == TSG_RING_MODP) {
    // at most two products: below 2 p^2 < p 2^32 (one reduction), or small with leaves
    const int leaves = A.leaf + B.leaf;
#pragma unroll
    for (int j = 0; j < V; ++j) x[j] = mont_finish_c(acc[j], leaves, pc);
  } else {
#pragma unroll
    for (int j = 0; j < V; ++j) x[j] = acc[j];
  }
}

// One thread of a fused step (count rings, V = 4 positions, NK summed combinations of the
// consumer unrolled): per residue plane, the NK x V values of P are computed from A and
// B, then combined with the other operand Y for every E combination, as in tile_thread.
template <int kRing, int NE, int NK, int NKP>
__device__ __forceinline__ void fused_thread(const TileArgs& a, const FusedArgs& f,
                                             const RingArgs& ring, const TileOperand& Y,
                                             uint64_t a0, uint64_t b0, uint64_t y0,
                                             uint64_t oo) {
  constexpr int V = 4;
  using T = typename std::conditional<kRing == TSG_RING_U64, uint64_t, uint32_t>::type;
  using VT = T;
  constexpr int PP = (kRing == TSG_RING_MODP) ? TSG_MAX_PRIMES : 1;
  constexpr int KU = NK;
  constexpr bool kHoist = NE * KU * V * sizeof(VT) <= 64;
  const int np = (kRing == TSG_RING_MODP) ? ring.np : 1;
  const TileOperand& A = f.op[0];
  const TileOperand& B = f.op[1];
  const int y_leaf = Y.leaf;
#pragma unroll 1
  for (int p = 0; p < PP; ++p) {
    if (p >= np) break;
    const PlaneConst pc = plane_const(ring, p);
    const uint64_t a_p = a0 + (A.leaf ? 0 : p * A.plane);
    const uint64_t b_p = b0 + (B.leaf ? 0 : p * B.plane);
    const uint64_t yp = y0 + (Y.leaf ? 0 : p * Y.plane);
    VT yh[kHoist ? NE : 1][KU][V];
    if constexpr (kHoist) {
#pragma unroll
      for (int e = 0; e < NE; ++e)
#pragma unroll
        for (int ku = 0; ku < KU; ++ku) tile_load<T, VT, V>(Y, yp + Y.e_off[e] + Y.k_off[ku], yh[e][ku]);
    }
    VT x[KU][V];
#pragma unroll
    for (int ku = 0; ku < KU; ++ku) fused_x<kRing, V, NKP>(f, a_p, b_p, ku, pc, x[ku]);
    constexpr bool kDouble = !kHoist && NE > 1;
    VT ycur[kDouble ? KU : 1][V], ynxt[kDouble ? KU : 1][V];
    if constexpr (kDouble) {
#pragma unroll
      for (int ku = 0; ku < KU; ++ku) tile_load<T, VT, V>(Y, yp + Y.e_off[0] + Y.k_off[ku], ycur[ku]);
    }
#pragma unroll
    for (int e = 0; e < NE; ++e) {
      if constexpr (kDouble) {
        if (e + 1 < NE) {
#pragma unroll
          for (int ku = 0; ku < KU; ++ku)
            tile_load<T, VT, V>(Y, yp + Y.e_off[e + 1] + Y.k_off[ku], ynxt[ku]);
        }
      }
      uint64_t acc[V];
      uint32_t done[V];
#pragma unroll
      for (int j = 0; j < V; ++j) {
        acc[j] = 0;
        done[j] = 0;
      }
#pragma unroll
      for (int ku = 0; ku < KU; ++ku) {
        VT yv[V];
        if constexpr (kHoist) {
#pragma unroll
          for (int j = 0; j < V; ++j) yv[j] = yh[e][ku][j];
        } else if constexpr (kDouble) {
#pragma unroll
          for (int j = 0; j < V; ++j) yv[j] = ycur[ku][j];
        } else {
          tile_load<T, VT, V>(Y, yp + Y.e_off[e] + Y.k_off[ku], yv);
        }
#pragma unroll
        for (int j = 0; j < V; ++j) acc[j] += (uint64_t)x[ku][j] * (uint64_t)yv[j];
        if constexpr (kRing == TSG_RING_MODP) {
          // two Montgomery products stay below p 2^32: reduce every pair of sums
          if (y_leaf == 0 && (ku & 1) && ku + 1 < KU) {
#pragma unroll
            for (int j = 0; j < V; ++j) {
              done[j] = add_mod(done[j], mont_redc(acc[j], pc.p, pc.pinv), pc.p);
              acc[j] = 0;
            }
          }
        }
      }
      const uint64_t oe = oo + a.o_e[e];
      if constexpr (kRing == TSG_RING_U64) {
        uint64_t* out = reinterpret_cast<uint64_t*>(a.out);
        if (a.o_contig) {
          reinterpret_cast<ulonglong2*>(out + oe)[0] = make_ulonglong2(acc[0], acc[1]);
          reinterpret_cast<ulonglong2*>(out + oe)[1] = make_ulonglong2(acc[2], acc[3]);
        } else {
#pragma unroll
          for (int j = 0; j < V; ++j) out[oe + a.o_tab[j]] = acc[j];
        }
      } else {
        // X is a residue, so the products have at most one leaf factor (Y)
        uint32_t* out = reinterpret_cast<uint32_t*>(a.out) + p * a.o_plane;
        uint32_t r[V];
#pragma unroll
        for (int j = 0; j < V; ++j) r[j] = add_mod(done[j], mont_finish_c(acc[j], y_leaf, pc), pc.p);
        if (a.o_contig) {
          *reinterpret_cast<uint4*>(out + oe) = make_uint4(r[0], r[1], r[2], r[3]);
        } else {
#pragma unroll
          for (int j = 0; j < V; ++j) out[oe + a.o_tab[j]] = r[j];
        }
      }
      if constexpr (kDouble) {
#pragma unroll
        for (int ku = 0; ku < KU; ++ku)
#pragma unroll
          for (int j = 0; j < V; ++j) ycur[ku][j] = ynxt[ku][j];
      }
    }
  }
}

// One thread of a fused OR-AND step: the four positions of each operand travel as one
// packed word of 0/1 bytes, so P's word for summed combination ku is the OR over the
// producer's summed combinations of (A word AND B word).
template <int NE, int NK, int NKP>
__device__ __forceinline__ void fused_thread_or_and(const TileArgs& a, const FusedArgs& f,
                                                    const TileOperand& Y, uint64_t a0,
                                                    uint64_t b0, uint64_t y0, uint64_t oo) {
  constexpr int KU = NK;
  const TileOperand& A = f.op[0];
  const TileOperand& B = f.op[1];
  uint32_t x[KU];
#pragma unroll
  for (int ku = 0; ku < KU; ++ku) {
    uint32_t w = 0;
#pragma unroll
    for (int kp = 0; kp < NKP; ++kp) {
      uint32_t aw[1], bw[1];
      tile_load_packed<4>(A, a0 + A.k_off[ku] + f.kp_off[0][kp], aw);
      tile_load_packed<4>(B, b0 + B.k_off[ku] + f.kp_off[1][kp], bw);
      w |= aw[0] & bw[0];
    }
    x[ku] = w;
  }
  uint32_t yh[NE][KU];
#pragma unroll
  for (int e = 0; e < NE; ++e)
#pragma unroll
    for (int ku = 0; ku < KU; ++ku) {
      uint32_t yw[1];
      tile_load_packed<4>(Y, y0 + Y.e_off[e] + Y.k_off[ku], yw);
      yh[e][ku] = yw[0];
    }
#pragma unroll
  for (int e = 0; e < NE; ++e) {
    uint32_t acc = 0;
#pragma unroll
    for (int ku = 0; ku < KU; ++ku) acc |= x[ku] & yh[e][ku];
    const uint64_t oe = oo + a.o_e[e];
    if (a.o_contig) {
      *reinterpret_cast<uint32_t*>(a.out + oe) = acc;
    } else {
#pragma unroll
      for (int j = 0; j < 4; ++j) a.out[oe + a.o_tab[j]] = (acc >> (8 * j)) & 0xff;
    }
  }
}

template <int kRing, int NE, int NK, int NKP>
__global__ void __launch_bounds__(kThreads, 2)
    tree_step_fused_kernel(TileArgs a, FusedArgs f, RingArgs ring) {
  const uint32_t g = blockIdx.y;
  const uint32_t f_hi = blockIdx.x << a.tile_bits;
  const uint32_t f_lo = threadIdx.x * 4u;
  auto offset = [&](const TileOperand& op) -> uint64_t {
    return op.base + scatter_bits(op.g, g) + scatter32(op.f_hi, f_hi) + scatter32(op.f_lo, f_lo);
  };
  const TileOperand& Y = a.op[1 - f.fx];
  const uint64_t oo = (uint64_t)g * a.n_out + scatter32(a.of_hi, f_hi) + scatter32(a.of_lo, f_lo);
  if constexpr (kRing == TSG_RING_OR_AND) {
    fused_thread_or_and<NE, NK, NKP>(a, f, Y, offset(f.op[0]), offset(f.op[1]), offset(Y), oo);
  } else {
    fused_thread<kRing, NE, NK, NKP>(a, f, ring, Y, offset(f.op[0]), offset(f.op[1]),
                                     offset(Y), oo);
  }
}

// ------------------------------------------------------------------------------------
// Streaming kernel for the large steps (the bulk of the HBM traffic). Persistent blocks
// walk the (tile, slice) work items with a warp-specialised pipeline:
//   * an item is one residue plane of one 1024-element tile of one slice;
//   * a producer warp stages items into a ring of `stages` shared-memory stages with TMA
//     bulk copies (cp.async.bulk ... mbarrier::complete_tx): the E-free operand's tile
//     for every summed combination and, where its offsets allow (s_span > 0), the other
//     operand's aligned blocks for the tile, plus the item's offsets in a stage header;
//   * 8 consumer warps (4 positions per thread) combine an item from its stage, write the
//     result from registers as 16-byte vectors, and release the stage (one arrival per
//     warp on the stage's `empty` barrier); nothing else synchronises the block.
// Every mbarrier wait is bounded (StreamArgs::wait_ns): on expiry the thread records an
// error in the executor's error record (StreamArgs::error) and sets the block's bail flag;
// the producer then waits (bounded by kDrainLimitNs) for the copies it has in flight and
// every thread returns.

constexpr int kStreamTileBits = 10;                      // 256 consumer threads x 4
constexpr int kStreamTile = 1 << kStreamTileBits;
constexpr int kStreamConsumers = 256;
constexpr int kStreamThreads = kStreamConsumers + 32;    // + the producer warp
constexpr int kStreamMaxStages = 8;
constexpr uint64_t kWaitLimitNs = 2000000000ull;         // default limit of one bounded wait: 2 s
// Limit of the producer's final wait for its own copies in flight: never shorter than the
// default, so that a block never exits while a bulk copy still writes its shared memory.
constexpr uint64_t kDrainLimitNs = kWaitLimitNs;
constexpr uint32_t kSuspendHintNs = 20000;               // longest suspension per try_wait


__device__ __forceinline__ uint32_t smem_addr(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count)
               : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)),
               "r"(bytes)
               : "memory");
}

__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_addr(bar)) : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n.reg .pred p;\n"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
      "selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(smem_addr(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

// try_wait that may suspend the thread in hardware for up to kSuspendHintNs while the
// phase is incomplete, instead of returning at once (no issue slots spent polling).
__device__ __forceinline__ bool mbar_try_wait_suspend(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n.reg .pred p;\n"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n"
      "selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(smem_addr(bar)), "r"(parity), "r"(kSuspendHintNs)
      : "memory");
  return ok != 0;
}

__device__ __forceinline__ uint64_t global_ns() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// Bounded wait for phase `parity` of `bar`: false when `limit_ns` of wall-clock time (the
// global nanosecond timer) passed without the phase completing.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, uint32_t parity,
                                                  uint64_t limit_ns) {
  if (mbar_try_wait_suspend(bar, parity)) return true;
  const uint64_t t0 = global_ns();
  for (;;) {
    if (mbar_try_wait_suspend(bar, parity)) return true;
    if (global_ns() - t0 > limit_ns) return false;
  }
}

// Warp-uniform bounded wait (every lane of the warp calls it): lane 0 polls, the outcome
// is broadcast, and on success every lane observes the completed phase itself (acquire).
__device__ __forceinline__ bool mbar_wait_warp(uint64_t* bar, uint32_t parity,
                                               uint64_t limit_ns) {
  int ok = 0;
  if ((threadIdx.x & 31) == 0) ok = mbar_wait_bounded(bar, parity, limit_ns) ? 1 : 0;
  ok = __shfl_sync(0xffffffffu, ok, 0);
  if (ok) (void)mbar_try_wait(bar, parity);
  return ok != 0;
}

__device__ __forceinline__ void tma_load_1d(void* dst, const void* src, uint32_t bytes,
                                            uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::
          "r"(smem_addr(dst)),
      "l"(src), "r"(bytes), "r"(smem_addr(bar))
      : "memory");
}

struct StreamArgs {
  int32_t big;           // operand staged through shared memory (0 = lhs, 1 = rhs)
  uint32_t tiles;        // tiles per slice
  uint64_t work;         // tiles * slices
  uint32_t chunk_bytes;  // one (plane, summed combination) chunk of the staged operand
  uint32_t s_span;       // elements of one staged chunk of the other operand per (plane, E
                         // combination, summed combination); 0: read from global memory
  uint32_t stage_bytes;  // one stage: the item's chunks of both operands
  int32_t stages;        // stages in the ring (2 .. kStreamMaxStages)
  int32_t kchunks;       // stages per item: its summed combinations, 4 (NK) per stage
  int* error;            // set to TSG_ERR_TIMEOUT when a bounded wait gives up
  uint64_t wait_ns;      // limit of every bounded wait of the pipeline (default 2 s)
  int64_t stop_after;    // testing hook: the producer stops after issuing this many stages
                         // (< 0: never), so that the consumers' next wait runs out
};

// Offsets of one staged item, written by the producer next to its stage.
struct StreamItem {
  uint64_t so;  // the other operand's offset for the tile and plane (positions excluded)
  uint64_t oo;  // output offset for the tile and plane (positions excluded)
  int32_t p;    // residue plane
};

// Loads the V values of the other operand from its staged chunk: `p` points at the
// thread's first position, the tile's positions sit at the operand's tab offsets. The
// load mode is a template parameter (the streaming consumer is specialised on it).
constexpr int kModeGlobal = -1;  // the streaming kernel's other operand is not staged

template <int kMode, typename T, int V>
__device__ __forceinline__ void stage_load(const TileOperand& op, const T* p, T (&out)[V]) {
  if constexpr (kMode == kModeContig) {
    if constexpr (sizeof(T) == 4) {
      const uint4 x = *reinterpret_cast<const uint4*>(p);
      out[0] = x.x;
      out[1 % V] = x.y;
      out[2 % V] = x.z;
      out[3 % V] = x.w;
    } else {
      const ulonglong2 x0 = reinterpret_cast<const ulonglong2*>(p)[0];
      const ulonglong2 x1 = reinterpret_cast<const ulonglong2*>(p)[1];
      out[0] = x0.x;
      out[1 % V] = x0.y;
      out[2 % V] = x1.x;
      out[3 % V] = x1.y;
    }
  } else if constexpr (kMode == kModeBcast) {
    const T x = p[0];
#pragma unroll
    for (int j = 0; j < V; ++j) out[j] = x;
  } else if constexpr (kMode == kModePair) {
    const T x0 = p[0], x1 = p[op.tab[3]];
#pragma unroll
    for (int j = 0; j < V; ++j) out[j] = ((op.pair_sel >> j) & 1) ? x1 : x0;
  } else {
#pragma unroll
    for (int j = 0; j < V; ++j) out[j] = p[op.tab[j]];
  }
}

// With NKP > 0 the kernel runs a fused step: the staged operand B is the result of a
// step that is never stored, and the consumer warps compute its values from that step's
// operands (FusedArgs, fused_x) instead of reading a staged tile; only the other operand
// is staged.
template <int kRing, int NE, int NK, int NKP>
__global__ void __launch_bounds__(kStreamThreads, 3)
    tree_step_stream_kernel(TileArgs a, RingArgs ring, StreamArgs sa, FusedArgs f) {
  using T = typename std::conditional<kRing == TSG_RING_U64, uint64_t, uint32_t>::type;
  constexpr int V = 4;
  constexpr int KU = NK;  // NK in {1, 2, 4}: 2^K summed combinations
  extern __shared__ __align__(128) uint8_t smem[];
  __shared__ __align__(8) uint64_t full[kStreamMaxStages], empty[kStreamMaxStages];
  __shared__ StreamItem head[kStreamMaxStages];
  __shared__ volatile int bail;
  const int np = (kRing == TSG_RING_MODP) ? ring.np : 1;
  const TileOperand& B = a.op[sa.big];
  const TileOperand& S = a.op[1 - sa.big];
  const bool s_staged = sa.s_span != 0;
  const uint32_t b_bytes = NKP > 0 ? 0u : (uint32_t)KU * sa.chunk_bytes;
  const uint32_t s_chunk = sa.s_span * (uint32_t)sizeof(T);
  const int nst = sa.stages;
  const uint64_t items = sa.work * (uint64_t)np;  // (tile, slice, residue plane)
  const int lane = threadIdx.x & 31;

  if (threadIdx.x == 0) {
    for (int s = 0; s < nst; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], kStreamConsumers / 32);
    }
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    bail = 0;
  }
  __syncthreads();

  if (threadIdx.x >= kStreamConsumers) {
    // producer warp: lane 0 writes the item's offsets into the stage header and arms the
    // stage's barrier with the byte count (its arrival releases the header), then the
    // lanes issue the bulk copies (KU tiles of B, NE x KU blocks of the other operand)
    const T* bsrc = reinterpret_cast<const T*>(B.ptr);
    const T* ssrc = reinterpret_cast<const T*>(S.ptr);
    const int nb_copies = NKP > 0 ? 0 : KU;  // tiles of B per stage (none when fused)
    const int ncopies = nb_copies + (s_staged ? NE * KU : 0);
    const uint64_t stride = gridDim.x;
    uint64_t i = 0;  // items issued by this block
    bool stop = false;
    for (uint64_t w0 = blockIdx.x; w0 < items && !stop; w0 += 32 * stride) {
      // lane L computes the offsets of the block's item w0 + L * stride
      const uint64_t wl = w0 + (uint64_t)lane * stride;
      uint64_t l_bo = 0, l_so = 0, l_oo = 0;
      int l_p = 0;
      if (wl < items) {
        l_p = (int)(wl % np);
        const uint64_t tw = wl / np;
        const uint32_t g = (uint32_t)(tw / sa.tiles);
        const uint32_t f_hi = (uint32_t)(tw % sa.tiles) << kStreamTileBits;
        l_bo = B.base + scatter_bits(B.g, g) + scatter32(B.f_hi, f_hi) + l_p * B.plane;
        l_so = S.base + scatter_bits(S.g, g) + scatter32(S.f_hi, f_hi) + (S.leaf ? 0 : l_p * S.plane);
        l_oo = (uint64_t)g * a.n_out + scatter32(a.of_hi, f_hi) + l_p * a.o_plane;
      }
      const uint64_t left = (items - w0 + stride - 1) / stride;
      const int nb = (int)(left < 32 ? left : 32);
      for (int k = 0; k < nb && !stop; ++k) {
        const uint64_t bo = __shfl_sync(0xffffffffu, l_bo, k);
        const uint64_t so = __shfl_sync(0xffffffffu, l_so, k);
        const uint64_t oo = __shfl_sync(0xffffffffu, l_oo, k);
        const int p = __shfl_sync(0xffffffffu, l_p, k);
        for (int kc = 0; kc < sa.kchunks; ++kc, ++i) {  // one stage per KU summed combinations
          const int s = (int)(i % nst);
          const uint32_t round = (uint32_t)(i / nst);
          if (__shfl_sync(0xffffffffu, (int)bail, 0) ||
              (sa.stop_after >= 0 && i >= (uint64_t)sa.stop_after)) {
            stop = true;
            break;
          }
          if (round > 0 && !mbar_wait_warp(&empty[s], (round - 1) & 1, sa.wait_ns)) {
            if (lane == 0) {
              atomicExch(sa.error, TSG_ERR_TIMEOUT);
              bail = 1;
            }
            stop = true;
            break;
          }
          uint8_t* dst = smem + (size_t)s * sa.stage_bytes;
          if (lane == 0) {
            head[s].so = so;
            head[s].oo = oo;
            head[s].p = p;
            mbar_expect_tx(&full[s], sa.stage_bytes);
          }
          __syncwarp();
          const int kb = kc * KU;
          for (int c = lane; c < ncopies; c += 32) {
            if (c < nb_copies) {
              tma_load_1d(dst + c * sa.chunk_bytes, bsrc + bo + B.k_off[kb + c], sa.chunk_bytes,
                          &full[s]);
            } else {
              const int j = c - nb_copies;
              const int e = j / KU, ku = j % KU;
              tma_load_1d(dst + b_bytes + j * s_chunk, ssrc + so + S.e_off[e] + S.k_off[kb + ku],
                          s_chunk, &full[s]);
            }
          }
        }
      }
    }
    // the copies of the last (up to) nst items may still be in flight: wait for them
    if (lane == 0) {
      const uint64_t first = i > (uint64_t)nst ? i - nst : 0;
      for (uint64_t j = first; j < i; ++j)
        (void)mbar_wait_bounded(&full[j % nst], (uint32_t)((j / nst) & 1), kDrainLimitNs);
    }
    return;
  }

  // consumer warps: one residue plane of one tile per item; the loop is specialised on how
  // the other operand is read (its staged load mode, or global loads when not staged)
  const uint32_t f_lo = threadIdx.x * V;
  const uint64_t s_lo = scatter32(S.f_lo, f_lo);
  // fused: the thread's position terms of the producer's operands
  const uint64_t fa_lo = NKP > 0 ? scatter32(f.op[0].f_lo, f_lo) : 0;
  const uint64_t fb_lo = NKP > 0 ? scatter32(f.op[1].f_lo, f_lo) : 0;
  const uint64_t o_lo = scatter32(a.of_lo, f_lo);
  // An item whose 2^K > 4 summed combinations span kchunks stages of KU = 4: partial sums
  // stay in registers (MODP: pairs of products reduced and added mod p; with a leaf
  // operand each stage's four small products are reduced at once) until the last stage.
  auto consume_chunked = [&](uint64_t& i, int leaves, auto mode_c) -> bool {
    constexpr int kSMode = decltype(mode_c)::value;
    using Acc = typename std::conditional<kRing == TSG_RING_U64, uint64_t, uint32_t>::type;
    Acc part[NE][V];
#pragma unroll
    for (int e = 0; e < NE; ++e)
#pragma unroll
      for (int j = 0; j < V; ++j) part[e][j] = 0;
    uint64_t so = 0, oo = 0;
    PlaneConst pc{0, 0, 0};
    for (int kc = 0; kc < sa.kchunks; ++kc, ++i) {
      const int s = (int)(i % nst);
      if (__shfl_sync(0xffffffffu, (int)bail, 0)) return false;
      if (!mbar_wait_warp(&full[s], (uint32_t)((i / nst) & 1), sa.wait_ns)) {
        if (lane == 0) {
          atomicExch(sa.error, TSG_ERR_TIMEOUT);
          bail = 1;
        }
        return false;
      }
      if (kc == 0) {
        so = head[s].so;
        oo = head[s].oo + o_lo;
        pc = plane_const(ring, head[s].p);
      }
      const uint8_t* st = smem + (size_t)s * sa.stage_bytes;
      T bv[KU][V];
#pragma unroll
      for (int ku = 0; ku < KU; ++ku) {
        const T* src = reinterpret_cast<const T*>(st + ku * sa.chunk_bytes) + f_lo;
        if constexpr (sizeof(T) == 4) {
          const uint4 x = *reinterpret_cast<const uint4*>(src);
          bv[ku][0] = x.x;
          bv[ku][1] = x.y;
          bv[ku][2] = x.z;
          bv[ku][3] = x.w;
        } else {
          const ulonglong2 x0 = reinterpret_cast<const ulonglong2*>(src)[0];
          const ulonglong2 x1 = reinterpret_cast<const ulonglong2*>(src)[1];
          bv[ku][0] = x0.x;
          bv[ku][1] = x0.y;
          bv[ku][2] = x1.x;
          bv[ku][3] = x1.y;
        }
      }
      const T* ss = reinterpret_cast<const T*>(st + b_bytes) + s_lo;
#pragma unroll
      for (int e = 0; e < NE; ++e) {
        uint64_t acc[V] = {0, 0, 0, 0};
#pragma unroll
        for (int ku = 0; ku < KU; ++ku) {
          T sv[V];
          if constexpr (kSMode == kModeGlobal)
            tile_load<T, T, V>(S, so + s_lo + S.e_off[e] + S.k_off[kc * KU + ku], sv);
          else
            stage_load<kSMode, T, V>(S, ss + (e * KU + ku) * sa.s_span, sv);
#pragma unroll
          for (int j = 0; j < V; ++j) acc[j] += (uint64_t)bv[ku][j] * (uint64_t)sv[j];
          if constexpr (kRing == TSG_RING_MODP) {
            if ((ku & 1) && leaves == 0) {
#pragma unroll
              for (int j = 0; j < V; ++j) {
                part[e][j] = add_mod(part[e][j], mont_redc(acc[j], pc.p, pc.pinv), pc.p);
                acc[j] = 0;
              }
            }
          }
        }
#pragma unroll
        for (int j = 0; j < V; ++j) {
          if constexpr (kRing == TSG_RING_U64) {
            part[e][j] += acc[j];
          } else {
            if (leaves != 0) part[e][j] = add_mod(part[e][j], small_mod(acc[j], pc.p), pc.p);
          }
        }
      }
      __syncwarp();
      if (lane == 0) mbar_arrive(&empty[s]);
    }
#pragma unroll
    for (int e = 0; e < NE; ++e) {
      const uint64_t oe = oo + a.o_e[e];
      if constexpr (kRing == TSG_RING_U64) {
        uint64_t* out = reinterpret_cast<uint64_t*>(a.out) + oe;
        reinterpret_cast<ulonglong2*>(out)[0] = make_ulonglong2(part[e][0], part[e][1]);
        reinterpret_cast<ulonglong2*>(out)[1] = make_ulonglong2(part[e][2], part[e][3]);
      } else {
        *reinterpret_cast<uint4*>(reinterpret_cast<uint32_t*>(a.out) + oe) =
            make_uint4(part[e][0], part[e][1], part[e][2], part[e][3]);
      }
    }
    return true;
  };
  auto consume = [&](auto mode_c) {
    constexpr int kSMode = decltype(mode_c)::value;  // kModeGlobal: not staged
    // staged operands are intermediates, so only a global operand can be a leaf
    const int leaves = kSMode == kModeGlobal ? S.leaf : 0;
    uint64_t i = 0;  // stages consumed
    for (uint64_t w = blockIdx.x; w < items; w += gridDim.x, ++i) {
      if constexpr (KU == 4 && NKP == 0) {
        if (sa.kchunks > 1) {  // the item spans kchunks stages
          if (!consume_chunked(i, leaves, mode_c)) return;
          --i;  // consume_chunked advanced i past the item's stages
          continue;
        }
      }
      const int s = (int)(i % nst);
      if (__shfl_sync(0xffffffffu, (int)bail, 0)) return;
      if (!mbar_wait_warp(&full[s], (uint32_t)((i / nst) & 1), sa.wait_ns)) {
        if (lane == 0) {
          atomicExch(sa.error, TSG_ERR_TIMEOUT);
          bail = 1;
        }
        return;
      }
      const uint64_t so = head[s].so;
      const uint64_t oo = head[s].oo + o_lo;
      const PlaneConst pc = plane_const(ring, head[s].p);
      const uint8_t* st = smem + (size_t)s * sa.stage_bytes;
      T bv[KU][V];
      if constexpr (NKP > 0) {
        // fused: B's values for this item from the producer's operands (same item order
        // as the producer warp: plane fastest, then tile, then slice)
        const int pp = head[s].p;
        const uint64_t tw = w / (uint64_t)np;
        const uint32_t g = (uint32_t)(tw / sa.tiles);
        const uint32_t f_hi = (uint32_t)(tw % sa.tiles) << kStreamTileBits;
        const TileOperand& FA = f.op[0];
        const TileOperand& FB = f.op[1];
        const uint64_t a_p = FA.base + scatter_bits(FA.g, g) + scatter32(FA.f_hi, f_hi) + fa_lo +
                             (FA.leaf ? 0 : pp * FA.plane);
        const uint64_t b_p = FB.base + scatter_bits(FB.g, g) + scatter32(FB.f_hi, f_hi) + fb_lo +
                             (FB.leaf ? 0 : pp * FB.plane);
#pragma unroll
        for (int ku = 0; ku < KU; ++ku) fused_x<kRing, V, NKP>(f, a_p, b_p, ku, pc, bv[ku]);
      } else {
#pragma unroll
        for (int ku = 0; ku < KU; ++ku) {
          const T* src = reinterpret_cast<const T*>(st + ku * sa.chunk_bytes) + f_lo;
          if constexpr (sizeof(T) == 4) {
            const uint4 x = *reinterpret_cast<const uint4*>(src);
            bv[ku][0] = x.x;
            bv[ku][1] = x.y;
            bv[ku][2] = x.z;
            bv[ku][3] = x.w;
          } else {
            const ulonglong2 x0 = reinterpret_cast<const ulonglong2*>(src)[0];
            const ulonglong2 x1 = reinterpret_cast<const ulonglong2*>(src)[1];
            bv[ku][0] = x0.x;
            bv[ku][1] = x0.y;
            bv[ku][2] = x1.x;
            bv[ku][3] = x1.y;
          }
        }
      }
      const T* ss = reinterpret_cast<const T*>(st + b_bytes) + s_lo;
#pragma unroll
      for (int e = 0; e < NE; ++e) {
        uint64_t acc[V] = {0, 0, 0, 0};  // U64: the sum; MODP: the current pair of products
        uint32_t done[V] = {0, 0, 0, 0};  // MODP, 4 summed combinations: first pair, reduced
#pragma unroll
        for (int ku = 0; ku < KU; ++ku) {
          T sv[V];
          if constexpr (kSMode == kModeGlobal)
            tile_load<T, T, V>(S, so + s_lo + S.e_off[e] + S.k_off[ku], sv);
          else
            stage_load<kSMode, T, V>(S, ss + (e * KU + ku) * sa.s_span, sv);
#pragma unroll
          for (int j = 0; j < V; ++j) acc[j] += (uint64_t)bv[ku][j] * (uint64_t)sv[j];
          if constexpr (kRing == TSG_RING_MODP && KU > 2) {
            // two Montgomery products stay below p 2^32: reduce each pair (with a leaf
            // operand the four products are small and are reduced once at the end)
            if (ku == 1 && leaves == 0) {
#pragma unroll
              for (int j = 0; j < V; ++j) {
                done[j] = mont_redc(acc[j], pc.p, pc.pinv);
                acc[j] = 0;
              }
            }
          }
        }
        const uint64_t oe = oo + a.o_e[e];
        if constexpr (kRing == TSG_RING_U64) {
          uint64_t* out = reinterpret_cast<uint64_t*>(a.out) + oe;
          reinterpret_cast<ulonglong2*>(out)[0] = make_ulonglong2(acc[0], acc[1]);
          reinterpret_cast<ulonglong2*>(out)[1] = make_ulonglong2(acc[2], acc[3]);
        } else {
          uint32_t r[V];
#pragma unroll
          for (int j = 0; j < V; ++j) {
            r[j] = kSMode == kModeGlobal ? mont_finish_c(acc[j], leaves, pc)
                                         : mont_redc(acc[j], pc.p, pc.pinv);
            if constexpr (KU > 2) r[j] = add_mod(done[j], r[j], pc.p);
          }
          *reinterpret_cast<uint4*>(reinterpret_cast<uint32_t*>(a.out) + oe) =
              make_uint4(r[0], r[1], r[2], r[3]);
        }
      }
      // release the stage: every lane of the warp is done reading it
      __syncwarp();
      if (lane == 0) mbar_arrive(&empty[s]);
    }
  };
  if (!s_staged) consume(std::integral_constant<int, kModeGlobal>{});
  else if (S.mode == kModeContig) consume(std::integral_constant<int, kModeContig>{});
  else if (S.mode == kModeBcast) consume(std::integral_constant<int, kModeBcast>{});
  else if (S.mode == kModePair) consume(std::integral_constant<int, kModePair>{});
  else consume(std::integral_constant<int, kModeGather>{});
}

// Combines the root tensors of `cnt` slices (layout [plane][cnt][E]) into result[E]
// (OR for OR_AND, sum mod 2^64 for U64, sum mod p per plane for MODP). One block per root
// entry; threads stride over slices, then a shared-memory tree reduction.
template <int kRing>
__global__ void __launch_bounds__(kThreads)
    root_reduce_kernel(const uint8_t* root, uint64_t cnt, uint64_t entries, uint64_t plane,
                       uint8_t* result, int accumulate, RingArgs ring) {
  __shared__ uint64_t red[kThreads];
  const int np = (kRing == TSG_RING_MODP) ? ring.np : 1;
  for (uint64_t e = blockIdx.x; e < entries; e += gridDim.x) {
    for (int p = 0; p < np; ++p) {
      uint64_t part = 0;
      for (uint64_t g = threadIdx.x; g < cnt; g += blockDim.x) {
        const uint64_t idx = p * plane + g * entries + e;
        if constexpr (kRing == TSG_RING_OR_AND) {
          part |= root[idx];
        } else if constexpr (kRing == TSG_RING_U64) {
          part += reinterpret_cast<const uint64_t*>(root)[idx];
        } else {
          // residues < 2^31 summed over at most 2^32 slices per thread stay below 2^63
          part += reinterpret_cast<const uint32_t*>(root)[idx];
        }
      }
      if constexpr (kRing == TSG_RING_MODP) part = barrett_reduce(part, ring.p[p], ring.m[p]);
      red[threadIdx.x] = part;
      __syncthreads();
      for (int s = blockDim.x / 2; s > 0; s >>= 1) {
        if ((int)threadIdx.x < s) {
          if constexpr (kRing == TSG_RING_OR_AND) {
            red[threadIdx.x] |= red[threadIdx.x + s];
          } else {
            red[threadIdx.x] += red[threadIdx.x + s];  // MODP: each term < 2^31, 256 terms
          }
        }
        __syncthreads();
      }
      if (threadIdx.x == 0) {
        uint64_t v = red[0];
        if constexpr (kRing == TSG_RING_OR_AND) {
          if (accumulate) v |= result[e];
          result[e] = v ? 1 : 0;
        } else if constexpr (kRing == TSG_RING_U64) {
          uint64_t* r = reinterpret_cast<uint64_t*>(result);
          r[e] = accumulate ? r[e] + v : v;
        } else {
          // v < 256 p: reduce, then leave Montgomery form (REDC of x < p is x R^-1 mod p)
          uint32_t* r = reinterpret_cast<uint32_t*>(result) + p * entries;
          uint64_t plain = mont_redc(barrett_reduce(v, ring.p[p], ring.m[p]), ring.p[p],
                                     ring.pinv[p]);
          if (accumulate) plain += r[e];
          r[e] = barrett_reduce(plain, ring.p[p], ring.m[p]);
        }
      }
      __syncthreads();
    }
  }
}

// Dynamic shared memory of one streaming block (its ring of stages): three blocks per SM.
constexpr uint64_t kStreamBlockSmem = 72 * 1024;
constexpr int kStreamBlocksPerSm = 3;

struct TileShape {
  int v, ne, nk;      // template parameters (nk 0: runtime summed count)
  unsigned threads;
  uint64_t tiles;
};

struct LaunchArgs {
  StepArgs a;       // general form (also used for the bounds check)
  TileArgs t;       // tile form, valid when `tile`
  TileShape shape;
  StreamArgs stream;
  FusedArgs f;      // fused form, valid when `fused`
  int nkp;          // fused: producer summed combinations (1 or 2)
  bool tile;
  bool streamed;    // run by the streaming (TMA-staged) kernel
  bool fused;       // run by the fused kernel (operand f.fx computed from f.op)
  bool is_leaf[2];
  uint64_t cnt;     // slices of this launch
};

// Per-ring launchers of the tile and streaming kernels (one translation unit each).
tsg_status launch_tile_or_and(const LaunchArgs& la, const RingArgs& ra, cudaStream_t st);
tsg_status launch_tile_modp(const LaunchArgs& la, const RingArgs& ra, cudaStream_t st);
tsg_status launch_tile_modp_ne1(const LaunchArgs& la, const RingArgs& ra, cudaStream_t st);
tsg_status launch_tile_modp_ne2(const LaunchArgs& la, const RingArgs& ra, cudaStream_t st);
tsg_status launch_tile_modp_ne4(const LaunchArgs& la, const RingArgs& ra, cudaStream_t st);
tsg_status launch_tile_u64(const LaunchArgs& la, const RingArgs& ra, cudaStream_t st);
tsg_status launch_stream_modp(const LaunchArgs& la, const RingArgs& ra, cudaStream_t st);
tsg_status launch_stream_u64(const LaunchArgs& la, const RingArgs& ra, cudaStream_t st);
tsg_status launch_fused_modp(const LaunchArgs& la, const RingArgs& ra, cudaStream_t st);
tsg_status launch_fused_u64(const LaunchArgs& la, const RingArgs& ra, cudaStream_t st);
tsg_status launch_fused_or_and(const LaunchArgs& la, const RingArgs& ra, cudaStream_t st);
tsg_status launch_stream_fused_modp(const LaunchArgs& la, const RingArgs& ra, cudaStream_t st);
tsg_status launch_stream_fused_u64(const LaunchArgs& la, const RingArgs& ra, cudaStream_t st);

// ------------------------------------------------------------------------------------
// Packed steps (tsg_batch_run_packed): the small steps of one tree level, of several
// instances at once, in one launch. A small step has at most 2^kPackTBits output entries
// (slots included) and 2^kPackKBits summed combinations; it is described by per-bit index
// maps instead of runs, and the whole launch's steps travel in the kernel parameters, so a
// packed launch needs no device-side table and records into a graph like any launch.
// One warp computes 32 consecutive entries of one step.

constexpr int kPackTBits = 16;
constexpr int kPackKBits = 5;
constexpr int kPackItems = 240;  // steps per launch (the parameters stay under 32 KB)
constexpr uint8_t kPackNone = 0xff;

struct PackOperand {
  const uint8_t* ptr;
  uint64_t base;   // constant element offset
  uint64_t plane;  // residue-plane stride (elements); unused for leaves
  uint8_t tdst[kPackTBits];  // operand bit of output-index bit b, kPackNone if absent
  uint8_t kdst[8];           // operand bit of summed bit b (first kPackKBits used)
};

struct PackItem {
  PackOperand op[2];
  uint8_t* out;
  uint64_t o_plane;  // residue-plane stride of the output (elements)
  uint32_t warp0;    // first warp of this step in the launch
  uint8_t t_bits;    // log2(output entries)
  uint8_t k_bits;
  uint8_t leaves;    // bit 0: lhs is a leaf (uint8 0/1), bit 1: rhs
  uint8_t pad;
};

struct PackArgs {
  int32_t n_items;
  uint32_t n_warps;
  PackItem items[kPackItems];
};
static_assert(sizeof(PackArgs) + sizeof(RingArgs) < 32000, "packed launch parameters over 32 KB");

__device__ __forceinline__ uint64_t pack_offset(const uint8_t* dst, int bits, uint64_t x) {
  uint64_t r = 0;
#pragma unroll 1
  for (int b = 0; b < bits; ++b) {
    const uint32_t d = dst[b];
    if (d != kPackNone) r |= ((x >> b) & 1ull) << d;
  }
  return r;
}

// Entry t of a packed step, the general kernel's arithmetic (tree_step_kernel).
template <int kRing, bool kLLeaf, bool kRLeaf>
__device__ __forceinline__ void pack_entry(const PackItem& it, uint64_t t, const RingArgs& ring) {
  const uint64_t lo = it.op[0].base + pack_offset(it.op[0].tdst, it.t_bits, t);
  const uint64_t ro = it.op[1].base + pack_offset(it.op[1].tdst, it.t_bits, t);
  const uint32_t nk = 1u << it.k_bits;
  const uint8_t* lhs = it.op[0].ptr;
  const uint8_t* rhs = it.op[1].ptr;
  if constexpr (kRing == TSG_RING_OR_AND) {
    uint32_t acc = 0;
    for (uint32_t kk = 0; kk < nk; ++kk) {
      acc |= (uint32_t)lhs[lo + pack_offset(it.op[0].kdst, it.k_bits, kk)] &
             (uint32_t)rhs[ro + pack_offset(it.op[1].kdst, it.k_bits, kk)];
    }
    it.out[t] = acc ? 1 : 0;
  } else if constexpr (kRing == TSG_RING_U64) {
    uint64_t acc = 0;
    for (uint32_t kk = 0; kk < nk; ++kk) {
      acc += load_elem<kLLeaf, uint64_t>(lhs, lo + pack_offset(it.op[0].kdst, it.k_bits, kk)) *
             load_elem<kRLeaf, uint64_t>(rhs, ro + pack_offset(it.op[1].kdst, it.k_bits, kk));
    }
    reinterpret_cast<uint64_t*>(it.out)[t] = acc;
  } else {
    constexpr int leaves = (kLLeaf ? 1 : 0) + (kRLeaf ? 1 : 0);
    uint32_t acc[TSG_MAX_PRIMES] = {0, 0, 0, 0};
    uint64_t part[TSG_MAX_PRIMES] = {0, 0, 0, 0};
    const uint64_t lp = it.op[0].plane, rp = it.op[1].plane;
    for (uint32_t kk = 0; kk < nk; ++kk) {
      const uint64_t lko = lo + pack_offset(it.op[0].kdst, it.k_bits, kk);
      const uint64_t rko = ro + pack_offset(it.op[1].kdst, it.k_bits, kk);
#pragma unroll
      for (int p = 0; p < TSG_MAX_PRIMES; ++p) {
        if (p < ring.np) {
          const uint32_t l = load_elem<kLLeaf, uint32_t>(lhs, lko + (kLLeaf ? 0 : p * lp));
          const uint32_t r = load_elem<kRLeaf, uint32_t>(rhs, rko + (kRLeaf ? 0 : p * rp));
          part[p] += (uint64_t)l * r;
          if (leaves == 0 ? (kk & 1) : ((kk & 15) == 15)) {
            acc[p] = add_mod(acc[p], mont_finish(part[p], leaves, ring, p), ring.p[p]);
            part[p] = 0;
          }
        }
      }
    }
    uint32_t* out = reinterpret_cast<uint32_t*>(it.out);
#pragma unroll
    for (int p = 0; p < TSG_MAX_PRIMES; ++p) {
      if (p < ring.np)
        out[t + p * it.o_plane] = add_mod(acc[p], mont_finish(part[p], leaves, ring, p), ring.p[p]);
    }
  }
}

// The steps of a packed launch: warp w belongs to the last step whose warp0 <= w.
template <int kRing>
__global__ void __launch_bounds__(kThreads) tree_pack_kernel(const __grid_constant__ PackArgs a,
                                                             RingArgs ring) {
  const uint32_t warp = blockIdx.x * (kThreads / 32) + threadIdx.x / 32;
  if (warp >= a.n_warps) return;
  int lo = 0, hi = a.n_items - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (a.items[mid].warp0 <= warp) lo = mid;
    else hi = mid - 1;
  }
  const PackItem& it = a.items[lo];
  const uint64_t t = (uint64_t)(warp - it.warp0) * 32 + (threadIdx.x & 31);
  if (t >= (1ull << it.t_bits)) return;
  if constexpr (kRing == TSG_RING_OR_AND) {
    pack_entry<kRing, true, true>(it, t, ring);  // every OR-AND operand is uint8
  } else {
    switch (it.leaves) {
      case 0: pack_entry<kRing, false, false>(it, t, ring); break;
      case 1: pack_entry<kRing, true, false>(it, t, ring); break;
      case 2: pack_entry<kRing, false, true>(it, t, ring); break;
      default: pack_entry<kRing, true, true>(it, t, ring); break;
    }
  }
}

// Launcher of the packed kernel (tsg_pack.cu).
tsg_status launch_pack(int ring, const PackArgs& a, const RingArgs& ra, cudaStream_t st);

}  // namespace dev
}  // namespace tsg
