// Launch templates of the tile and streaming kernels, included by the per-ring
// translation units (tsg_tile_*.cu, tsg_stream_*.cu) so that each ring's kernels compile
// in their own unit.
#pragma once

#include "tsg_tree_dev.cuh"

namespace tsg {
namespace dev {
namespace {

template <int kRing, int V, int NE, int NK>
void launch_tile_t(const LaunchArgs& la, const RingArgs& ra, cudaStream_t st) {
  dim3 grid((unsigned)la.shape.tiles, (unsigned)la.cnt,
            la.t.plane_split ? (unsigned)ra.np : 1u);
  tree_step_tile_kernel<kRing, V, NE, NK><<<grid, la.shape.threads, 0, st>>>(la.t, ra);
}

template <int kRing, int V, int NE>
void launch_tile_nk(const LaunchArgs& la, const RingArgs& ra, cudaStream_t st) {
  switch (la.shape.nk) {
    case 1: launch_tile_t<kRing, V, NE, 1>(la, ra, st); break;
    case 2: launch_tile_t<kRing, V, NE, 2>(la, ra, st); break;
    case 4:  // unrolled only for OR-AND (the count rings stream their large K = 2 steps)
      if constexpr (kRing == TSG_RING_OR_AND) launch_tile_t<kRing, V, NE, 4>(la, ra, st);
      else launch_tile_t<kRing, V, NE, 0>(la, ra, st);
      break;
    default: launch_tile_t<kRing, V, NE, 0>(la, ra, st); break;
  }
}

template <int kRing, int V>
void launch_tile_ne(const LaunchArgs& la, const RingArgs& ra, cudaStream_t st) {
  switch (la.shape.ne) {
    case 1: launch_tile_nk<kRing, V, 1>(la, ra, st); break;
    case 2: launch_tile_nk<kRing, V, 2>(la, ra, st); break;
    default: launch_tile_nk<kRing, V, 4>(la, ra, st); break;
  }
}

// One E count of a ring (the vector width V chosen at run time).
template <int kRing, int NE>
void launch_tile_ring_ne(const LaunchArgs& la, const RingArgs& ra, cudaStream_t st) {
  if constexpr (kRing == TSG_RING_OR_AND) {
    if (la.shape.v == 16) {
      launch_tile_nk<kRing, 16, NE>(la, ra, st);
      return;
    }
  }
  if (la.shape.v == 4) launch_tile_nk<kRing, 4, NE>(la, ra, st);
  else launch_tile_nk<kRing, 1, NE>(la, ra, st);
}

template <int kRing>
void launch_tile_ring(const LaunchArgs& la, const RingArgs& ra, cudaStream_t st) {
  if constexpr (kRing == TSG_RING_OR_AND) {
    if (la.shape.v == 16) {
      launch_tile_ne<kRing, 16>(la, ra, st);
      return;
    }
  }
  if (la.shape.v == 4) launch_tile_ne<kRing, 4>(la, ra, st);
  else launch_tile_ne<kRing, 1>(la, ra, st);
}

template <int kRing, int NE, int NK, int NKP = 0>
tsg_status launch_stream_t(const LaunchArgs& la, const RingArgs& ra, cudaStream_t st) {
  auto kernel = tree_step_stream_kernel<kRing, NE, NK, NKP>;
  const size_t smem = (size_t)la.stream.stages * la.stream.stage_bytes;
  if (la.stream.stages < 2 || la.stream.stages > kStreamMaxStages || smem > kStreamBlockSmem)
    return fail(TSG_ERR_INVALID_ARGUMENT, "stream kernel: stage ring outside its limits");
  static bool configured[64] = {};  // one attribute call per instantiation and device
  int dev = 0;
  TSG_CUDA_TRY(cudaGetDevice(&dev));
  if (dev < 0 || dev >= 64) return fail(TSG_ERR_UNSUPPORTED, "device ordinal outside 0..63");
  if (!configured[dev]) {
    TSG_CUDA_TRY(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      (int)kStreamBlockSmem));
    configured[dev] = true;
  }
  const int np = kRing == TSG_RING_MODP ? ra.np : 1;
  const uint64_t blocks = std::min<uint64_t>(la.stream.work * np,
                                             (uint64_t)device_sm_count() * kStreamBlocksPerSm);
  kernel<<<(unsigned)blocks, kStreamThreads, smem, st>>>(la.t, ra, la.stream, la.f);
  return TSG_OK;
}

template <int kRing, int NE>
tsg_status launch_stream_nk(const LaunchArgs& la, const RingArgs& ra, cudaStream_t st) {
  switch (std::min(la.t.n_k, 4)) {
    case 1: return launch_stream_t<kRing, NE, 1>(la, ra, st);
    case 2: return launch_stream_t<kRing, NE, 2>(la, ra, st);
    default: return launch_stream_t<kRing, NE, 4>(la, ra, st);
  }
}

// Fused streaming steps: the consumer's summed count NK in {1, 2, 4} (one stage per item)
// and the producer's NKP in {1, 2}.
template <int kRing, int NE>
tsg_status launch_stream_fused_nk(const LaunchArgs& la, const RingArgs& ra, cudaStream_t st) {
  if (la.t.n_k > 4 || la.stream.kchunks != 1 || la.nkp < 1 || la.nkp > 2)
    return fail(TSG_ERR_INVALID_ARGUMENT, "fused stream kernel: shape outside its instantiations");
  const bool two = la.nkp == 2;
  switch (la.t.n_k) {
    case 1: return two ? launch_stream_t<kRing, NE, 1, 2>(la, ra, st) : launch_stream_t<kRing, NE, 1, 1>(la, ra, st);
    case 2: return two ? launch_stream_t<kRing, NE, 2, 2>(la, ra, st) : launch_stream_t<kRing, NE, 2, 1>(la, ra, st);
    default: return two ? launch_stream_t<kRing, NE, 4, 2>(la, ra, st) : launch_stream_t<kRing, NE, 4, 1>(la, ra, st);
  }
}

template <int kRing>
tsg_status launch_stream_fused_ring(const LaunchArgs& la, const RingArgs& ra, cudaStream_t st) {
  switch (la.shape.ne) {
    case 1: return launch_stream_fused_nk<kRing, 1>(la, ra, st);
    case 2: return launch_stream_fused_nk<kRing, 2>(la, ra, st);
    default: return launch_stream_fused_nk<kRing, 4>(la, ra, st);
  }
}

template <int kRing>
tsg_status launch_stream_ring(const LaunchArgs& la, const RingArgs& ra, cudaStream_t st) {
  switch (la.shape.ne) {
    case 1: return launch_stream_nk<kRing, 1>(la, ra, st);
    case 2: return launch_stream_nk<kRing, 2>(la, ra, st);
    default: return launch_stream_nk<kRing, 4>(la, ra, st);
  }
}

template <int kRing, int NE, int NK, int NKP>
void launch_fused_t(const LaunchArgs& la, const RingArgs& ra, cudaStream_t st) {
  dim3 grid((unsigned)la.shape.tiles, (unsigned)la.cnt);
  tree_step_fused_kernel<kRing, NE, NK, NKP><<<grid, la.shape.threads, 0, st>>>(la.t, la.f, ra);
}

template <int kRing, int NE, int NK>
void launch_fused_nkp(const LaunchArgs& la, const RingArgs& ra, cudaStream_t st) {
  if (la.nkp == 2) launch_fused_t<kRing, NE, NK, 2>(la, ra, st);
  else launch_fused_t<kRing, NE, NK, 1>(la, ra, st);
}

template <int kRing, int NE>
void launch_fused_nk(const LaunchArgs& la, const RingArgs& ra, cudaStream_t st) {
  switch (la.shape.nk) {
    case 1: launch_fused_nkp<kRing, NE, 1>(la, ra, st); break;
    case 2: launch_fused_nkp<kRing, NE, 2>(la, ra, st); break;
    default: launch_fused_nkp<kRing, NE, 4>(la, ra, st); break;
  }
}

// The fused kernel: V = 4, the consumer's summed count (1, 2 or 4) and the producer's (1
// or 2) are template parameters; the host only fuses steps within these limits.
template <int kRing>
tsg_status launch_fused_ring(const LaunchArgs& la, const RingArgs& ra, cudaStream_t st) {
  if (la.shape.v != 4 || (la.shape.nk != 1 && la.shape.nk != 2 && la.shape.nk != 4) ||
      la.nkp < 1 || la.nkp > 2)
    return fail(TSG_ERR_INVALID_ARGUMENT, "fused kernel: shape outside its instantiations");
  switch (la.shape.ne) {
    case 1: launch_fused_nk<kRing, 1>(la, ra, st); break;
    case 2: launch_fused_nk<kRing, 2>(la, ra, st); break;
    default: launch_fused_nk<kRing, 4>(la, ra, st); break;
  }
  return TSG_OK;
}

}  // namespace
}  // namespace dev
}  // namespace tsg
