// Tree executor of the tensorsat_gb300 C ABI: runs every pairwise contraction of a
// contraction tree over bit-indexed tensors (all wires of dimension 2) on the device, for
// a range of slices, and combines the per-slice roots. This replaces the per-node loop of
// SimpleContraction.contract (tensorsat/contractions/simple.py:251-292) and of cotengra's
// tree.contract behind CotengraContraction.contract (tensorsat/contractions/cotengra.py:
// 100-128), each node of which ends in FinRel._contract2 (tensorsat/lang/fin_rel.py:255-288).
//
// Data layout in HBM. A tensor over r bit-wires is a dense array of 2^r entries; bit i of
// the linear index is the value of the tensor's i-th wire counted from the last port
// (numpy C order). Slice-dependent intermediates hold `group` slices back to back:
// element (g, x) lives at g * 2^r + x. TSG_RING_MODP tensors keep one uint32 plane per
// prime, planes back to back. Leaves are uint8 {0,1} in one pool and keep their sliced
// wires; the executor selects the slice by fixing those bits.
//
// Index mapping. A step's thread index t packs (group slot g, output index o) as
// g * 2^out_bits + o. Each operand offset is a bit scatter of t plus a bit scatter of the
// summed index k, both encoded as runs (src bit, length, dst bit) so contiguous wires move
// as one shift-and-mask.

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstring>
#include <deque>
#include <type_traits>
#include <map>
#include <memory>
#include <mutex>
#include <vector>

#include "tsg_common.cuh"
#include "tsg_tree_dev.cuh"

namespace tsg {
using namespace dev;
namespace {

// Device-side failure record of the streaming kernels (they receive its address).
__device__ int g_device_error = 0;  // 0 = ok, else TSG_ERR_TIMEOUT

// Limit of each bounded device-side wait of the streaming kernels (tsg_set_wait_limit_ns)
// and the producer stall of tsg_debug_stall_producer (< 0: off). Read at every launch.
std::atomic<uint64_t> g_wait_limit_ns{kWaitLimitNs};
std::atomic<int64_t> g_stall_after{-1};

// Fused steps (tsg_set_fusion): on by default; read when a layout is made.
std::atomic<int> g_fusion{1};

// Address of g_device_error on the current device (looked up once per device).
tsg_status device_error_address(int** out) {
  static std::mutex mu;
  static int* addr[64] = {};
  int dev = 0;
  TSG_CUDA_TRY(cudaGetDevice(&dev));
  if (dev < 0 || dev >= 64) return fail(TSG_ERR_UNSUPPORTED, "device ordinal outside 0..63");
  std::lock_guard<std::mutex> lock(mu);
  if (!addr[dev]) {
    void* p = nullptr;
    TSG_CUDA_TRY(cudaGetSymbolAddress(&p, g_device_error));
    addr[dev] = static_cast<int*>(p);
  }
  *out = addr[dev];
  return TSG_OK;
}

// ------------------------------------------------------------------------------------
// Host side.

struct LeafInfo {
  int rank;
  int64_t offset;
  std::vector<int> spos;  // bit position of each sliced wire, -1 if absent
  bool dep;
};

struct StepInfo {
  int op[2];
  int out_bits, k_bits;
  int pos[2][TSG_MAX_BITS];
  bool dep;
};

struct Layout {
  int64_t group;
  int64_t elem_bytes;
  int planes;
  bool fusion;                  // fused steps enabled when the layout was made
  bool all_dep;                 // every step per slot (leaf variants: no shared prologue)
  bool levels;                  // buffers placed for level-order execution (packed runs)
  std::vector<int> level;       // tree level of each step (1 + its operands' highest)
  std::vector<int64_t> offset;  // byte offset of each step's output in the workspace
                                // (-1: computed inside its consumer, never stored)
  std::vector<int64_t> plane;   // plane stride (elements) of each step's output
  std::vector<int> fused_from;  // step whose result this step computes itself, or -1
  std::vector<char> fused_away; // the step is computed inside its consumer (no launch)
  int64_t bytes;
};

bool operand_dep(const std::vector<LeafInfo>& leaves, const std::vector<StepInfo>& steps, int v) {
  return v >= 0 ? leaves[v].dep : steps[-v - 1].dep;
}

int operand_rank(const std::vector<LeafInfo>& leaves, const std::vector<StepInfo>& steps, int v) {
  return v >= 0 ? leaves[v].rank : steps[-v - 1].out_bits;
}

int64_t align256(int64_t x) { return (x + 255) & ~int64_t(255); }

// First-fit allocator over a byte range, used to place intermediates by liveness.
class Arena {
 public:
  int64_t alloc(int64_t bytes) {
    for (auto it = free_.begin(); it != free_.end(); ++it) {
      if (it->second >= bytes) {
        const int64_t off = it->first;
        const int64_t rest = it->second - bytes;
        free_.erase(it);
        if (rest > 0) free_[off + bytes] = rest;
        return off;
      }
    }
    const int64_t off = top_;
    top_ += bytes;
    return off;
  }
  void release(int64_t off, int64_t bytes) {
    auto it = free_.emplace(off, bytes).first;
    auto nx = std::next(it);
    if (nx != free_.end() && it->first + it->second == nx->first) {
      it->second += nx->second;
      free_.erase(nx);
    }
    if (it != free_.begin()) {
      auto pv = std::prev(it);
      if (pv->first + pv->second == it->first) {
        pv->second += it->second;
        free_.erase(it);
      }
    }
    // give back a free block that touches the top
    if (!free_.empty()) {
      auto last = std::prev(free_.end());
      if (last->first + last->second == top_) {
        top_ = last->first;
        free_.erase(last);
      }
    }
  }
  int64_t peak() const { return peak_; }
  void note() { peak_ = std::max(peak_, top_); }

 private:
  std::map<int64_t, int64_t> free_;
  int64_t top_ = 0;
  int64_t peak_ = 0;
};

}  // namespace
}  // namespace tsg

struct tsg_plan {
  std::vector<tsg::LeafInfo> leaves;
  std::vector<tsg::StepInfo> steps;
  int num_sliced = 0;
  int root_bits = 0;
  int64_t max_entry_bits = 0;
  // cache keyed by (group, elem_bytes, planes, fusion, all_dep, levels); a deque keeps the
  // addresses of cached layouts valid while new ones are added
  std::deque<tsg::Layout> layouts;
  // per-step kernel options of each ring (TSG_STEP_*; tsg_plan_set_step_options), indexed
  // by ring; empty = none set
  std::vector<int32_t> options[3];
};

namespace tsg {
namespace {

tsg_status elem_info(int32_t ring, int32_t num_primes, int64_t* elem_bytes, int* planes) {
  switch (ring) {
    case TSG_RING_OR_AND:
      *elem_bytes = 1;
      *planes = 1;
      return TSG_OK;
    case TSG_RING_U64:
      *elem_bytes = 8;
      *planes = 1;
      return TSG_OK;
    case TSG_RING_MODP:
      if (num_primes < 1 || num_primes > TSG_MAX_PRIMES)
        return fail(TSG_ERR_INVALID_ARGUMENT, "plan_run: MODP needs 1..4 primes");
      *elem_bytes = 4;
      *planes = num_primes;
      return TSG_OK;
    default:
      return fail(TSG_ERR_INVALID_ARGUMENT, "plan_run: unknown ring");
  }
}

// Kernel options of step s in the ring of a layout's element size (0 when none are set).
int32_t step_option(const tsg_plan* plan, int64_t elem_bytes, int s) {
  const int ring = elem_bytes == 1 ? TSG_RING_OR_AND : (elem_bytes == 8 ? TSG_RING_U64 : TSG_RING_MODP);
  const std::vector<int32_t>& o = plan->options[ring];
  return o.empty() ? 0 : o[s];
}

// Live (unsliced) bits of operand v: a leaf's rank less its sliced bits, or a step's
// output bits.
int live_bits(const tsg_plan* plan, int v) {
  if (v < 0) return plan->steps[-v - 1].out_bits;
  const LeafInfo& lf = plan->leaves[v];
  int r = lf.rank;
  for (int p : lf.spos)
    if (p >= 0) r--;
  return r;
}

// Fused steps of a layout (every ring), for producers whose step options ask for it
// (TSG_STEP_FUSE; the autotuner sets it where fusing measured faster): a step p whose
// result P is read by exactly
// one consumer s is computed inside s, never stored, when
//   - P carries every output bit of s but at most two (the enumerated E bits of s's tile
//     form, so each entry of P is computed once per launch) and at least as many output
//     bits as s's other operand (P is the operand the tile form reuses across E);
//   - s sums at most 2 bits and p at most 1 (the fused kernel's instantiations), s has at
//     least two F bits (4 positions per thread) and at most 30 output bits, every tensor
//     involved has at most 31 bits, and both steps depend on the slice alike;
//   - P expands its operands: 2^bits(P) >= 2^16 and >= 4 x (entries of A + entries of B);
//   - s's other operand C is small (the tile form re-reads it per thread), or, in the
//     count rings, P carries s's 10 fastest F bits as its own bits 0-9 (s can stream,
//     staging C and computing P in its consumer warps);
//   - neither p's operands nor s take part in another fusion (decided in step order).
// Returns fused_from[s] = p or -1.
std::vector<int> choose_fusion(const tsg_plan* plan, int64_t group, int64_t elem_bytes) {
  const auto& steps = plan->steps;
  const int ns = (int)steps.size();
  std::vector<int> fused_from(ns, -1);
  std::vector<char> away(ns, 0);
  if (group > 65535) return fused_from;
  auto rank_ok = [&](int v) {
    return v >= 0 ? plan->leaves[v].rank <= 31 : steps[-v - 1].out_bits <= 31;
  };
  for (int s = 0; s < ns; ++s) {
    const StepInfo& cs = steps[s];
    if (away[s] || fused_from[s] >= 0) continue;
    if (cs.k_bits > 2 || cs.out_bits > 30 || cs.out_bits < 2) continue;
    for (int xo = 0; xo < 2; ++xo) {
      const int v = cs.op[xo];
      if (v >= 0) continue;
      const int p = -v - 1;
      const StepInfo& ps = steps[p];
      if (ps.dep != cs.dep || ps.k_bits > 1 || fused_from[p] >= 0) continue;
      const int32_t popt = step_option(plan, elem_bytes, p);
      if (popt & TSG_STEP_NO_FUSE) continue;
      if (ps.out_bits < 16) continue;
      if (!rank_ok(ps.op[0]) || !rank_ok(ps.op[1]) || !rank_ok(cs.op[1 - xo])) continue;
      int carried[2] = {0, 0};
      for (int o = 0; o < 2; ++o)
        for (int i = 0; i < cs.out_bits; ++i) carried[o] += cs.pos[o][i] >= 0;
      const int ne_bits = cs.out_bits - carried[xo];
      if (ne_bits > 2 || cs.out_bits - ne_bits < 2) continue;
      if (carried[xo] < carried[1 - xo] || (carried[xo] == carried[1 - xo] && xo != 0)) continue;
      const double pe = std::ldexp(1.0, ps.out_bits);
      const double ab = std::ldexp(1.0, live_bits(plan, ps.op[0])) +
                        std::ldexp(1.0, live_bits(plan, ps.op[1]));
      if (pe < 4.0 * ab) continue;
      // The tile form reads the consumer's other operand C per thread and E combination:
      // it must stay small (cache resident). Count rings may instead stream the fused
      // step, which stages C: P must then carry s's 10 fastest F bits as its bits 0-9.
      const int c_bits = live_bits(plan, cs.op[1 - xo]);
      const bool c_small = c_bits <= (elem_bytes == 1 ? 24 : 20);
      bool streamable = false;
      if (elem_bytes != 1) {
        int f = 0;
        streamable = true;
        for (int i = 0; i < cs.out_bits && f < kStreamTileBits; ++i) {
          if (cs.pos[xo][i] < 0) continue;  // an E bit
          streamable = streamable && cs.pos[xo][i] == f;
          ++f;
        }
        streamable = streamable && f == kStreamTileBits;
      }
      // fused steps trade P's HBM round trip for gathers of A and B in the consumer: only
      // where they were measured faster (TSG_STEP_FUSE on the producer, the autotuner's)
      if (!(popt & TSG_STEP_FUSE) || (!c_small && !streamable)) continue;
      fused_from[s] = p;
      away[p] = 1;
      break;
    }
  }
  return fused_from;
}

// Buffer placement of a plan for one slice group, element type and plane count. Steps
// run in step order (prologue of slice-independent steps, then each group), or, for
// `levels` (packed runs, one group holding every slice), level by level: all steps of a
// level may run at once, so a level's outputs are placed before its operands are freed.
tsg_status get_layout(tsg_plan* plan, int64_t group, int64_t elem_bytes, int planes,
                      const Layout** out, bool all_dep = false, bool levels = false) {
  const bool fusion = g_fusion.load(std::memory_order_relaxed) != 0;
  for (const Layout& l : plan->layouts) {
    if (l.group == group && l.elem_bytes == elem_bytes && l.planes == planes &&
        l.fusion == fusion && l.all_dep == all_dep && l.levels == levels) {
      *out = &l;
      return TSG_OK;
    }
  }
  const auto& steps = plan->steps;
  const int ns = (int)steps.size();
  Layout lay;
  lay.group = group;
  lay.elem_bytes = elem_bytes;
  lay.planes = planes;
  lay.fusion = fusion;
  lay.all_dep = all_dep;
  lay.levels = levels;
  auto dep = [&](int x) { return all_dep || steps[x].dep; };
  lay.level.assign(ns, 1);
  int max_level = 0;
  for (int s = 0; s < ns; ++s) {
    int l = 0;
    for (int o = 0; o < 2; ++o)
      if (steps[s].op[o] < 0) l = std::max(l, lay.level[-steps[s].op[o] - 1]);
    lay.level[s] = l + 1;
    max_level = std::max(max_level, l + 1);
  }
  lay.offset.assign(ns, -1);
  lay.plane.assign(ns, 0);
  lay.fused_from = fusion ? choose_fusion(plan, group, elem_bytes) : std::vector<int>(ns, -1);
  lay.fused_away.assign(ns, 0);
  for (int s = 0; s < ns; ++s)
    if (lay.fused_from[s] >= 0) lay.fused_away[lay.fused_from[s]] = 1;
  std::vector<int64_t> bytes(ns, 0);
  for (int s = 0; s < ns; ++s) {
    const int64_t slices = dep(s) ? group : 1;
    if (steps[s].out_bits + 64 - __builtin_clzll((unsigned long long)slices) > 62)
      return fail(TSG_ERR_TOO_LARGE, "plan_run: group * tensor size exceeds 2^62 entries");
    const int64_t elems = slices << steps[s].out_bits;
    lay.plane[s] = elems;
    const long double b = (long double)elems * elem_bytes * planes;
    if (b > 9.0e18L) return fail(TSG_ERR_TOO_LARGE, "plan_run: tensor bytes overflow");
    bytes[s] = align256(elems * elem_bytes * planes);
  }
  Arena arena;
  // prologue: slice-independent steps; then one group of slice-dependent steps. A fused
  // step gets no buffer; its operands stay live until its consumer has run.
  auto release_operands = [&](int s, int r) {
    for (int o = 0; o < 2; ++o) {
      const int v = steps[r].op[o];
      if (v >= 0) continue;
      const int x = -v - 1;
      if (lay.fused_away[x]) continue;
      // an independent result read by a dependent step is re-read by every group
      if (!dep(x) && dep(s)) continue;
      arena.release(lay.offset[x], bytes[x]);
    }
  };
  if (levels) {
    // one group: every operand is read once, by the level after its own or later
    auto release_all = [&](int r) {
      for (int o = 0; o < 2; ++o) {
        const int v = steps[r].op[o];
        if (v < 0 && !lay.fused_away[-v - 1]) arena.release(lay.offset[-v - 1], bytes[-v - 1]);
      }
    };
    for (int l = 1; l <= max_level; ++l) {
      for (int s = 0; s < ns; ++s) {
        if (lay.level[s] != l || lay.fused_away[s]) continue;
        lay.offset[s] = arena.alloc(bytes[s]);
        arena.note();
      }
      for (int s = 0; s < ns; ++s) {
        if (lay.level[s] != l || lay.fused_away[s]) continue;
        release_all(s);
        if (lay.fused_from[s] >= 0) release_all(lay.fused_from[s]);
      }
    }
  } else {
    for (int phase = 0; phase < 2; ++phase) {
      for (int s = 0; s < ns; ++s) {
        if (dep(s) != (phase == 1) || lay.fused_away[s]) continue;
        lay.offset[s] = arena.alloc(bytes[s]);
        arena.note();
        release_operands(s, s);
        if (lay.fused_from[s] >= 0) release_operands(s, lay.fused_from[s]);
      }
    }
  }
  lay.bytes = std::max<int64_t>(arena.peak(), 256);
  plan->layouts.push_back(lay);
  *out = &plan->layouts.back();
  return TSG_OK;
}

// Encodes (src bit -> dst bit) pairs, sorted by src, as runs.
tsg_status make_bitmap(std::vector<std::pair<int, int>> pairs, BitMap* m) {
  std::sort(pairs.begin(), pairs.end());
  std::memset(m, 0, sizeof(*m));
  for (const auto& pr : pairs) {
    if (m->n > 0) {
      const int i = m->n - 1;
      if (m->src[i] + m->len[i] == pr.first && m->dst[i] + m->len[i] == pr.second) {
        m->len[i]++;
        continue;
      }
    }
    if (m->n >= kMaxRuns) return fail(TSG_ERR_TOO_LARGE, "plan_run: too many bit runs");
    m->src[m->n] = (uint8_t)pr.first;
    m->dst[m->n] = (uint8_t)pr.second;
    m->len[m->n] = 1;
    m->n++;
  }
  return TSG_OK;
}

struct RunCtx {
  const tsg_plan* plan;
  const Layout* lay;
  int ring;
  RingArgs ra;
  const uint8_t* pool;
  uint8_t* ws;
  cudaStream_t stream;
  int g_bits;  // log2(slices per launch group)
  // leaf variants (tsg_plan_run_variants): the launch's slots are variant * 2^g_bits +
  // slice; every step runs per slot, and variant v's leaves sit v * 2^vstride_bits bytes
  // further into the pool
  bool all_dep = false;
  int v_bits = 0;
  int vstride_bits = 0;
  uint64_t leaf_extra = 0;  // ((2^v_bits - 1) << vstride_bits): extra extent of every leaf
  bool dep(const StepInfo& st) const { return all_dep || st.dep; }
};

template <int kRing, bool kL, bool kR>
void launch_step_t(const StepArgs& a, const RingArgs& ra, cudaStream_t st) {
  tree_step_kernel<kRing, kL, kR><<<grid_for(a.total, kThreads, 8), kThreads, 0, st>>>(a, ra);
}

template <int kRing, bool kL, bool kR>
void launch_sum_t(const StepArgs& a, const RingArgs& ra, cudaStream_t st) {
  const unsigned blocks = (unsigned)std::min<uint64_t>(a.total, (uint64_t)device_sm_count() * 16);
  tree_step_sum_kernel<kRing, kL, kR><<<blocks, kThreads, 0, st>>>(a, ra);
}

// A step of the general form with few outputs and many summed combinations runs one block
// per output (tree_step_sum_kernel); every other one thread per output.
bool use_sum_kernel(const StepArgs& a) {
  return a.k_bits >= 6 && a.total <= (uint64_t)device_sm_count() * 32;
}

template <int kRing>
void launch_step_ring(bool l_leaf, bool r_leaf, const StepArgs& a, const RingArgs& ra,
                      cudaStream_t st) {
  if (use_sum_kernel(a)) {
    if (l_leaf) {
      if (r_leaf) launch_sum_t<kRing, true, true>(a, ra, st);
      else launch_sum_t<kRing, true, false>(a, ra, st);
    } else {
      if (r_leaf) launch_sum_t<kRing, false, true>(a, ra, st);
      else launch_sum_t<kRing, false, false>(a, ra, st);
    }
    return;
  }
  if (l_leaf) {
    if (r_leaf) launch_step_t<kRing, true, true>(a, ra, st);
    else launch_step_t<kRing, true, false>(a, ra, st);
  } else {
    if (r_leaf) launch_step_t<kRing, false, true>(a, ra, st);
    else launch_step_t<kRing, false, false>(a, ra, st);
  }
}

// Largest value scatter_bits(m, x) takes for any x < 2^bits (the runs are disjoint bit
// fields, so setting every source bit maximises the result).
uint64_t scatter_max(const BitMap& m, int bits) {
  uint64_t r = 0;
  for (int i = 0; i < m.n; ++i) {
    for (int b = 0; b < m.len[i]; ++b) {
      if (m.src[i] + b < bits) r |= 1ull << (m.dst[i] + b);
    }
  }
  return r;
}

int bit_width(uint64_t x) { return x == 0 ? 0 : 64 - __builtin_clzll((unsigned long long)x); }

// Host-side bounds check of one launch: every element offset the kernel can form for an
// operand must stay inside that operand (its leaf, or its workspace buffer), and the
// output index inside the output buffer. Runs before every launch and in
// tsg_plan_validate, so an inconsistent plan is reported instead of reaching the GPU.
tsg_status check_step_bounds(const RunCtx& c, int s, const StepArgs& a, const bool is_leaf[2]) {
  const tsg_plan* plan = c.plan;
  const StepInfo& st = plan->steps[s];
  const int tbits = bit_width(a.total - 1);
  if (a.total > (uint64_t)c.lay->plane[s])
    return fail(TSG_ERR_INVALID_ARGUMENT, "plan bounds: output exceeds its buffer");
  for (int o = 0; o < 2; ++o) {
    const BitMap& tm = o == 0 ? a.lt : a.rt;
    const BitMap& km = o == 0 ? a.lk : a.rk;
    const uint64_t base = o == 0 ? a.l_base : a.r_base;
    const uint64_t hi = base + scatter_max(tm, tbits) + scatter_max(km, st.k_bits);
    const int v = st.op[o];
    uint64_t lo_ext, hi_ext;
    if (is_leaf[o]) {
      const LeafInfo& lf = plan->leaves[v];
      lo_ext = (uint64_t)lf.offset;
      hi_ext = lo_ext + (1ull << lf.rank) + c.leaf_extra;
    } else {
      lo_ext = 0;
      hi_ext = (uint64_t)c.lay->plane[-v - 1];
    }
    if (base < lo_ext || hi >= hi_ext)
      return fail(TSG_ERR_INVALID_ARGUMENT, "plan bounds: operand offset outside its tensor");
  }
  return TSG_OK;
}

// Index description of one operand of one launch: output-bit, summed-bit and slot-bit
// pairs (source bit -> operand bit) and the constant element offset.
struct OperandDesc {
  std::vector<std::pair<int, int>> tp, kp, gp;
  uint64_t base = 0;
  const uint8_t* ptr = nullptr;
  uint64_t plane = 0;
  bool leaf = false;
};

OperandDesc describe_operand(const RunCtx& c, const StepInfo& st, int o, int64_t base) {
  const tsg_plan* plan = c.plan;
  const int gb = c.dep(st) ? c.g_bits : 0;
  OperandDesc d;
  const int v = st.op[o];
  for (int i = 0; i < st.out_bits; ++i)
    if (st.pos[o][i] >= 0) d.tp.push_back({i, st.pos[o][i]});
  for (int i = 0; i < st.k_bits; ++i)
    if (st.pos[o][st.out_bits + i] >= 0) d.kp.push_back({i, st.pos[o][st.out_bits + i]});
  if (v >= 0) {
    const LeafInfo& lf = plan->leaves[v];
    d.ptr = c.pool;
    d.base = (uint64_t)lf.offset;
    for (int j = 0; j < plan->num_sliced; ++j) {
      if (lf.spos[j] < 0 || !c.dep(st)) continue;
      if (j < gb) {
        d.gp.push_back({j, lf.spos[j]});
      } else {
        d.base += (uint64_t)((base >> j) & 1) << lf.spos[j];
      }
    }
    // variant bits of the slot select the variant's copy of the pool
    for (int i = 0; i < c.v_bits; ++i) d.gp.push_back({gb + i, c.vstride_bits + i});
    d.leaf = true;
  } else {
    const int x = -v - 1;
    const StepInfo& xs = plan->steps[x];
    d.ptr = (c.ws && c.lay->offset[x] >= 0) ? c.ws + c.lay->offset[x] : nullptr;
    d.plane = (uint64_t)c.lay->plane[x];
    if (c.dep(xs))
      for (int j = 0; j < gb + c.v_bits; ++j) d.gp.push_back({j, xs.out_bits + j});
  }
  return d;
}

tsg_status make_narrow(std::vector<std::pair<int, int>> pairs, NarrowMap* m, bool* ok) {
  std::sort(pairs.begin(), pairs.end());
  std::memset(m, 0, sizeof(*m));
  for (const auto& pr : pairs) {
    if (pr.second >= 32 || pr.first >= 32) {
      *ok = false;
      return TSG_OK;
    }
    if (m->n > 0) {
      const int i = m->n - 1;
      if (m->src[i] + m->len[i] == pr.first && m->dst[i] + m->len[i] == pr.second) {
        m->len[i]++;
        continue;
      }
    }
    if (m->n >= kMaxNarrowRuns) {
      *ok = false;
      return TSG_OK;
    }
    m->src[m->n] = (uint8_t)pr.first;
    m->dst[m->n] = (uint8_t)pr.second;
    m->len[m->n] = 1;
    m->n++;
  }
  return TSG_OK;
}

// Scatter of x through (src bit -> dst bit) pairs, computed directly on the host.
uint64_t scatter_pairs(const std::vector<std::pair<int, int>>& pairs, uint64_t x) {
  uint64_t r = 0;
  for (const auto& pr : pairs)
    if ((x >> pr.first) & 1) r |= 1ull << pr.second;
  return r;
}


// Index bits of a tile form: the F bits (threads and tiles, fastest first) and the E bits
// (enumerated inside a thread) of the step's output.
struct TileBits {
  std::vector<int> fbits, ebits;
};

// Fills the tile operand `op` of an operand whose output-bit positions are pos[0 ..
// out_bits) (-1: not carried) and whose summed, slot and constant terms are in `d`;
// sets *ok = false when the operand is outside what the tile kernel handles.
tsg_status fill_tile_operand(TileOperand& op, const int* pos, const OperandDesc& d,
                             const uint8_t* ptr, const TileBits& tb, int tile_bits, int v,
                             int n_k, int ring, bool* ok) {
  const std::vector<int>& fbits = tb.fbits;
  const std::vector<int>& ebits = tb.ebits;
  const int nf = (int)fbits.size();
  const int ne = 1 << ebits.size();
  op.ptr = ptr;
  op.base = d.base;
  op.plane = d.plane;
  op.leaf = d.leaf ? 1 : 0;
  std::vector<std::pair<int, int>> lo, hi, ep;
  for (int fi = 0; fi < nf; ++fi) {
    const int p = pos[fbits[fi]];
    if (p >= 0) (fi < tile_bits ? lo : hi).push_back({fi, p});
  }
  for (size_t b = 0; b < ebits.size(); ++b) {
    const int p = pos[ebits[b]];
    if (p >= 0) ep.push_back({(int)b, p});
  }
  TSG_TRY(make_narrow(lo, &op.f_lo, ok));
  if (*ok) TSG_TRY(make_narrow(hi, &op.f_hi, ok));
  for (const auto& pr : d.kp)
    if (pr.second >= 32) *ok = false;
  if (!*ok) return TSG_OK;
  TSG_TRY(make_bitmap(d.gp, &op.g));
  bool contig = v >= 4, bcast = true;
  for (int j = 0; j < v; ++j) {
    op.tab[j] = (uint32_t)scatter_pairs(lo, j);
    contig = contig && op.tab[j] == (uint32_t)j;
    bcast = bcast && op.tab[j] == 0;
  }
  // vector loads need every start offset to be a multiple of V elements: the fastest
  // output bits occupy the operand's fastest bits, so only the constant part can break
  // that (leaf offsets are the caller's; workspace buffers are 256-byte aligned)
  if (contig && (op.base & (uint64_t)(v - 1)) != 0) contig = false;
  op.mode = contig ? kModeContig : (bcast ? kModeBcast : kModeGather);
  if (op.mode == kModeGather && v == 4) {
    // exactly two distinct offsets, 0 and tab[3] (one of the two fastest output bits)
    bool pair = op.tab[0] == 0 && op.tab[3] != 0;
    int sel = 0;
    for (int j = 0; j < v && pair; ++j) {
      if (op.tab[j] == op.tab[3]) sel |= 1 << j;
      else if (op.tab[j] != 0) pair = false;
    }
    if (pair) {
      op.mode = kModePair;
      op.pair_sel = sel;
    }
  }
  // positions {0, 1, d, d + 1}: two 2-element vector loads (count rings: intermediates;
  // OR-AND: any operand, two 2-byte loads), decided once the E and summed offsets are known
  const bool dual_shape = op.mode == kModeGather && v == 4 &&
                          (ring == TSG_RING_OR_AND || !op.leaf) && op.tab[0] == 0 &&
                          op.tab[1] == 1 && op.tab[2] != 0 && op.tab[3] == op.tab[2] + 1;
  if (op.mode == kModeGather && v == 16) {
    // carried fast F bits (F index, operand bit), ascending F index: distinct value d
    // has bit k of d = carried bit k of the position
    std::vector<std::pair<int, int>> cb;
    for (const auto& pr : lo)
      if (pr.first < 4) cb.push_back(pr);
    if (cb.size() == 4) {
      // kModeQuad (quad_operand admitted it): F bits fa, fb are operand bits 0, 1; fc, fd
      // select one of four words
      int fbyte[2] = {-1, -1};
      std::vector<std::pair<int, int>> word;  // (F bit, operand bit) of the word-selecting bits
      for (const auto& pr : cb) {
        if (pr.second <= 1) fbyte[pr.second] = pr.first;
        else word.push_back(pr);
      }
      if (fbyte[0] < 0 || fbyte[1] < 0 || word.size() != 2) {
        *ok = false;
        return TSG_OK;
      }
      op.mode = kModeQuad;
      for (int q = 0; q < 4; ++q)
        op.dtab[q] = ((q & 1) ? (1u << word[0].second) : 0u) + ((q & 2) ? (1u << word[1].second) : 0u);
      for (int i = 0; i < 4; ++i) {
        int src[2] = {-1, -1};
        uint32_t sel = 0;
        for (int t = 0; t < 4; ++t) {
          const int j = 4 * i + t;
          const int q = ((j >> word[0].first) & 1) | (((j >> word[1].first) & 1) << 1);
          const int byte = ((j >> fbyte[0]) & 1) | (((j >> fbyte[1]) & 1) << 1);
          int slot = q == src[0] ? 0 : (q == src[1] ? 1 : -1);
          if (slot < 0) {
            slot = src[0] < 0 ? 0 : 1;
            if (src[slot] >= 0) {
              *ok = false;  // three source words: excluded by quad_operand
              return TSG_OK;
            }
            src[slot] = q;
          }
          sel |= (uint32_t)(slot * 4 + byte) << (4 * t);
        }
        if (src[1] < 0) src[1] = src[0];
        op.qsrc[i] = (uint32_t)src[0] | ((uint32_t)src[1] << 2);
        op.psel[i] = sel;
      }
    } else {
      if (cb.empty() || cb.size() > 3) {
        *ok = false;  // excluded by the choice of V
        return TSG_OK;
      }
      op.mode = kModePerm;
      op.pn = 1 << cb.size();
      for (int dd = 0; dd < op.pn; ++dd) {
        uint32_t off = 0;
        for (size_t k = 0; k < cb.size(); ++k)
          if ((dd >> k) & 1) off |= 1u << cb[k].second;
        op.dtab[dd] = off;
      }
      for (int i = 0; i < 4; ++i) {
        uint32_t sel = 0;
        for (int t = 0; t < 4; ++t) {
          const int j = 4 * i + t;
          uint32_t dd = 0;
          for (size_t k = 0; k < cb.size(); ++k) dd |= (uint32_t)((j >> cb[k].first) & 1) << k;
          sel |= dd << (4 * t);
        }
        op.psel[i] = sel;
      }
    }
  }
  op.has_e = ep.empty() ? 0 : 1;
  for (int e = 0; e < ne; ++e) op.e_off[e] = (uint32_t)scatter_pairs(ep, e);
  for (int kk = 0; kk < n_k; ++kk) op.k_off[kk] = (uint32_t)scatter_pairs(d.kp, kk);
  if (dual_shape) {
    // every offset term but the first position bit even: each pair starts on an even
    // element (check_tile_bounds proves the same again before the launch)
    bool even = (op.tab[2] & 1) == 0 && (op.base & 1) == 0 && (op.plane & 1) == 0;
    for (int i = 0; i < op.g.n; ++i) even = even && op.g.dst[i] >= 1;
    for (const NarrowMap* m : {&op.f_hi, &op.f_lo})
      for (int i = 0; i < m->n; ++i) even = even && !(m->dst[i] < 1 && m->src[i] >= 1);
    for (int e = 0; e < ne; ++e) even = even && (op.e_off[e] & 1) == 0;
    for (int kk = 0; kk < n_k; ++kk) even = even && (op.k_off[kk] & 1) == 0;
    if (even) op.mode = kModeDual;
  }
  return TSG_OK;
}

// OR-AND, V = 16, an operand carrying all four fastest output bits (F bits 0-3): readable
// as four aligned 4-byte words when two of those bits are its own bits 0 and 1, at most
// one of the other two is an F bit below 2 (so each output word draws on at most two
// words), and every other term of its offsets is a multiple of 4 (its constant offset,
// output bits above 3, summed and slot bits).
bool quad_operand(const StepInfo& st, const OperandDesc& d, int o) {
  int low = 0, hi_small = 0;
  for (int b = 0; b < 4; ++b) {
    const int p = st.pos[o][b];
    if (p < 0) return false;
    if (p <= 1) low++;
    else if (b < 2) hi_small++;
  }
  if (low != 2 || hi_small > 1 || (d.base & 3) != 0) return false;
  for (int i = 4; i < st.out_bits; ++i)
    if (st.pos[o][i] >= 0 && st.pos[o][i] < 2) return false;
  for (const auto& pr : d.kp)
    if (pr.second < 2) return false;
  for (const auto& pr : d.gp)
    if (pr.second < 2) return false;
  return true;
}

// Builds the tile form of step s from the operand descriptions; sets *ok = false when the
// step is outside what the tile kernel handles (it then runs the general kernel). The
// chosen F and E bits go to *bits_out when given.
tsg_status build_tile(const StepInfo& st, const OperandDesc d[2], const StepArgs& a,
                      uint64_t cnt, int ring, TileArgs* t, TileShape* shape, bool* ok,
                      TileBits* bits_out = nullptr, bool allow_v16 = true) {
  std::memset(t, 0, sizeof(*t));
  *ok = st.out_bits <= 30 && st.k_bits <= 6 && cnt <= 65535;
  if (!*ok) return TSG_OK;
  // E: output bits the larger operand does not carry (at most 2, highest first)
  int carried[2] = {0, 0};
  for (int o = 0; o < 2; ++o)
    for (const auto& pr : d[o].tp) carried[o]++;
  const int big = carried[0] >= carried[1] ? 0 : 1;
  TileBits tb;
  std::vector<int>& ebits = tb.ebits;
  std::vector<int>& fbits = tb.fbits;
  {
    std::vector<int> cand;
    for (int i = 0; i < st.out_bits; ++i)
      if (st.pos[big][i] < 0) cand.push_back(i);
    while (cand.size() > 2) cand.erase(cand.begin());  // keep the two highest
    ebits = cand;
    for (int i = 0; i < st.out_bits; ++i)
      if (std::find(ebits.begin(), ebits.end(), i) == ebits.end()) fbits.push_back(i);
  }
  const int nf = (int)fbits.size();
  int v = nf >= 2 ? 4 : 1;
  if (ring == TSG_RING_OR_AND && nf >= 4 && allow_v16) {
    // 16 byte-wide positions when the output takes the 4 fastest F bits as its 4 fastest
    // bits and every operand carries them as its own 4 fastest bits (vector load), at most
    // 3 of them (byte permutes of <= 8 distinct values) or none (broadcast)
    bool ok16 = true;
    for (int b = 0; b < 4 && ok16; ++b) ok16 = fbits[b] == b;
    for (int o = 0; o < 2 && ok16; ++o) {
      int carried = 0;
      bool ident = true;
      for (int b = 0; b < 4; ++b) {
        const int p = st.pos[o][fbits[b]];
        if (p >= 0) {
          carried++;
          ident = ident && p == b;
        }
      }
      if (carried == 4 && !(ident && (d[o].base & 15) == 0))
        ok16 = quad_operand(st, d[o], o);
    }
    if (ok16) v = 16;
  }
  const int ne = 1 << ebits.size();
  uint64_t positions = (uint64_t)1 << nf;           // F positions per slice
  uint64_t threads = std::min<uint64_t>(kThreads, positions / v);
  if (threads == 0) threads = 1;
  int tile_bits = 0;
  while (((uint64_t)1 << tile_bits) < threads * v) tile_bits++;
  shape->v = v;
  shape->ne = ne;
  shape->nk = st.k_bits <= 2 ? (1 << st.k_bits) : 0;  // unrolled summed combinations
  shape->threads = (unsigned)threads;
  shape->tiles = positions >> tile_bits;
  if (shape->tiles >= (1ull << 31)) {
    *ok = false;
    return TSG_OK;
  }
  t->tile_bits = tile_bits;
  t->n_k = 1 << st.k_bits;
  t->n_out = 1u << st.out_bits;
  t->out = a.out;
  t->o_plane = a.o_plane;
  // output maps: F index bit fi -> output bit fbits[fi]; E combo bits -> output bits
  std::vector<std::pair<int, int>> olo, ohi, oe;
  for (int fi = 0; fi < nf; ++fi) (fi < tile_bits ? olo : ohi).push_back({fi, fbits[fi]});
  for (size_t b = 0; b < ebits.size(); ++b) oe.push_back({(int)b, ebits[b]});
  TSG_TRY(make_narrow(olo, &t->of_lo, ok));
  if (*ok) TSG_TRY(make_narrow(ohi, &t->of_hi, ok));
  if (!*ok) return TSG_OK;
  bool ocontig = v >= 4;
  for (int j = 0; j < v; ++j) {
    t->o_tab[j] = (uint32_t)scatter_pairs(olo, j);
    ocontig = ocontig && t->o_tab[j] == (uint32_t)j;
  }
  t->o_contig = ocontig ? 1 : 0;
  for (int e = 0; e < ne; ++e) t->o_e[e] = (uint32_t)scatter_pairs(oe, e);
  for (int o = 0; o < 2; ++o) {
    TSG_TRY(fill_tile_operand(t->op[o], st.pos[o], d[o], o == 0 ? a.lhs : a.rhs, tb,
                              tile_bits, v, t->n_k, ring, ok));
    if (!*ok) return TSG_OK;
  }
  if (bits_out) *bits_out = tb;
  return TSG_OK;
}

// Largest scatter of a source value whose set bits lie in [from, to).
uint32_t narrow_max(const NarrowMap& m, int to, int from = 0) {
  uint32_t r = 0;
  for (int i = 0; i < m.n; ++i)
    for (int b = 0; b < m.len[i]; ++b) {
      const int src = m.src[i] + b;
      if (src >= from && src < to) r |= 1u << (m.dst[i] + b);
    }
  return r;
}

// Bounds check of the tile form: the largest offset each term can take (slot, tile,
// thread, V position, E combination, summed combination) added up must stay inside the
// operand and the output buffer.
tsg_status check_tile_bounds(const RunCtx& c, int s, const LaunchArgs& la) {
  const tsg_plan* plan = c.plan;
  const StepInfo& st = plan->steps[s];
  const TileArgs& t = la.t;
  const TileShape& sh = la.shape;
  const int gbits = bit_width(la.cnt - 1);
  const int nbits = bit_width(sh.tiles - 1) + t.tile_bits;
  const int vbits = sh.v == 16 ? 4 : (sh.v == 4 ? 2 : 0);  // thread positions: multiples of V
  if ((uint64_t)sh.threads * sh.v != (1ull << t.tile_bits))
    return fail(TSG_ERR_INVALID_ARGUMENT, "tile bounds: threads x V is not the tile size");
  for (int o = 0; o < 2; ++o) {
    const TileOperand& op = t.op[o];
    uint32_t tab = 0, eo = 0, ko = 0;
    for (int j = 0; j < sh.v; ++j) tab = std::max(tab, op.tab[j]);
    for (int e = 0; e < sh.ne; ++e) eo = std::max(eo, op.e_off[e]);
    for (int kk = 0; kk < t.n_k; ++kk) ko = std::max(ko, op.k_off[kk]);
    const uint64_t hi = op.base + scatter_max(op.g, gbits) + narrow_max(op.f_hi, nbits) +
                        narrow_max(op.f_lo, t.tile_bits, vbits) + tab + eo + ko;
    const int v = st.op[o];
    const uint64_t lo_ext = la.is_leaf[o] ? (uint64_t)plan->leaves[v].offset : 0;
    const uint64_t hi_ext = la.is_leaf[o] ? lo_ext + (1ull << plan->leaves[v].rank) + c.leaf_extra
                                          : (uint64_t)c.lay->plane[-v - 1];
    if (op.base < lo_ext || hi >= hi_ext)
      return fail(TSG_ERR_INVALID_ARGUMENT, "tile bounds: operand offset outside its tensor");
  }
  // Vector accesses: a contiguous operand (V positions = its V fastest elements) and a
  // contiguous output are read / written V elements at a time, so every other term of
  // their offsets must be a multiple of V: bit positions of the slot, tile, E and summed
  // maps at or above log2(V), constant and plane offsets multiples of V.
  const uint32_t vmask = (uint32_t)sh.v - 1;
  const int vb = vbits;
  auto map_ok = [&](const NarrowMap& m) {
    for (int i = 0; i < m.n; ++i)
      if (m.dst[i] < vb && m.src[i] >= vb) return false;
    return true;
  };
  auto bitmap_ok = [&](const BitMap& m) {
    for (int i = 0; i < m.n; ++i)
      if (m.dst[i] < vb) return false;
    return true;
  };
  for (int o = 0; o < 2 && sh.v > 1; ++o) {
    const TileOperand& op = t.op[o];
    if (op.mode != kModeContig) continue;
    bool ok = (op.base & vmask) == 0 && (op.plane & vmask) == 0 && bitmap_ok(op.g) &&
              map_ok(op.f_hi) && map_ok(op.f_lo);
    for (int j = 0; j < sh.v; ++j) ok = ok && op.tab[j] == (uint32_t)j;
    for (int e = 0; e < sh.ne; ++e) ok = ok && (op.e_off[e] & vmask) == 0;
    for (int kk = 0; kk < t.n_k; ++kk) ok = ok && (op.k_off[kk] & vmask) == 0;
    if (!ok) return fail(TSG_ERR_INVALID_ARGUMENT, "tile bounds: vector load not aligned");
  }
  // Word loads of kModeQuad: every offset term but the four fastest positions, and every
  // word offset, must be a multiple of 4 bytes.
  for (int o = 0; o < 2 && sh.v == 16; ++o) {
    const TileOperand& op = t.op[o];
    if (op.mode != kModeQuad) continue;
    bool ok = (op.base & 3) == 0 && (op.plane & 3) == 0;
    for (int i = 0; i < op.g.n; ++i) ok = ok && op.g.dst[i] >= 2;
    for (int i = 0; i < op.f_hi.n; ++i) ok = ok && op.f_hi.dst[i] >= 2;
    for (int i = 0; i < op.f_lo.n; ++i)
      for (int b = 0; b < op.f_lo.len[i]; ++b)
        if (op.f_lo.src[i] + b >= 4) ok = ok && op.f_lo.dst[i] + b >= 2;
    for (int q = 0; q < 4; ++q) ok = ok && (op.dtab[q] & 3) == 0;
    for (int e = 0; e < sh.ne; ++e) ok = ok && (op.e_off[e] & 3) == 0;
    for (int kk = 0; kk < t.n_k; ++kk) ok = ok && (op.k_off[kk] & 3) == 0;
    if (!ok) return fail(TSG_ERR_INVALID_ARGUMENT, "tile bounds: word loads not aligned");
  }
  // Two-element vector loads (kModeDual): every offset term but the first position bit
  // must be even.
  for (int o = 0; o < 2 && sh.v == 4; ++o) {
    const TileOperand& op = t.op[o];
    if (op.mode != kModeDual) continue;
    auto map1 = [](const NarrowMap& m) {
      for (int i = 0; i < m.n; ++i)
        if (m.dst[i] < 1 && m.src[i] >= 1) return false;
      return true;
    };
    bool ok = (op.base & 1) == 0 && (op.plane & 1) == 0 && (op.tab[2] & 1) == 0 &&
              op.tab[1] == 1 && map1(op.f_hi) && map1(op.f_lo);
    for (int i = 0; i < op.g.n; ++i) ok = ok && op.g.dst[i] >= 1;
    for (int e = 0; e < sh.ne; ++e) ok = ok && (op.e_off[e] & 1) == 0;
    for (int kk = 0; kk < t.n_k; ++kk) ok = ok && (op.k_off[kk] & 1) == 0;
    if (!ok) return fail(TSG_ERR_INVALID_ARGUMENT, "tile bounds: paired vector load not aligned");
  }
  if (t.o_contig && sh.v > 1) {
    bool ok = (t.n_out & vmask) == 0 && (la.a.o_plane & vmask) == 0 && map_ok(t.of_hi) &&
              map_ok(t.of_lo);
    for (int j = 0; j < sh.v; ++j) ok = ok && t.o_tab[j] == (uint32_t)j;
    for (int e = 0; e < sh.ne; ++e) ok = ok && (t.o_e[e] & vmask) == 0;
    if (!ok) return fail(TSG_ERR_INVALID_ARGUMENT, "tile bounds: vector store not aligned");
  }
  uint32_t otab = 0, oe = 0;
  for (int j = 0; j < sh.v; ++j) otab = std::max(otab, t.o_tab[j]);
  for (int e = 0; e < sh.ne; ++e) oe = std::max(oe, t.o_e[e]);
  const uint64_t ohi = (la.cnt - 1) * (uint64_t)t.n_out + narrow_max(t.of_hi, nbits) +
                       narrow_max(t.of_lo, t.tile_bits, vbits) + otab + oe;
  if (ohi >= (uint64_t)c.lay->plane[s])
    return fail(TSG_ERR_INVALID_ARGUMENT, "tile bounds: output offset outside its buffer");
  return TSG_OK;
}

// The streaming kernel takes large steps whose E-free operand is an intermediate read
// as whole 1024-element tiles: its first 10 F bits are its own bits 0-9, every other
// offset term is a multiple of 1024 elements (so each chunk is contiguous and 16-byte
// aligned for TMA), and the tile kernel would use 256 threads x 4 positions.

// Bytes of one stage (one residue plane of one tile): the staged operand's tile per
// summed combination and, with span > 0, the other operand's blocks.
uint64_t stream_stage_bytes(int ne, int nk, uint32_t chunk_bytes, uint32_t span, uint32_t esize) {
  return (uint64_t)nk * chunk_bytes + (uint64_t)ne * nk * span * esize;
}

// Span of the staged chunks of the other operand of a streamed step, or 0 (plain loads).
// Per (plane, E combination, summed combination) the tile reads that operand at
// base + slot terms + tile terms + e_off + k_off + its within-tile offsets; the
// within-tile offsets stay below span = 2^b and every other term is a multiple of span,
// so one aligned block of span elements holds them all. The blocks must be whole 16-byte
// bulk copies, end inside the operand's buffer (`extent` elements per plane), and fit the
// shared-memory budget; leaves (uint8) are never staged.
uint32_t stream_span(const LaunchArgs& la, int np, uint32_t esize, uint64_t extent) {
  const TileArgs& t = la.t;
  const TileShape& sh = la.shape;
  const TileOperand& s = t.op[1 - la.stream.big];
  if (s.leaf) return 0;
  int b = bit_width(narrow_max(s.f_lo, kStreamTileBits));
  while ((1u << b) * esize < 16) b++;
  const uint32_t span = 1u << b;
  const uint64_t mask = span - 1;
  bool ok = (s.base & mask) == 0 && (s.plane & mask) == 0;
  for (int i = 0; i < s.g.n; ++i) ok = ok && s.g.dst[i] >= b;
  for (int i = 0; i < s.f_hi.n; ++i) ok = ok && s.f_hi.dst[i] >= b;
  uint32_t eo = 0, ko = 0;
  for (int e = 0; e < sh.ne; ++e) {
    ok = ok && (s.e_off[e] & mask) == 0;
    eo = std::max(eo, s.e_off[e]);
  }
  for (int kk = 0; kk < t.n_k; ++kk) {
    ok = ok && (s.k_off[kk] & mask) == 0;
    ko = std::max(ko, s.k_off[kk]);
  }
  const int gbits = bit_width(la.cnt - 1);
  const int nbits = bit_width(sh.tiles - 1) + t.tile_bits;
  const uint64_t end = s.base + scatter_max(s.g, gbits) + narrow_max(s.f_hi, nbits) + eo + ko + span;
  ok = ok && end <= extent;
  ok = ok && 2 * stream_stage_bytes(sh.ne, std::min(t.n_k, 4), la.stream.chunk_bytes, span, esize) <=
                 kStreamBlockSmem;
  return ok ? span : 0;
}

// With fused_big >= 0 the step is fused: operand fused_big (never stored) is the one the
// kernel would stage, the consumer warps compute it instead, and a stage holds only the
// other operand's blocks (which must then be stageable).
void choose_stream(LaunchArgs& la, int ring, int np, const uint64_t extent[2],
                   int fused_big = -1) {
  if (ring == TSG_RING_OR_AND) return;
  const TileArgs& t = la.t;
  const TileShape& sh = la.shape;
  // the streaming kernel stores 4 consecutive outputs as one vector: only when the 4
  // positions of a thread are 4 consecutive, aligned outputs
  // up to 16 summed combinations, at most 4 per stage (an item spans n_k / 4 stages)
  if (sh.v != 4 || t.n_k > 16 || t.tile_bits != kStreamTileBits || !t.o_contig)
    return;
  if (sh.tiles * la.cnt < (uint64_t)device_sm_count() * 8) return;  // too small to stream
  if (fused_big >= 0 && t.n_k > 4) return;
  int big = -1;
  for (int o = 0; o < 2; ++o) {
    const TileOperand& op = t.op[o];
    if (fused_big >= 0 && o != fused_big) continue;
    if (op.leaf || op.has_e) continue;
    if (op.f_lo.n != 1 || op.f_lo.src[0] != 0 || op.f_lo.dst[0] != 0 ||
        op.f_lo.len[0] != kStreamTileBits)
      continue;
    bool aligned = (op.base % kStreamTile) == 0 && (op.plane % kStreamTile) == 0;
    for (int i = 0; i < op.g.n; ++i) aligned = aligned && op.g.dst[i] >= kStreamTileBits;
    for (int i = 0; i < op.f_hi.n; ++i) aligned = aligned && op.f_hi.dst[i] >= kStreamTileBits;
    for (int kk = 0; kk < t.n_k; ++kk) aligned = aligned && (op.k_off[kk] % kStreamTile) == 0;
    if (aligned) {
      big = o;
      break;
    }
  }
  if (big < 0) return;
  const uint32_t esize = ring == TSG_RING_U64 ? 8 : 4;
  la.stream.big = big;
  la.stream.tiles = (uint32_t)sh.tiles;
  la.stream.work = sh.tiles * la.cnt;
  la.stream.chunk_bytes = kStreamTile * esize;
  la.stream.s_span = stream_span(la, np, esize, extent[1 - big]);
  if (fused_big >= 0 && la.stream.s_span == 0) return;
  const uint64_t stage = stream_stage_bytes(sh.ne, std::min(t.n_k, 4),
                                            fused_big >= 0 ? 0u : la.stream.chunk_bytes,
                                            la.stream.s_span, esize);
  if (2 * stage > kStreamBlockSmem) return;  // fewer than two stages fit
  la.stream.stage_bytes = (uint32_t)stage;
  la.stream.stages = (int)std::min<uint64_t>(kStreamMaxStages, kStreamBlockSmem / stage);
  la.stream.kchunks = t.n_k > 4 ? t.n_k / 4 : 1;
  la.streamed = true;
}

// Bounds of one operand read through a tile operand: the largest offset its terms can
// form (slot, tile, thread, V position, E, summed and extra terms) must stay inside
// [lo_ext, hi_ext), and a vector-read operand's terms must keep V-element alignment.
tsg_status check_operand_tile(const TileOperand& op, const TileArgs& t, const TileShape& sh,
                              uint64_t cnt, uint32_t extra_max,
                              const std::vector<uint32_t>& extra_terms, uint64_t lo_ext,
                              uint64_t hi_ext) {
  const int gbits = bit_width(cnt - 1);
  const int nbits = bit_width(sh.tiles - 1) + t.tile_bits;
  const int vbits = sh.v == 16 ? 4 : (sh.v == 4 ? 2 : 0);
  uint32_t tab = 0, eo = 0, ko = 0;
  for (int j = 0; j < sh.v; ++j) tab = std::max(tab, op.tab[j]);
  for (int e = 0; e < sh.ne; ++e) eo = std::max(eo, op.e_off[e]);
  for (int kk = 0; kk < t.n_k; ++kk) ko = std::max(ko, op.k_off[kk]);
  const uint64_t hi = op.base + scatter_max(op.g, gbits) + narrow_max(op.f_hi, nbits) +
                      narrow_max(op.f_lo, t.tile_bits, vbits) + tab + eo + ko + extra_max;
  if (op.base < lo_ext || hi >= hi_ext)
    return fail(TSG_ERR_INVALID_ARGUMENT, "fused bounds: operand offset outside its tensor");
  if (op.mode == kModeContig && sh.v > 1) {
    const uint32_t vmask = (uint32_t)sh.v - 1;
    bool good = (op.base & vmask) == 0 && (op.plane & vmask) == 0;
    for (int i = 0; i < op.g.n; ++i) good = good && op.g.dst[i] >= vbits;
    for (const NarrowMap* m : {&op.f_hi, &op.f_lo})
      for (int i = 0; i < m->n; ++i) good = good && !(m->dst[i] < vbits && m->src[i] >= vbits);
    for (int j = 0; j < sh.v; ++j) good = good && op.tab[j] == (uint32_t)j;
    for (int e = 0; e < sh.ne; ++e) good = good && (op.e_off[e] & vmask) == 0;
    for (int kk = 0; kk < t.n_k; ++kk) good = good && (op.k_off[kk] & vmask) == 0;
    for (uint32_t x : extra_terms) good = good && (x & vmask) == 0;
    if (!good) return fail(TSG_ERR_INVALID_ARGUMENT, "fused bounds: vector load not aligned");
  }
  if (op.mode == kModeDual && sh.v == 4) {
    bool good = (op.base & 1) == 0 && (op.plane & 1) == 0 && (op.tab[2] & 1) == 0 &&
                op.tab[1] == 1;
    for (int i = 0; i < op.g.n; ++i) good = good && op.g.dst[i] >= 1;
    for (const NarrowMap* m : {&op.f_hi, &op.f_lo})
      for (int i = 0; i < m->n; ++i) good = good && !(m->dst[i] < 1 && m->src[i] >= 1);
    for (int e = 0; e < sh.ne; ++e) good = good && (op.e_off[e] & 1) == 0;
    for (int kk = 0; kk < t.n_k; ++kk) good = good && (op.k_off[kk] & 1) == 0;
    for (uint32_t x : extra_terms) good = good && (x & 1) == 0;
    if (!good)
      return fail(TSG_ERR_INVALID_ARGUMENT, "fused bounds: paired vector load not aligned");
  }
  return TSG_OK;
}

// Fused form of consumer step s, whose operand P (the result of step p, never stored) is
// computed from p's operands A and B: their tile operands are built in s's index space by
// composing s's map onto P with p's maps onto A and B; p's summed bits become the extra
// offsets kp_off. Checks every offset on the host like the other launch forms.
tsg_status build_fused(const RunCtx& c, int s, int64_t base, const TileBits& tb,
                       LaunchArgs* la) {
  const tsg_plan* plan = c.plan;
  const StepInfo& st = plan->steps[s];
  const int p = c.lay->fused_from[s];
  const StepInfo& ps = plan->steps[p];
  int xo = -1;
  for (int o = 0; o < 2; ++o)
    if (st.op[o] == -p - 1) xo = o;
  const TileShape& sh = la->shape;
  if (xo < 0 || sh.v != 4 || (sh.nk != 1 && sh.nk != 2 && sh.nk != 4) || ps.k_bits > 1 ||
      la->t.op[xo].has_e)
    return fail(TSG_ERR_UNSUPPORTED, "plan_run: fused step outside the fused kernel");
  FusedArgs& f = la->f;
  std::memset(&f, 0, sizeof(f));
  f.fx = xo;
  la->nkp = 1 << ps.k_bits;
  for (int o = 0; o < 2; ++o) {
    const OperandDesc dp = describe_operand(c, ps, o, base);
    // A's bit of the consumer's output bit i: P bit j = st.pos[xo][i] is p's output bit j
    int pos[TSG_MAX_BITS];
    for (int i = 0; i < st.out_bits; ++i) {
      const int j = st.pos[xo][i];
      pos[i] = j >= 0 ? ps.pos[o][j] : -1;
    }
    OperandDesc dc;
    dc.base = dp.base;
    dc.ptr = dp.ptr;
    dc.plane = dp.plane;
    dc.leaf = dp.leaf;
    dc.gp = dp.gp;
    for (int m = 0; m < st.k_bits; ++m) {
      const int j = st.pos[xo][st.out_bits + m];
      if (j >= 0 && ps.pos[o][j] >= 0) dc.kp.push_back({m, ps.pos[o][j]});
    }
    bool ok = true;
    TSG_TRY(fill_tile_operand(f.op[o], pos, dc, dp.ptr, tb, la->t.tile_bits, sh.v,
                              la->t.n_k, c.ring, &ok));
    if (!ok || f.op[o].has_e)
      return fail(TSG_ERR_UNSUPPORTED, "plan_run: fused operand outside the tile kernel");
    std::vector<uint32_t> extra;
    uint32_t extra_max = 0;
    for (int kp = 0; kp < la->nkp; ++kp) {
      uint32_t off = 0;
      for (int m = 0; m < ps.k_bits; ++m) {
        const int q = ps.pos[o][ps.out_bits + m];
        if (q >= 0 && ((kp >> m) & 1)) off |= 1u << q;
      }
      f.kp_off[o][kp] = off;
      extra.push_back(off);
      extra_max = std::max(extra_max, off);
    }
    // paired loads need even producer offsets too; otherwise the operand is gathered
    if (f.op[o].mode == kModeDual)
      for (uint32_t x : extra)
        if (x & 1) f.op[o].mode = kModeGather;
    const int v = ps.op[o];
    const uint64_t lo_ext = dp.leaf ? (uint64_t)plan->leaves[v].offset : 0;
    const uint64_t hi_ext = dp.leaf ? lo_ext + (1ull << plan->leaves[v].rank) + c.leaf_extra
                                    : (uint64_t)c.lay->plane[-v - 1];
    TSG_TRY(check_operand_tile(f.op[o], la->t, sh, la->cnt, extra_max, extra, lo_ext, hi_ext));
  }
  la->t.op[xo].ptr = nullptr;  // P is never read
  la->fused = true;
  return TSG_OK;
}

// Fills the kernel arguments of step s for slices [base, base + cnt) (cnt == 1 and base
// ignored for slice-independent steps) and bounds-checks them.
tsg_status build_step(const RunCtx& c, int s, int64_t base, int64_t cnt, LaunchArgs* la) {
  const tsg_plan* plan = c.plan;
  const StepInfo& st = plan->steps[s];
  StepArgs& a = la->a;
  std::memset(&a, 0, sizeof(a));
  std::memset(&la->f, 0, sizeof(la->f));
  la->nkp = 0;
  la->cnt = (uint64_t)(c.dep(st) ? cnt : 1);
  a.total = la->cnt << st.out_bits;
  a.k_bits = st.k_bits;
  a.out = c.ws ? c.ws + c.lay->offset[s] : nullptr;
  a.o_plane = (uint64_t)c.lay->plane[s];
  OperandDesc d[2] = {describe_operand(c, st, 0, base), describe_operand(c, st, 1, base)};
  for (int o = 0; o < 2; ++o) {
    std::vector<std::pair<int, int>> tp = d[o].tp;
    for (const auto& pr : d[o].gp) tp.push_back({st.out_bits + pr.first, pr.second});
    TSG_TRY(make_bitmap(tp, o == 0 ? &a.lt : &a.rt));
    TSG_TRY(make_bitmap(d[o].kp, o == 0 ? &a.lk : &a.rk));
    (o == 0 ? a.lhs : a.rhs) = d[o].ptr;
    (o == 0 ? a.l_base : a.r_base) = d[o].base;
    (o == 0 ? a.l_plane : a.r_plane) = d[o].plane;
    la->is_leaf[o] = d[o].leaf;
  }
  TSG_TRY(check_step_bounds(c, s, a, la->is_leaf));
  bool ok = false;
  TileBits tb;
  // a fused consumer takes 4 positions per thread in every ring (the fused kernel's form)
  TSG_TRY(build_tile(st, d, a, la->cnt, c.ring, &la->t, &la->shape, &ok, &tb,
                     /*allow_v16=*/c.lay->fused_from[s] < 0));
  la->tile = ok;
  la->streamed = false;
  la->fused = false;
  if (ok) TSG_TRY(check_tile_bounds(c, s, *la));
  // MODP tile launches: every residue plane in one thread (the E-free operand of the next
  // plane prefetched) unless the step's options ask for one plane per block
  la->t.plane_split = (ok && c.ring == TSG_RING_MODP && c.ra.np > 1 &&
                       (step_option(plan, c.lay->elem_bytes, s) & TSG_STEP_PLANE_SPLIT)) ? 1 : 0;
  if (c.lay->fused_from[s] >= 0) {
    if (!ok)
      return fail(TSG_ERR_UNSUPPORTED, "plan_run: fused step outside the tile kernel");
    TSG_TRY(build_fused(c, s, base, tb, la));
    if (!(step_option(plan, c.lay->elem_bytes, s) & TSG_STEP_NO_STREAM)) {
      uint64_t extent[2];
      for (int o = 0; o < 2; ++o)
        extent[o] = la->is_leaf[o] ? 0 : (uint64_t)c.lay->plane[-st.op[o] - 1];
      choose_stream(*la, c.ring, c.ring == TSG_RING_MODP ? c.ra.np : 1, extent, la->f.fx);
    }
    return TSG_OK;
  }
  if (ok && !(step_option(plan, c.lay->elem_bytes, s) & TSG_STEP_NO_STREAM)) {
    uint64_t extent[2];
    for (int o = 0; o < 2; ++o)
      extent[o] = la->is_leaf[o] ? 0 : (uint64_t)c.lay->plane[-st.op[o] - 1];
    choose_stream(*la, c.ring, c.ring == TSG_RING_MODP ? c.ra.np : 1, extent);
  }
  return TSG_OK;
}

tsg_status launch_step(const RunCtx& c, int s, int64_t base, int64_t cnt) {
  LaunchArgs la;
  TSG_TRY(build_step(c, s, base, cnt, &la));
  if (la.streamed) {
    TSG_TRY(device_error_address(&la.stream.error));
    la.stream.wait_ns = g_wait_limit_ns.load(std::memory_order_relaxed);
    la.stream.stop_after = g_stall_after.load(std::memory_order_relaxed);
    if (la.fused) {
      if (c.ring == TSG_RING_U64) TSG_TRY(launch_stream_fused_u64(la, c.ra, c.stream));
      else TSG_TRY(launch_stream_fused_modp(la, c.ra, c.stream));
    } else if (c.ring == TSG_RING_U64) {
      TSG_TRY(launch_stream_u64(la, c.ra, c.stream));
    } else {
      TSG_TRY(launch_stream_modp(la, c.ra, c.stream));
    }
    TSG_CUDA_TRY(cudaGetLastError());
    return TSG_OK;
  }
  if (la.fused) {
    if (c.ring == TSG_RING_U64) TSG_TRY(launch_fused_u64(la, c.ra, c.stream));
    else if (c.ring == TSG_RING_OR_AND) TSG_TRY(launch_fused_or_and(la, c.ra, c.stream));
    else TSG_TRY(launch_fused_modp(la, c.ra, c.stream));
    TSG_CUDA_TRY(cudaGetLastError());
    return TSG_OK;
  }
  if (la.tile) {
    switch (c.ring) {
      case TSG_RING_OR_AND:
        TSG_TRY(launch_tile_or_and(la, c.ra, c.stream));
        break;
      case TSG_RING_U64:
        TSG_TRY(launch_tile_u64(la, c.ra, c.stream));
        break;
      default:
        TSG_TRY(launch_tile_modp(la, c.ra, c.stream));
        break;
    }
    TSG_CUDA_TRY(cudaGetLastError());
    return TSG_OK;
  }
  const StepArgs& a = la.a;
  switch (c.ring) {
    case TSG_RING_OR_AND:
      // every OR_AND operand is uint8, leaf or not
      if (use_sum_kernel(a)) launch_sum_t<TSG_RING_OR_AND, true, true>(a, c.ra, c.stream);
      else launch_step_t<TSG_RING_OR_AND, true, true>(a, c.ra, c.stream);
      break;
    case TSG_RING_U64:
      launch_step_ring<TSG_RING_U64>(la.is_leaf[0], la.is_leaf[1], a, c.ra, c.stream);
      break;
    default:
      launch_step_ring<TSG_RING_MODP>(la.is_leaf[0], la.is_leaf[1], a, c.ra, c.stream);
      break;
  }
  TSG_CUDA_TRY(cudaGetLastError());
  return TSG_OK;
}

tsg_status launch_reduce(const RunCtx& c, int64_t cnt, uint8_t* result, int accumulate,
                         int64_t slot0 = 0) {
  const tsg_plan* plan = c.plan;
  const int root = (int)plan->steps.size() - 1;
  const uint64_t entries = 1ull << plan->root_bits;
  // slots [slot0, slot0 + cnt) of the root (a variant's slices in a variant run)
  const uint8_t* rp = c.ws + c.lay->offset[root] + (uint64_t)slot0 * entries * c.lay->elem_bytes;
  const uint64_t plane = (uint64_t)c.lay->plane[root];
  unsigned blocks = (unsigned)std::min<uint64_t>(entries, (uint64_t)device_sm_count() * 8);
  switch (c.ring) {
    case TSG_RING_OR_AND:
      root_reduce_kernel<TSG_RING_OR_AND><<<blocks, kThreads, 0, c.stream>>>(
          rp, (uint64_t)cnt, entries, plane, result, accumulate, c.ra);
      break;
    case TSG_RING_U64:
      root_reduce_kernel<TSG_RING_U64><<<blocks, kThreads, 0, c.stream>>>(
          rp, (uint64_t)cnt, entries, plane, result, accumulate, c.ra);
      break;
    default:
      root_reduce_kernel<TSG_RING_MODP><<<blocks, kThreads, 0, c.stream>>>(
          rp, (uint64_t)cnt, entries, plane, result, accumulate, c.ra);
      break;
  }
  TSG_CUDA_TRY(cudaGetLastError());
  return TSG_OK;
}

bool is_pow2(int64_t x) { return x > 0 && (x & (x - 1)) == 0; }

tsg_status check_range(const tsg_plan* plan, int64_t slice_begin, int64_t slice_end,
                       int64_t group) {
  const int64_t nslices = int64_t(1) << plan->num_sliced;
  if (!is_pow2(group)) return fail(TSG_ERR_INVALID_ARGUMENT, "plan_run: group size must be a power of two");
  if (slice_begin < 0 || slice_end > nslices || slice_begin >= slice_end)
    return fail(TSG_ERR_INVALID_ARGUMENT, "plan_run: empty or out-of-range slice range");
  if (slice_begin % group != 0)
    return fail(TSG_ERR_INVALID_ARGUMENT, "plan_run: slice_begin must be a multiple of the group size");
  if (plan->num_sliced == 0 && group != 1)
    return fail(TSG_ERR_INVALID_ARGUMENT, "plan_run: unsliced plans run with group size 1");
  if (group > nslices) return fail(TSG_ERR_INVALID_ARGUMENT, "plan_run: group larger than the slice count");
  return TSG_OK;
}

}  // namespace
}  // namespace tsg

namespace tsg {
namespace {

// Per-launch device times of one run (tsg_plan_run_timed): an event is recorded on the
// run's stream before the first launch and after every launch; launch i took
// elapsed(ev[i], ev[i + 1]) and belongs to step ids[i] (num_steps: root reduction).
struct RunTimer {
  std::vector<cudaEvent_t> ev;
  std::vector<int> ids;
  ~RunTimer() {
    for (cudaEvent_t e : ev) cudaEventDestroy(e);
  }
  tsg_status record(cudaStream_t stream, int id) {
    cudaEvent_t e;
    TSG_CUDA_TRY(cudaEventCreate(&e));
    ev.push_back(e);
    if (id >= 0) ids.push_back(id);
    TSG_CUDA_TRY(cudaEventRecord(e, stream));
    return TSG_OK;
  }
  tsg_status collect(int num_steps, float* step_ms) {
    for (int s = 0; s <= num_steps; ++s) step_ms[s] = 0.f;
    if (ev.empty()) return TSG_OK;
    TSG_CUDA_TRY(cudaEventSynchronize(ev.back()));
    for (size_t i = 0; i + 1 < ev.size(); ++i) {
      float ms = 0.f;
      TSG_CUDA_TRY(cudaEventElapsedTime(&ms, ev[i], ev[i + 1]));
      step_ms[ids[i]] += ms;
    }
    return TSG_OK;
  }
};

// Kernel and template parameters of one built launch, as tsg_plan_describe reports them
// (the same selection as launch_step and the launch_tile_* / launch_stream_* switches).
void describe_launch(const LaunchArgs& la, int ring, int32_t* out) {
  if (la.fused) {
    out[0] = TSG_KERNEL_FUSED;
    out[1] = la.streamed ? 0 : la.shape.v;  // 0: the fused streaming kernel
    out[2] = la.shape.ne == 1 || la.shape.ne == 2 ? la.shape.ne : 4;
    out[3] = la.shape.nk;
  } else if (la.streamed) {
    const int nk = std::min(la.t.n_k, 4);
    out[0] = TSG_KERNEL_STREAM;
    out[1] = 0;
    out[2] = la.shape.ne == 1 || la.shape.ne == 2 ? la.shape.ne : 4;
    out[3] = nk == 1 || nk == 2 ? nk : 4;
  } else if (la.tile) {
    const int nk = la.shape.nk;
    out[0] = TSG_KERNEL_TILE;
    out[1] = la.shape.v;
    out[2] = la.shape.ne == 1 || la.shape.ne == 2 ? la.shape.ne : 4;
    out[3] = nk == 1 || nk == 2 ? nk : (nk == 4 && ring == TSG_RING_OR_AND ? 4 : 0);
  } else if (use_sum_kernel(la.a)) {
    out[0] = TSG_KERNEL_SUM;
    out[1] = out[2] = out[3] = 0;
  } else {
    out[0] = TSG_KERNEL_GENERAL;
    out[1] = out[2] = out[3] = 0;
  }
}

// Shared body of tsg_plan_run, tsg_plan_run_timed, tsg_plan_validate and
// tsg_plan_describe. With dry == true no pointer is dereferenced and nothing is launched:
// every launch's arguments are built and bounds-checked only (and, with `kinds`, each
// step's kernel of the first slice group is recorded). With a timer, every launch is
// followed by an event record.
// Leaf variants of one plan contracted together (tsg_plan_run_variants): `count` (a power
// of two) copies of the leaf pool, 2^stride_bits bytes apart; results `result_bytes` apart.
// Ring constants of a run: for MODP the moduli with their Barrett and Montgomery constants.
tsg_status make_ring_args(int32_t ring, int32_t num_primes, const uint32_t* primes,
                          RingArgs* out) {
  RingArgs& ra = *out;
  std::memset(&ra, 0, sizeof(ra));
  if (ring != TSG_RING_MODP) return TSG_OK;
  if (!primes) return fail(TSG_ERR_INVALID_ARGUMENT, "plan_run: MODP needs primes");
  ra.np = num_primes;
  for (int p = 0; p < num_primes; ++p) {
    if (primes[p] <= (1u << 31) - (1u << 26) || primes[p] >= (1u << 31) || (primes[p] % 2) == 0)
      return fail(TSG_ERR_INVALID_ARGUMENT,
                  "plan_run: moduli must be odd and in (2^31 - 2^26, 2^31)");
    ra.p[p] = primes[p];
    ra.m[p] = UINT64_MAX / primes[p];
    uint32_t inv = primes[p];  // Newton iteration for p^-1 mod 2^32 (5 steps: 2^32 bits)
    for (int it = 0; it < 5; ++it) inv *= 2u - primes[p] * inv;
    ra.pinv[p] = 0u - inv;
    ra.r1[p] = (uint32_t)((1ull << 32) % primes[p]);
  }
  return TSG_OK;
}

struct VariantSpec {
  int64_t count;
  int stride_bits;
  int64_t result_bytes;
};

tsg_status run_impl(const tsg_plan* plan, int32_t ring, int32_t num_primes,
                    const uint32_t* primes, const uint8_t* pool, int64_t slice_begin,
                    int64_t slice_end, int64_t group_size, void* workspace,
                    int64_t workspace_bytes, void* result_dev, int32_t accumulate,
                    cudaStream_t stream, bool dry, RunTimer* timer = nullptr,
                    int32_t* kinds = nullptr, const VariantSpec* vs = nullptr) {
  TSG_TRY(check_range(plan, slice_begin, slice_end, group_size));
  int64_t eb;
  int planes;
  TSG_TRY(elem_info(ring, num_primes, &eb, &planes));
  RingArgs ra;
  TSG_TRY(make_ring_args(ring, num_primes, primes, &ra));
  int v_bits = 0;
  if (vs) {
    while ((int64_t(1) << v_bits) < vs->count) v_bits++;
    if (int64_t(1) << v_bits != vs->count)
      return fail(TSG_ERR_INVALID_ARGUMENT, "plan_run_variants: the variant count must be a power of two");
  }
  const Layout* lay;
  TSG_TRY(get_layout(const_cast<tsg_plan*>(plan), group_size << v_bits, eb, planes, &lay,
                     vs != nullptr));
  if (!dry) {
    if (!workspace || workspace_bytes < lay->bytes)
      return fail(TSG_ERR_WORKSPACE, "plan_run: workspace smaller than tsg_plan_workspace_bytes");
    if (((uintptr_t)workspace & 255) != 0)
      return fail(TSG_ERR_WORKSPACE, "plan_run: workspace must be 256-byte aligned");
  }
  RunCtx c;
  c.plan = plan;
  c.lay = lay;
  c.ring = ring;
  c.ra = ra;
  c.pool = pool;
  c.ws = (uint8_t*)workspace;
  c.stream = stream;
  c.g_bits = 0;
  while ((int64_t(1) << c.g_bits) < group_size) c.g_bits++;
  if (vs) {
    c.all_dep = true;
    c.v_bits = v_bits;
    c.vstride_bits = vs->stride_bits;
    c.leaf_extra = ((uint64_t(1) << v_bits) - 1) << vs->stride_bits;
  }
  const int ns = (int)plan->steps.size();
  if (timer && !dry) TSG_TRY(timer->record(stream, -1));
  auto timed = [&](int id) -> tsg_status {
    return (timer && !dry) ? timer->record(stream, id) : TSG_OK;
  };
  auto step = [&](int s, int64_t base, int64_t cnt) -> tsg_status {
    if (lay->fused_away[s]) {  // computed inside its consumer: no launch
      if (dry && kinds) {
        kinds[4 * s] = TSG_KERNEL_NONE;
        kinds[4 * s + 1] = kinds[4 * s + 2] = kinds[4 * s + 3] = 0;
      }
      return TSG_OK;
    }
    if (dry) {
      LaunchArgs la;
      TSG_TRY(build_step(c, s, base, cnt, &la));
      if (kinds && (!c.dep(plan->steps[s]) || base == slice_begin))
        describe_launch(la, ring, kinds + 4 * s);
      return TSG_OK;
    }
    TSG_TRY(launch_step(c, s, base, cnt));
    return timed(s);
  };
  auto reduce = [&](int64_t cnt, uint8_t* result, int acc) -> tsg_status {
    if (dry) return TSG_OK;
    TSG_TRY(launch_reduce(c, cnt, result, acc));
    return timed(ns);
  };
  uint8_t* result = (uint8_t*)result_dev;
  if (vs) {
    // every step per slot (variant-major slots), then each variant's slices reduced into
    // its own result
    bool first = true;
    for (int64_t base = slice_begin; base < slice_end; base += group_size) {
      const int64_t cnt = std::min<int64_t>(group_size, slice_end - base);
      for (int s = 0; s < ns; ++s) TSG_TRY(step(s, base, group_size << v_bits));
      if (!dry) {
        for (int64_t v = 0; v < vs->count; ++v) {
          TSG_TRY(launch_reduce(c, cnt, result + v * vs->result_bytes,
                                first ? accumulate : 1, v * group_size));
          TSG_TRY(timed(ns));
        }
      }
      first = false;
    }
    return TSG_OK;
  }
  for (int s = 0; s < ns; ++s)
    if (!plan->steps[s].dep) TSG_TRY(step(s, 0, 1));
  if (!plan->steps.back().dep) return reduce(1, result, accumulate);
  bool first = true;
  for (int64_t base = slice_begin; base < slice_end; base += group_size) {
    const int64_t cnt = std::min<int64_t>(group_size, slice_end - base);
    for (int s = 0; s < ns; ++s)
      if (plan->steps[s].dep) TSG_TRY(step(s, base, cnt));
    TSG_TRY(reduce(cnt, result, first ? accumulate : 1));
    first = false;
  }
  return TSG_OK;
}

}  // namespace
}  // namespace tsg

namespace tsg {
namespace {

constexpr int kMaxLanes = 32;

// Lanes of a batched run (tsg_batch_run_lanes): instances are spread over `lanes`
// streams that fork from the caller's stream and join it again, so the small launches of
// different instances overlap on the GPU. Each lane has its own workspace region.

// Estimated work of one instance: index-space entries of every launch (slice-dependent
// steps once per slice).
double instance_cost(const tsg_plan* plan) {
  const double slices = std::ldexp(1.0, plan->num_sliced);
  double c = 0;
  for (const StepInfo& st : plan->steps)
    c += std::ldexp(1.0, st.out_bits + st.k_bits) * (st.dep ? slices : 1.0);
  return c;
}

// Lane of every instance: longest-processing-time-first over the estimated costs (ties by
// instance order), so the lanes finish at about the same time. Deterministic.
std::vector<int> assign_lanes(int32_t n, const tsg_plan* const* plans, int lanes) {
  std::vector<int> order(n);
  std::vector<double> cost(n);
  for (int i = 0; i < n; ++i) {
    order[i] = i;
    cost[i] = instance_cost(plans[i]);
  }
  std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return cost[a] > cost[b]; });
  std::vector<double> load(lanes, 0.0);
  std::vector<int> lane(n, 0);
  for (int i : order) {
    int best = 0;
    for (int l = 1; l < lanes; ++l)
      if (load[l] < load[best]) best = l;
    lane[i] = best;
    load[best] += cost[i];
  }
  return lane;
}

// Workspace region of each lane (256-byte aligned offsets) and the total.
tsg_status lane_regions(int32_t n, const tsg_plan* const* plans, int32_t ring,
                        int32_t num_primes, const int64_t* group_sizes, int lanes,
                        const std::vector<int>& lane, std::vector<int64_t>* offset,
                        std::vector<int64_t>* bytes, int64_t* total) {
  bytes->assign(lanes, 0);
  for (int i = 0; i < n; ++i) {
    int64_t b = 0;
    TSG_TRY(tsg_plan_workspace_bytes(plans[i], ring, num_primes, group_sizes[i], &b));
    (*bytes)[lane[i]] = std::max((*bytes)[lane[i]], b);
  }
  offset->assign(lanes, 0);
  int64_t off = 0;
  for (int l = 0; l < lanes; ++l) {
    (*offset)[l] = off;
    off += align256((*bytes)[l]);
  }
  *total = std::max<int64_t>(off, 256);
  return TSG_OK;
}

// Streams and events of the lanes, made once per host thread and device.
struct LaneSet {
  std::vector<cudaStream_t> streams;
  std::vector<cudaEvent_t> joins;
  cudaEvent_t fork = nullptr;
};

tsg_status lane_set(int lanes, LaneSet** out) {
  thread_local std::map<int, LaneSet> sets;
  int dev = 0;
  TSG_CUDA_TRY(cudaGetDevice(&dev));
  LaneSet& ls = sets[dev];
  if (!ls.fork) TSG_CUDA_TRY(cudaEventCreateWithFlags(&ls.fork, cudaEventDisableTiming));
  while ((int)ls.streams.size() < lanes) {
    cudaStream_t st;
    cudaEvent_t ev;
    TSG_CUDA_TRY(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
    TSG_CUDA_TRY(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
    ls.streams.push_back(st);
    ls.joins.push_back(ev);
  }
  *out = &ls;
  return TSG_OK;
}

// ------------------------------------------------------------------------------------
// Packed batches (tsg_batch_run_packed). The instances of a lane are grouped into packs
// whose workspaces fit side by side in the lane's region; a pack runs level by level: the
// small steps of one tree level of every member go into shared packed launches
// (tree_pack_kernel), the member's other steps follow as their own launches, and each
// member ends with its root reduction. An instance whose slices need several groups runs
// alone, step by step.

// The packed form of a launch, or false when the step is not small (more than
// 2^kPackTBits entries or 2^kPackKBits summed combinations) or runs on the streaming or
// fused kernel.
bool pack_item(const LaunchArgs& la, PackItem* it) {
  const StepArgs& a = la.a;
  if (la.streamed || la.fused) return false;
  if (a.total == 0 || (a.total & (a.total - 1)) != 0) return false;
  const int tb = bit_width(a.total - 1);
  if (tb > kPackTBits || a.k_bits < 0 || a.k_bits > kPackKBits) return false;
  std::memset(it, 0, sizeof(*it));
  for (int o = 0; o < 2; ++o) {
    PackOperand& op = it->op[o];
    const BitMap& tm = o == 0 ? a.lt : a.rt;
    const BitMap& km = o == 0 ? a.lk : a.rk;
    std::memset(op.tdst, kPackNone, sizeof(op.tdst));
    std::memset(op.kdst, kPackNone, sizeof(op.kdst));
    for (int r = 0; r < tm.n; ++r)
      for (int b = 0; b < tm.len[r]; ++b) {
        if (tm.src[r] + b >= tb) return false;
        op.tdst[tm.src[r] + b] = (uint8_t)(tm.dst[r] + b);
      }
    for (int r = 0; r < km.n; ++r)
      for (int b = 0; b < km.len[r]; ++b) {
        if (km.src[r] + b >= a.k_bits) return false;
        op.kdst[km.src[r] + b] = (uint8_t)(km.dst[r] + b);
      }
    op.ptr = o == 0 ? a.lhs : a.rhs;
    op.base = o == 0 ? a.l_base : a.r_base;
    op.plane = o == 0 ? a.l_plane : a.r_plane;
  }
  it->out = a.out;
  it->o_plane = a.o_plane;
  it->t_bits = (uint8_t)tb;
  it->k_bits = (uint8_t)a.k_bits;
  it->leaves = (uint8_t)((la.is_leaf[0] ? 1 : 0) | (la.is_leaf[1] ? 2 : 0));
  return true;
}

struct PackMember {
  const tsg_plan* plan;
  const uint8_t* pool;
  uint8_t* ws;
  void* result;
  int64_t group;  // every slice of the instance
};

// Runs one pack (dry: builds and checks every launch, issues none) and adds its launch
// count to *launches.
tsg_status run_pack(const std::vector<PackMember>& mem, int32_t ring, const RingArgs& ra,
                    int64_t eb, int planes, cudaStream_t stream, bool dry, int64_t* launches) {
  const int n = (int)mem.size();
  std::vector<RunCtx> ctx(n);
  int max_level = 0;
  for (int i = 0; i < n; ++i) {
    const Layout* lay;
    TSG_TRY(get_layout(const_cast<tsg_plan*>(mem[i].plan), mem[i].group, eb, planes, &lay,
                       /*all_dep=*/false, /*levels=*/true));
    RunCtx& c = ctx[i];
    c.plan = mem[i].plan;
    c.lay = lay;
    c.ring = ring;
    c.ra = ra;
    c.pool = mem[i].pool;
    c.ws = mem[i].ws;
    c.stream = stream;
    c.g_bits = 0;
    while ((int64_t(1) << c.g_bits) < mem[i].group) c.g_bits++;
    for (int l : lay->level) max_level = std::max(max_level, l);
  }
  std::unique_ptr<PackArgs> pa(new PackArgs);
  pa->n_items = 0;
  pa->n_warps = 0;
  int64_t count = 0;
  auto flush = [&]() -> tsg_status {
    if (pa->n_items == 0) return TSG_OK;
    if (!dry) TSG_TRY(launch_pack(ring, *pa, ra, stream));
    count++;
    pa->n_items = 0;
    pa->n_warps = 0;
    return TSG_OK;
  };
  std::vector<std::pair<int, int>> singles;
  for (int l = 1; l <= max_level; ++l) {
    singles.clear();
    for (int i = 0; i < n; ++i) {
      const RunCtx& c = ctx[i];
      const int ns = (int)c.plan->steps.size();
      for (int s = 0; s < ns; ++s) {
        if (c.lay->level[s] != l || c.lay->fused_away[s]) continue;
        LaunchArgs la;
        TSG_TRY(build_step(c, s, 0, mem[i].group, &la));
        PackItem& it = pa->items[pa->n_items];
        if (!pack_item(la, &it)) {
          singles.push_back({i, s});
          continue;
        }
        it.warp0 = pa->n_warps;
        pa->n_warps += (uint32_t)((la.a.total + 31) / 32);
        if (++pa->n_items == kPackItems) TSG_TRY(flush());
      }
    }
    TSG_TRY(flush());
    for (const auto& is : singles) {
      if (!dry) TSG_TRY(launch_step(ctx[is.first], is.second, 0, mem[is.first].group));
      count++;
    }
  }
  for (int i = 0; i < n; ++i) {
    const int64_t cnt = ctx[i].plan->steps.back().dep ? mem[i].group : 1;
    if (!dry) TSG_TRY(launch_reduce(ctx[i], cnt, (uint8_t*)mem[i].result, 0));
    count++;
  }
  if (launches) *launches += count;
  return TSG_OK;
}

// Lanes, packs and workspace regions of a packed batch.
struct PackSchedule {
  int used = 1;
  std::vector<int> lane;                              // lane of every instance
  std::vector<std::vector<std::vector<int>>> packs;  // per lane, its packs in run order
  std::vector<char> packed;        // the instance runs in a pack (one group of all slices)
  std::vector<int64_t> inst_off;   // workspace offset of the instance in its lane's region
  std::vector<int64_t> inst_bytes;
  std::vector<int64_t> lane_off, lane_bytes;
  int64_t total = 0;
};

// Lanes by estimated cost (assign_lanes); each lane's region holds its largest instance;
// the lane's instances, largest workspace first, fill packs first-fit within the region.
tsg_status plan_packs(int32_t n, const tsg_plan* const* plans, int32_t ring,
                      int32_t num_primes, const int64_t* group_sizes, int lanes,
                      PackSchedule* ps) {
  int64_t eb;
  int planes;
  TSG_TRY(elem_info(ring, num_primes, &eb, &planes));
  ps->used = std::max(1, std::min<int>(lanes, n));
  ps->lane = assign_lanes(n, plans, ps->used);
  ps->packed.assign(n, 0);
  ps->inst_off.assign(n, 0);
  ps->inst_bytes.assign(n, 0);
  for (int i = 0; i < n; ++i) {
    const int64_t ns = int64_t(1) << plans[i]->num_sliced;
    TSG_TRY(check_range(plans[i], 0, ns, group_sizes[i]));
    if (group_sizes[i] == ns) {
      const Layout* lay;
      TSG_TRY(get_layout(const_cast<tsg_plan*>(plans[i]), ns, eb, planes, &lay, false, true));
      ps->inst_bytes[i] = align256(lay->bytes);
      ps->packed[i] = 1;
    } else {
      int64_t b = 0;
      TSG_TRY(tsg_plan_workspace_bytes(plans[i], ring, num_primes, group_sizes[i], &b));
      ps->inst_bytes[i] = align256(b);
    }
  }
  ps->lane_bytes.assign(ps->used, 0);
  for (int i = 0; i < n; ++i)
    ps->lane_bytes[ps->lane[i]] = std::max(ps->lane_bytes[ps->lane[i]], ps->inst_bytes[i]);
  ps->packs.assign(ps->used, {});
  for (int l = 0; l < ps->used; ++l) {
    std::vector<int> order;
    for (int i = 0; i < n; ++i)
      if (ps->lane[i] == l) order.push_back(i);
    std::stable_sort(order.begin(), order.end(),
                     [&](int a, int b) { return ps->inst_bytes[a] > ps->inst_bytes[b]; });
    std::vector<int> cur;
    int64_t used_bytes = 0;
    for (int i : order) {
      if (!ps->packed[i]) {
        ps->packs[l].push_back({i});
        continue;
      }
      if (!cur.empty() && used_bytes + ps->inst_bytes[i] > ps->lane_bytes[l]) {
        ps->packs[l].push_back(cur);
        cur.clear();
        used_bytes = 0;
      }
      ps->inst_off[i] = used_bytes;
      used_bytes += ps->inst_bytes[i];
      cur.push_back(i);
    }
    if (!cur.empty()) ps->packs[l].push_back(cur);
  }
  ps->lane_off.assign(ps->used, 0);
  int64_t off = 0;
  for (int l = 0; l < ps->used; ++l) {
    ps->lane_off[l] = off;
    off += align256(ps->lane_bytes[l]);
  }
  ps->total = std::max<int64_t>(off, 256);
  return TSG_OK;
}

// Scratch memory of tsg_plan_run_static: a fixed 64 MiB array in device global memory,
// owned by this library, held by every GPU that loads it until the process exits. Host
// code cannot use the array's name as a device address; the address comes from
// cudaGetSymbolAddress, resolved once per device (with that device current) on the first
// call and cached.
constexpr int64_t kStaticScratchBytes = int64_t(64) << 20;
static __device__ __align__(256) uint8_t g_static_scratch[kStaticScratchBytes];

std::mutex g_static_scratch_mu;
void* g_static_scratch_ptr[64] = {};

tsg_status static_scratch_address(void** out) {
  int dev = 0;
  TSG_CUDA_TRY(cudaGetDevice(&dev));
  if (dev < 0 || dev >= 64)
    return fail(TSG_ERR_UNSUPPORTED, "plan_run_static: device ordinal outside 0..63");
  std::lock_guard<std::mutex> lock(g_static_scratch_mu);
  if (g_static_scratch_ptr[dev] == nullptr) {
    void* ptr = nullptr;
    const cudaError_t err = cudaGetSymbolAddress(&ptr, g_static_scratch);
    if (err != cudaSuccess) return cuda_status(err, "cudaGetSymbolAddress(static scratch)");
    g_static_scratch_ptr[dev] = ptr;
  }
  *out = g_static_scratch_ptr[dev];
  return TSG_OK;
}

}  // namespace
}  // namespace tsg

using namespace tsg;

extern "C" {

tsg_status tsg_plan_create(int32_t num_leaves, const int32_t* leaf_ranks,
                           const int64_t* leaf_offsets, int32_t num_sliced,
                           const int32_t* leaf_slice_pos, int32_t num_steps,
                           const int32_t* step_operands, const int32_t* step_out_bits,
                           const int32_t* step_sum_bits, const int32_t* step_lhs_pos,
                           const int32_t* step_rhs_pos, tsg_plan** plan_out) {
  if (!plan_out) return fail(TSG_ERR_INVALID_ARGUMENT, "plan_create: null output pointer");
  *plan_out = nullptr;
  if (num_leaves < 1 || num_steps < 1 || num_steps != num_leaves - 1)
    return fail(TSG_ERR_INVALID_ARGUMENT, "plan_create: a tree over L leaves has L-1 steps (L >= 2)");
  if (num_sliced < 0 || num_sliced > 62)
    return fail(TSG_ERR_INVALID_ARGUMENT, "plan_create: sliced wires must number 0..62");
  if (!leaf_ranks || !leaf_offsets || (num_sliced > 0 && !leaf_slice_pos) || !step_operands ||
      !step_out_bits || !step_sum_bits || !step_lhs_pos || !step_rhs_pos)
    return fail(TSG_ERR_INVALID_ARGUMENT, "plan_create: null array");
  tsg_plan* plan = new tsg_plan();
  auto bad = [&](tsg_status code, const std::string& msg) {
    delete plan;
    return fail(code, msg);
  };
  plan->num_sliced = num_sliced;
  plan->leaves.resize(num_leaves);
  std::vector<int> sliced_seen(num_sliced, 0);
  for (int l = 0; l < num_leaves; ++l) {
    LeafInfo& lf = plan->leaves[l];
    lf.rank = leaf_ranks[l];
    lf.offset = leaf_offsets[l];
    if (lf.rank < 0 || lf.rank > TSG_MAX_BITS || lf.offset < 0)
      return bad(TSG_ERR_INVALID_ARGUMENT, "plan_create: leaf rank or offset out of range");
    lf.spos.assign(num_sliced, -1);
    lf.dep = false;
    for (int j = 0; j < num_sliced; ++j) {
      const int p = leaf_slice_pos[(int64_t)l * num_sliced + j];
      if (p < -1 || p >= lf.rank)
        return bad(TSG_ERR_INVALID_ARGUMENT, "plan_create: sliced bit position outside the leaf");
      lf.spos[j] = p;
      if (p >= 0) {
        lf.dep = true;
        sliced_seen[j] = 1;
      }
    }
  }
  for (int j = 0; j < num_sliced; ++j)
    if (!sliced_seen[j])
      return bad(TSG_ERR_INVALID_ARGUMENT, "plan_create: a sliced wire appears in no leaf");
  std::vector<int> leaf_uses(num_leaves, 0), step_uses(num_steps, 0);
  plan->steps.resize(num_steps);
  for (int s = 0; s < num_steps; ++s) {
    StepInfo& st = plan->steps[s];
    st.out_bits = step_out_bits[s];
    st.k_bits = step_sum_bits[s];
    if (st.out_bits < 0 || st.k_bits < 0 || st.out_bits + st.k_bits > TSG_MAX_BITS)
      return bad(TSG_ERR_INVALID_ARGUMENT, "plan_create: step index space exceeds 62 bits");
    for (int o = 0; o < 2; ++o) {
      const int v = step_operands[2 * s + o];
      st.op[o] = v;
      if (v >= 0) {
        if (v >= num_leaves) return bad(TSG_ERR_INVALID_ARGUMENT, "plan_create: leaf id out of range");
        leaf_uses[v]++;
      } else {
        const int x = -v - 1;
        if (x >= s) return bad(TSG_ERR_INVALID_ARGUMENT, "plan_create: step reads a later step");
        step_uses[x]++;
      }
      const int32_t* pos = (o == 0 ? step_lhs_pos : step_rhs_pos) + (int64_t)s * TSG_MAX_BITS;
      const int rank = operand_rank(plan->leaves, plan->steps, v);
      // every bit of the operand must be an output bit, a summed bit or a sliced bit
      std::vector<int> cover(rank, 0);
      for (int i = 0; i < st.out_bits + st.k_bits; ++i) {
        const int p = pos[i];
        st.pos[o][i] = p;
        if (p < -1 || p >= rank)
          return bad(TSG_ERR_INVALID_ARGUMENT, "plan_create: bit position outside the operand");
        if (p >= 0) {
          if (cover[p]) return bad(TSG_ERR_INVALID_ARGUMENT, "plan_create: operand bit mapped twice");
          cover[p] = 1;
        }
      }
      for (int i = st.out_bits + st.k_bits; i < TSG_MAX_BITS; ++i) st.pos[o][i] = -1;
      if (v >= 0) {
        for (int j = 0; j < num_sliced; ++j) {
          const int p = plan->leaves[v].spos[j];
          if (p < 0) continue;
          if (cover[p]) return bad(TSG_ERR_INVALID_ARGUMENT, "plan_create: sliced bit also indexed");
          cover[p] = 1;
        }
      }
      for (int b = 0; b < rank; ++b)
        if (!cover[b]) return bad(TSG_ERR_INVALID_ARGUMENT, "plan_create: operand bit not covered");
    }
    // every summed bit must be carried by at least one operand, every output bit too
    for (int i = 0; i < st.out_bits + st.k_bits; ++i)
      if (st.pos[0][i] < 0 && st.pos[1][i] < 0)
        return bad(TSG_ERR_INVALID_ARGUMENT, "plan_create: index bit carried by neither operand");
    st.dep = operand_dep(plan->leaves, plan->steps, st.op[0]) ||
             operand_dep(plan->leaves, plan->steps, st.op[1]);
  }
  for (int l = 0; l < num_leaves; ++l)
    if (leaf_uses[l] != 1) return bad(TSG_ERR_INVALID_ARGUMENT, "plan_create: each leaf is used once");
  for (int s = 0; s + 1 < num_steps; ++s)
    if (step_uses[s] != 1)
      return bad(TSG_ERR_INVALID_ARGUMENT, "plan_create: each non-root step is consumed once");
  if (step_uses[num_steps - 1] != 0)
    return bad(TSG_ERR_INVALID_ARGUMENT, "plan_create: the root step must not be consumed");
  plan->root_bits = plan->steps.back().out_bits;
  *plan_out = plan;
  return TSG_OK;
}

void tsg_plan_destroy(tsg_plan* plan) { delete plan; }

tsg_status tsg_plan_root_bits(const tsg_plan* plan, int32_t* bits_out) {
  if (!plan || !bits_out) return fail(TSG_ERR_INVALID_ARGUMENT, "plan_root_bits: null pointer");
  *bits_out = plan->root_bits;
  return TSG_OK;
}

tsg_status tsg_plan_workspace_bytes(const tsg_plan* plan, int32_t ring, int32_t num_primes,
                                    int64_t group_size, int64_t* bytes_out) {
  if (!plan || !bytes_out) return fail(TSG_ERR_INVALID_ARGUMENT, "workspace_bytes: null pointer");
  if (!is_pow2(group_size)) return fail(TSG_ERR_INVALID_ARGUMENT, "workspace_bytes: group must be a power of two");
  int64_t eb;
  int planes;
  TSG_TRY(elem_info(ring, num_primes, &eb, &planes));
  const Layout* lay;
  TSG_TRY(get_layout(const_cast<tsg_plan*>(plan), group_size, eb, planes, &lay));
  *bytes_out = lay->bytes;
  return TSG_OK;
}

tsg_status tsg_plan_launch_count(const tsg_plan* plan, int64_t slice_begin, int64_t slice_end,
                                 int64_t group_size, int64_t* count_out) {
  if (!plan || !count_out) return fail(TSG_ERR_INVALID_ARGUMENT, "launch_count: null pointer");
  TSG_TRY(check_range(plan, slice_begin, slice_end, group_size));
  int64_t indep = 0, dep = 0;
  for (const auto& s : plan->steps) (s.dep ? dep : indep)++;
  const int64_t groups = (slice_end - slice_begin + group_size - 1) / group_size;
  *count_out = plan->steps.back().dep ? indep + groups * (dep + 1) : indep + 1;
  return TSG_OK;
}

tsg_status tsg_plan_launches(const tsg_plan* plan, int32_t ring, int32_t num_primes,
                             int64_t slice_begin, int64_t slice_end, int64_t group_size,
                             int64_t* count_out) {
  if (!plan || !count_out) return fail(TSG_ERR_INVALID_ARGUMENT, "launches: null pointer");
  TSG_TRY(check_range(plan, slice_begin, slice_end, group_size));
  int64_t eb;
  int planes;
  TSG_TRY(elem_info(ring, num_primes, &eb, &planes));
  const Layout* lay;
  TSG_TRY(get_layout(const_cast<tsg_plan*>(plan), group_size, eb, planes, &lay));
  int64_t indep = 0, dep = 0;
  for (size_t s = 0; s < plan->steps.size(); ++s)
    if (!lay->fused_away[s]) (plan->steps[s].dep ? dep : indep)++;
  const int64_t groups = (slice_end - slice_begin + group_size - 1) / group_size;
  *count_out = plan->steps.back().dep ? indep + groups * (dep + 1) : indep + 1;
  return TSG_OK;
}

tsg_status tsg_plan_set_step_options(tsg_plan* plan, int32_t ring, const int32_t* options) {
  if (!plan) return fail(TSG_ERR_INVALID_ARGUMENT, "set_step_options: null plan");
  if (ring != TSG_RING_OR_AND && ring != TSG_RING_MODP && ring != TSG_RING_U64)
    return fail(TSG_ERR_INVALID_ARGUMENT, "set_step_options: unknown ring");
  const size_t ns = plan->steps.size();
  if (options) {
    for (size_t i = 0; i < ns; ++i)
      if (options[i] & ~(TSG_STEP_NO_STREAM | TSG_STEP_NO_FUSE | TSG_STEP_FUSE |
                         TSG_STEP_PLANE_SPLIT))
        return fail(TSG_ERR_INVALID_ARGUMENT, "set_step_options: unknown option bit");
    plan->options[ring].assign(options, options + ns);
  } else {
    plan->options[ring].clear();
  }
  // layouts depend on the fusion choices: drop the cached ones of this ring
  const int64_t eb = ring == TSG_RING_OR_AND ? 1 : (ring == TSG_RING_U64 ? 8 : 4);
  plan->layouts.erase(std::remove_if(plan->layouts.begin(), plan->layouts.end(),
                                     [&](const Layout& l) { return l.elem_bytes == eb; }),
                      plan->layouts.end());
  return TSG_OK;
}

tsg_status tsg_plan_variants_workspace_bytes(const tsg_plan* plan, int32_t ring,
                                             int32_t num_primes, int64_t group_size,
                                             int64_t num_variants, int64_t* bytes_out) {
  if (!plan || !bytes_out)
    return fail(TSG_ERR_INVALID_ARGUMENT, "variants_workspace_bytes: null pointer");
  if (!is_pow2(group_size) || !is_pow2(num_variants))
    return fail(TSG_ERR_INVALID_ARGUMENT,
                "variants_workspace_bytes: group and variant count must be powers of two");
  int64_t eb;
  int planes;
  TSG_TRY(elem_info(ring, num_primes, &eb, &planes));
  const Layout* lay;
  TSG_TRY(get_layout(const_cast<tsg_plan*>(plan), group_size * num_variants, eb, planes, &lay,
                     /*all_dep=*/true));
  *bytes_out = lay->bytes;
  return TSG_OK;
}

tsg_status tsg_plan_run_variants(const tsg_plan* plan, int32_t ring, int32_t num_primes,
                                 const uint32_t* primes, const uint8_t* leaf_pools_dev,
                                 int64_t pool_stride, int64_t num_variants, int64_t group_size,
                                 void* workspace_dev, int64_t workspace_bytes,
                                 void* results_dev, int32_t accumulate, void* stream) {
  if (!plan || !leaf_pools_dev || !results_dev)
    return fail(TSG_ERR_INVALID_ARGUMENT, "plan_run_variants: null pointer");
  if (!is_pow2(num_variants) || !is_pow2(pool_stride) || pool_stride < 16)
    return fail(TSG_ERR_INVALID_ARGUMENT,
                "plan_run_variants: variant count and pool stride must be powers of two "
                "(stride >= 16 bytes)");
  int64_t pool_end = 0;
  for (const LeafInfo& lf : plan->leaves)
    pool_end = std::max<int64_t>(pool_end, lf.offset + (int64_t(1) << lf.rank));
  if (pool_stride < pool_end)
    return fail(TSG_ERR_INVALID_ARGUMENT, "plan_run_variants: pool stride smaller than one pool");
  int64_t eb;
  int planes;
  TSG_TRY(elem_info(ring, num_primes, &eb, &planes));
  VariantSpec vs;
  vs.count = num_variants;
  vs.stride_bits = 0;
  while ((int64_t(1) << vs.stride_bits) < pool_stride) vs.stride_bits++;
  vs.result_bytes = (int64_t(1) << plan->root_bits) * eb * planes;
  const int64_t ns = int64_t(1) << plan->num_sliced;
  // every launch is built and bounds-checked on the host before the first one is issued
  TSG_TRY(run_impl(plan, ring, num_primes, primes, nullptr, 0, ns, group_size, nullptr, 0,
                   nullptr, 0, nullptr, /*dry=*/true, nullptr, nullptr, &vs));
  return run_impl(plan, ring, num_primes, primes, leaf_pools_dev, 0, ns, group_size,
                  workspace_dev, workspace_bytes, results_dev, accumulate,
                  (cudaStream_t)stream, /*dry=*/false, nullptr, nullptr, &vs);
}

tsg_status tsg_set_fusion(int32_t enabled) {
  g_fusion.store(enabled ? 1 : 0, std::memory_order_relaxed);
  return TSG_OK;
}

int32_t tsg_fusion_enabled(void) { return g_fusion.load(std::memory_order_relaxed); }

tsg_status tsg_plan_run(const tsg_plan* plan, int32_t ring, int32_t num_primes,
                        const uint32_t* primes, const uint8_t* leaf_pool_dev,
                        int64_t slice_begin, int64_t slice_end, int64_t group_size,
                        void* workspace_dev, int64_t workspace_bytes, void* result_dev,
                        int32_t accumulate, void* stream) {
  if (!plan || !leaf_pool_dev || !result_dev)
    return fail(TSG_ERR_INVALID_ARGUMENT, "plan_run: null pointer");
  return run_impl(plan, ring, num_primes, primes, leaf_pool_dev, slice_begin, slice_end,
                  group_size, workspace_dev, workspace_bytes, result_dev, accumulate,
                  (cudaStream_t)stream, /*dry=*/false);
}

tsg_status tsg_plan_run_timed(const tsg_plan* plan, int32_t ring, int32_t num_primes,
                              const uint32_t* primes, const uint8_t* leaf_pool_dev,
                              int64_t slice_begin, int64_t slice_end, int64_t group_size,
                              void* workspace_dev, int64_t workspace_bytes, void* result_dev,
                              int32_t accumulate, void* stream, float* step_ms) {
  if (!plan || !leaf_pool_dev || !result_dev || !step_ms)
    return fail(TSG_ERR_INVALID_ARGUMENT, "plan_run_timed: null pointer");
  RunTimer timer;
  TSG_TRY(run_impl(plan, ring, num_primes, primes, leaf_pool_dev, slice_begin, slice_end,
                   group_size, workspace_dev, workspace_bytes, result_dev, accumulate,
                   (cudaStream_t)stream, /*dry=*/false, &timer));
  return timer.collect((int)plan->steps.size(), step_ms);
}

tsg_status tsg_plan_validate(const tsg_plan* plan, int32_t ring, int32_t num_primes,
                             const uint32_t* primes, int64_t slice_begin, int64_t slice_end,
                             int64_t group_size) {
  if (!plan) return fail(TSG_ERR_INVALID_ARGUMENT, "plan_validate: null plan");
  return run_impl(plan, ring, num_primes, primes, nullptr, slice_begin, slice_end, group_size,
                  nullptr, 0, nullptr, 0, nullptr, /*dry=*/true);
}

tsg_status tsg_plan_describe(const tsg_plan* plan, int32_t ring, int32_t num_primes,
                             const uint32_t* primes, int64_t group_size, int32_t* kinds) {
  if (!plan || !kinds) return fail(TSG_ERR_INVALID_ARGUMENT, "plan_describe: null pointer");
  const int64_t slices = int64_t(1) << plan->num_sliced;
  if (group_size < 1 || group_size > slices)
    return fail(TSG_ERR_INVALID_ARGUMENT, "plan_describe: group_size outside [1, slices]");
  return run_impl(plan, ring, num_primes, primes, nullptr, 0, group_size, group_size,
                  nullptr, 0, nullptr, 0, nullptr, /*dry=*/true, nullptr, kinds);
}

tsg_status tsg_batch_workspace_bytes(int32_t num_instances, const tsg_plan* const* plans,
                                     int32_t ring, int32_t num_primes,
                                     const int64_t* group_sizes, int64_t* bytes_out) {
  if (num_instances < 0 || (num_instances > 0 && (!plans || !group_sizes)) || !bytes_out)
    return fail(TSG_ERR_INVALID_ARGUMENT, "batch_workspace_bytes: null pointer or negative count");
  int64_t most = 0;
  for (int32_t i = 0; i < num_instances; ++i) {
    if (!plans[i]) return fail(TSG_ERR_INVALID_ARGUMENT, "batch_workspace_bytes: null plan");
    int64_t b = 0;
    TSG_TRY(tsg_plan_workspace_bytes(plans[i], ring, num_primes, group_sizes[i], &b));
    most = std::max(most, b);
  }
  *bytes_out = most;
  return TSG_OK;
}

tsg_status tsg_batch_run(int32_t num_instances, const tsg_plan* const* plans, int32_t ring,
                         int32_t num_primes, const uint32_t* primes,
                         const uint8_t* const* leaf_pools, const int64_t* group_sizes,
                         void* workspace_dev, int64_t workspace_bytes, void* const* results_dev,
                         void* stream) {
  if (num_instances < 0 ||
      (num_instances > 0 && (!plans || !leaf_pools || !group_sizes || !results_dev)))
    return fail(TSG_ERR_INVALID_ARGUMENT, "batch_run: null pointer or negative count");
  // every instance is checked (arguments, bounds of every launch) before anything runs
  for (int32_t i = 0; i < num_instances; ++i) {
    if (!plans[i] || !leaf_pools[i] || !results_dev[i])
      return fail(TSG_ERR_INVALID_ARGUMENT,
                  "batch_run: null plan, pool or result of instance " + std::to_string(i));
    const int64_t ns = int64_t(1) << plans[i]->num_sliced;
    tsg_status st = run_impl(plans[i], ring, num_primes, primes, nullptr, 0, ns,
                             group_sizes[i], nullptr, 0, nullptr, 0, nullptr, /*dry=*/true);
    if (st != TSG_OK)
      return fail(st, "batch_run: instance " + std::to_string(i) + ": " + tsg_last_error());
  }
  for (int32_t i = 0; i < num_instances; ++i) {
    const int64_t ns = int64_t(1) << plans[i]->num_sliced;
    TSG_TRY(run_impl(plans[i], ring, num_primes, primes, leaf_pools[i], 0, ns, group_sizes[i],
                     workspace_dev, workspace_bytes, results_dev[i], 0, (cudaStream_t)stream,
                     /*dry=*/false));
  }
  return TSG_OK;
}

tsg_status tsg_batch_lanes_workspace_bytes(int32_t num_instances, const tsg_plan* const* plans,
                                           int32_t ring, int32_t num_primes,
                                           const int64_t* group_sizes, int32_t lanes,
                                           int64_t* bytes_out) {
  if (num_instances < 0 || (num_instances > 0 && (!plans || !group_sizes)) || !bytes_out)
    return fail(TSG_ERR_INVALID_ARGUMENT, "batch_lanes_workspace_bytes: null pointer or negative count");
  if (lanes < 1 || lanes > kMaxLanes)
    return fail(TSG_ERR_INVALID_ARGUMENT, "batch_lanes_workspace_bytes: lanes outside 1..32");
  for (int32_t i = 0; i < num_instances; ++i)
    if (!plans[i]) return fail(TSG_ERR_INVALID_ARGUMENT, "batch_lanes_workspace_bytes: null plan");
  const int used = std::max(1, std::min<int>(lanes, num_instances));
  const std::vector<int> lane = assign_lanes(num_instances, plans, used);
  std::vector<int64_t> off, bytes;
  return lane_regions(num_instances, plans, ring, num_primes, group_sizes, used, lane, &off,
                      &bytes, bytes_out);
}

tsg_status tsg_batch_run_lanes(int32_t num_instances, const tsg_plan* const* plans,
                               int32_t ring, int32_t num_primes, const uint32_t* primes,
                               const uint8_t* const* leaf_pools, const int64_t* group_sizes,
                               int32_t lanes, void* workspace_dev, int64_t workspace_bytes,
                               void* const* results_dev, void* stream) {
  if (num_instances < 0 ||
      (num_instances > 0 && (!plans || !leaf_pools || !group_sizes || !results_dev)))
    return fail(TSG_ERR_INVALID_ARGUMENT, "batch_run_lanes: null pointer or negative count");
  if (lanes < 1 || lanes > kMaxLanes)
    return fail(TSG_ERR_INVALID_ARGUMENT, "batch_run_lanes: lanes outside 1..32");
  if (num_instances == 0) return TSG_OK;
  for (int32_t i = 0; i < num_instances; ++i) {
    if (!plans[i] || !leaf_pools[i] || !results_dev[i])
      return fail(TSG_ERR_INVALID_ARGUMENT,
                  "batch_run_lanes: null plan, pool or result of instance " + std::to_string(i));
    const int64_t ns = int64_t(1) << plans[i]->num_sliced;
    tsg_status st = run_impl(plans[i], ring, num_primes, primes, nullptr, 0, ns,
                             group_sizes[i], nullptr, 0, nullptr, 0, nullptr, /*dry=*/true);
    if (st != TSG_OK)
      return fail(st, "batch_run_lanes: instance " + std::to_string(i) + ": " + tsg_last_error());
  }
  const int used = std::max(1, std::min<int>(lanes, num_instances));
  const std::vector<int> lane = assign_lanes(num_instances, plans, used);
  std::vector<int64_t> off, bytes;
  int64_t total = 0;
  TSG_TRY(lane_regions(num_instances, plans, ring, num_primes, group_sizes, used, lane, &off,
                       &bytes, &total));
  if (!workspace_dev || workspace_bytes < total)
    return fail(TSG_ERR_WORKSPACE,
                "batch_run_lanes: workspace smaller than tsg_batch_lanes_workspace_bytes");
  if (((uintptr_t)workspace_dev & 255) != 0)
    return fail(TSG_ERR_WORKSPACE, "batch_run_lanes: workspace must be 256-byte aligned");
  cudaStream_t origin = (cudaStream_t)stream;
  uint8_t* ws = (uint8_t*)workspace_dev;
  if (used == 1) {
    for (int32_t i = 0; i < num_instances; ++i) {
      const int64_t ns = int64_t(1) << plans[i]->num_sliced;
      TSG_TRY(run_impl(plans[i], ring, num_primes, primes, leaf_pools[i], 0, ns,
                       group_sizes[i], ws, bytes[0], results_dev[i], 0, origin, /*dry=*/false));
    }
    return TSG_OK;
  }
  LaneSet* ls = nullptr;
  TSG_TRY(lane_set(used, &ls));
  // fork: every lane waits for the work issued before this call on the caller's stream
  TSG_CUDA_TRY(cudaEventRecord(ls->fork, origin));
  for (int l = 0; l < used; ++l) TSG_CUDA_TRY(cudaStreamWaitEvent(ls->streams[l], ls->fork, 0));
  for (int32_t i = 0; i < num_instances; ++i) {
    const int l = lane[i];
    const int64_t ns = int64_t(1) << plans[i]->num_sliced;
    TSG_TRY(run_impl(plans[i], ring, num_primes, primes, leaf_pools[i], 0, ns, group_sizes[i],
                     ws + off[l], bytes[l], results_dev[i], 0, ls->streams[l], /*dry=*/false));
  }
  // join: the caller's stream waits for every lane
  for (int l = 0; l < used; ++l) {
    TSG_CUDA_TRY(cudaEventRecord(ls->joins[l], ls->streams[l]));
    TSG_CUDA_TRY(cudaStreamWaitEvent(origin, ls->joins[l], 0));
  }
  return TSG_OK;
}

tsg_status tsg_batch_packed_workspace_bytes(int32_t num_instances,
                                            const tsg_plan* const* plans, int32_t ring,
                                            int32_t num_primes, const int64_t* group_sizes,
                                            int32_t lanes, int64_t* bytes_out) {
  if (num_instances < 0 || (num_instances > 0 && (!plans || !group_sizes)) || !bytes_out)
    return fail(TSG_ERR_INVALID_ARGUMENT, "batch_packed_workspace_bytes: null pointer or negative count");
  if (lanes < 1 || lanes > kMaxLanes)
    return fail(TSG_ERR_INVALID_ARGUMENT, "batch_packed_workspace_bytes: lanes outside 1..32");
  for (int32_t i = 0; i < num_instances; ++i)
    if (!plans[i]) return fail(TSG_ERR_INVALID_ARGUMENT, "batch_packed_workspace_bytes: null plan");
  if (num_instances == 0) {
    *bytes_out = 256;
    return TSG_OK;
  }
  PackSchedule ps;
  TSG_TRY(plan_packs(num_instances, plans, ring, num_primes, group_sizes, lanes, &ps));
  *bytes_out = ps.total;
  return TSG_OK;
}

tsg_status tsg_batch_run_packed(int32_t num_instances, const tsg_plan* const* plans,
                                int32_t ring, int32_t num_primes, const uint32_t* primes,
                                const uint8_t* const* leaf_pools, const int64_t* group_sizes,
                                int32_t lanes, void* workspace_dev, int64_t workspace_bytes,
                                void* const* results_dev, void* stream, int64_t* launches_out) {
  if (num_instances < 0 ||
      (num_instances > 0 && (!plans || !leaf_pools || !group_sizes || !results_dev)))
    return fail(TSG_ERR_INVALID_ARGUMENT, "batch_run_packed: null pointer or negative count");
  if (lanes < 1 || lanes > kMaxLanes)
    return fail(TSG_ERR_INVALID_ARGUMENT, "batch_run_packed: lanes outside 1..32");
  if (launches_out) *launches_out = 0;
  if (num_instances == 0) return TSG_OK;
  for (int32_t i = 0; i < num_instances; ++i)
    if (!plans[i] || !leaf_pools[i] || !results_dev[i])
      return fail(TSG_ERR_INVALID_ARGUMENT,
                  "batch_run_packed: null plan, pool or result of instance " + std::to_string(i));
  PackSchedule ps;
  TSG_TRY(plan_packs(num_instances, plans, ring, num_primes, group_sizes, lanes, &ps));
  if (!workspace_dev || workspace_bytes < ps.total)
    return fail(TSG_ERR_WORKSPACE,
                "batch_run_packed: workspace smaller than tsg_batch_packed_workspace_bytes");
  if (((uintptr_t)workspace_dev & 255) != 0)
    return fail(TSG_ERR_WORKSPACE, "batch_run_packed: workspace must be 256-byte aligned");
  int64_t eb;
  int planes;
  TSG_TRY(elem_info(ring, num_primes, &eb, &planes));
  RingArgs ra;
  TSG_TRY(make_ring_args(ring, num_primes, primes, &ra));
  uint8_t* ws = (uint8_t*)workspace_dev;
  // one pass that checks every launch of every pack before anything runs, one that runs
  int64_t launches = 0;
  for (int pass = 0; pass < 2; ++pass) {
    const bool dry = pass == 0;
    LaneSet* ls = nullptr;
    cudaStream_t origin = (cudaStream_t)stream;
    if (!dry && ps.used > 1) {
      TSG_TRY(lane_set(ps.used, &ls));
      // fork: every lane waits for the work issued before this call on the caller's stream
      TSG_CUDA_TRY(cudaEventRecord(ls->fork, origin));
      for (int l = 0; l < ps.used; ++l)
        TSG_CUDA_TRY(cudaStreamWaitEvent(ls->streams[l], ls->fork, 0));
    }
    for (int l = 0; l < ps.used; ++l) {
      cudaStream_t st = ls ? ls->streams[l] : origin;
      uint8_t* region = ws + ps.lane_off[l];
      for (const std::vector<int>& pack : ps.packs[l]) {
        const int first = pack[0];
        if (!ps.packed[first]) {
          const int64_t ns = int64_t(1) << plans[first]->num_sliced;
          tsg_status sst = run_impl(plans[first], ring, num_primes, primes,
                                    dry ? nullptr : leaf_pools[first], 0, ns, group_sizes[first],
                                    dry ? nullptr : region, dry ? 0 : ps.lane_bytes[l],
                                    dry ? nullptr : results_dev[first], 0, st, dry);
          if (sst != TSG_OK)
            return fail(sst, "batch_run_packed: instance " + std::to_string(first) + ": " +
                                 tsg_last_error());
          if (!dry) {
            int64_t c = 0;
            TSG_TRY(tsg_plan_launches(plans[first], ring, num_primes, 0, ns, group_sizes[first], &c));
            launches += c;
          }
          continue;
        }
        std::vector<PackMember> mem;
        for (int i : pack)
          mem.push_back(PackMember{plans[i], leaf_pools[i], dry ? nullptr : region + ps.inst_off[i],
                                   results_dev[i], group_sizes[i]});
        tsg_status sst = run_pack(mem, ring, ra, eb, planes, st, dry, dry ? nullptr : &launches);
        if (sst != TSG_OK)
          return fail(sst, "batch_run_packed: pack of instance " + std::to_string(first) + ": " +
                               tsg_last_error());
      }
    }
    if (ls) {
      // join: the caller's stream waits for every lane
      for (int l = 0; l < ps.used; ++l) {
        TSG_CUDA_TRY(cudaEventRecord(ls->joins[l], ls->streams[l]));
        TSG_CUDA_TRY(cudaStreamWaitEvent(origin, ls->joins[l], 0));
      }
    }
  }
  if (launches_out) *launches_out = launches;
  return TSG_OK;
}

int64_t tsg_static_scratch_bytes(void) { return kStaticScratchBytes; }

tsg_status tsg_set_wait_limit_ns(uint64_t limit_ns) {
  if (limit_ns < 1000 || limit_ns > kWaitLimitNs)
    return fail(TSG_ERR_INVALID_ARGUMENT, "set_wait_limit_ns: limit outside [1 us, 2 s]");
  g_wait_limit_ns.store(limit_ns, std::memory_order_relaxed);
  return TSG_OK;
}

uint64_t tsg_wait_limit_ns(void) { return g_wait_limit_ns.load(std::memory_order_relaxed); }

tsg_status tsg_debug_stall_producer(int64_t stages) {
  g_stall_after.store(stages < 0 ? -1 : stages, std::memory_order_relaxed);
  return TSG_OK;
}

tsg_status tsg_take_device_error(void* stream) {
  int err = 0;
  const int zero = 0;
  cudaStream_t st = (cudaStream_t)stream;
  TSG_CUDA_TRY(cudaMemcpyFromSymbolAsync(&err, g_device_error, sizeof(int), 0,
                                         cudaMemcpyDeviceToHost, st));
  TSG_CUDA_TRY(cudaStreamSynchronize(st));
  if (err == 0) return TSG_OK;
  TSG_CUDA_TRY(cudaMemcpyToSymbolAsync(g_device_error, &zero, sizeof(int), 0,
                                       cudaMemcpyHostToDevice, st));
  TSG_CUDA_TRY(cudaStreamSynchronize(st));
  return fail(TSG_ERR_TIMEOUT, "a bounded device-side wait gave up (TMA staging did not "
                               "complete); results of the affected runs are invalid");
}

tsg_status tsg_peek_device_error_async(int32_t* host_dst, void* stream) {
  if (!host_dst) return fail(TSG_ERR_INVALID_ARGUMENT, "peek_device_error: null destination");
  TSG_CUDA_TRY(cudaMemcpyFromSymbolAsync(host_dst, g_device_error, sizeof(int), 0,
                                         cudaMemcpyDeviceToHost, (cudaStream_t)stream));
  return TSG_OK;
}

tsg_status tsg_plan_run_static(const tsg_plan* plan, int32_t ring, int32_t num_primes,
                               const uint32_t* primes, const uint8_t* leaf_pool_dev,
                               int64_t slice_begin, int64_t slice_end, int64_t group_size,
                               void* result_dev, int32_t accumulate, void* stream) {
  if (!plan || !leaf_pool_dev || !result_dev)
    return fail(TSG_ERR_INVALID_ARGUMENT, "plan_run_static: null pointer");
  // the size check and every argument check happen on the host, before any device work
  int64_t need = 0;
  TSG_TRY(tsg_plan_workspace_bytes(plan, ring, num_primes, group_size, &need));
  if (need > kStaticScratchBytes)
    return fail(TSG_ERR_WORKSPACE,
                "plan_run_static: this plan and group size need " + std::to_string(need) +
                    " bytes of scratch, more than the 64 MiB static array; use tsg_plan_run "
                    "with a caller workspace or a smaller group size");
  void* scratch = nullptr;
  TSG_TRY(static_scratch_address(&scratch));
  return run_impl(plan, ring, num_primes, primes, leaf_pool_dev, slice_begin, slice_end,
                  group_size, scratch, kStaticScratchBytes, result_dev, accumulate,
                  (cudaStream_t)stream, /*dry=*/false);
}

}  // extern "C"
