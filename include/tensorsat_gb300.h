/*
 * tensorsat_gb300.h -- C ABI of the GB300 (sm_103a) executor for TensorSat's hot path:
 * contracting the Boolean tensor network a CNF instance compiles to, pairwise, along a
 * contraction tree, in the OR-AND semiring (SAT bit) or over exact integers (model count).
 *
 * Conventions (all entry points):
 *   - plain C types only; every pointer named `*_dev` or documented as "device" is a
 *     device pointer owned by the caller; host arrays are read during the call only;
 *   - tensors are dense and C-ordered (first port = slowest-varying index), exactly like
 *     the numpy arrays held by tensorsat's FinRel;
 *   - `stream` is a cudaStream_t (NULL = legacy default stream); every call is
 *     asynchronous with respect to the host unless stated otherwise;
 *   - no entry point allocates device memory on the contraction path: the tree executor
 *     runs inside a caller-provided workspace whose size tsg_plan_workspace_bytes reports;
 *   - errors are returned as status codes (never as exceptions); tsg_last_error() returns
 *     a message describing the last failing call on the calling thread.
 *
 * Reference interfaces replaced (paths are relative to the tensorsat project root):
 *   tsg_contract2_or_and     FinRel._contract2            tensorsat/lang/fin_rel.py:255-288
 *   tsg_contract2_count_u64, tsg_contract2_modp
 *                            the unclamped einsum of the #SAT prototype
 *                            notebooks/prototypes/2025-02-13-#sat-tensor-contraction.ipynb
 *                            (cells 11-12); the count semantics FinRel itself never offers
 *   tsg_rewire_or_and        FinRel._rewire                tensorsat/lang/fin_rel.py:379-393
 *                            (with misc.rewire_array       tensorsat/_utils/misc.py:104-123)
 *   tsg_union_or             FinRel._union                 tensorsat/lang/fin_rel.py:345-346
 *   tsg_spider_fill          FinRel._spider                tensorsat/lang/fin_rel.py:290-298
 *   tsg_plan_create / tsg_plan_run
 *                            the per-node loop of a contraction tree:
 *                            SimpleContraction.contract    tensorsat/contractions/simple.py:251-292
 *                            and CotengraContraction.contract (tree.contract, one einsum per
 *                            node through tensorsat/_autoray.py:31-62)
 *                                                          tensorsat/contractions/cotengra.py:100-128
 *                            with sliced indices combined by `+` (OR for FinRel,
 *                            tensorsat/diagrams.py:965-970) or by integer sum (counts).
 */
#ifndef TENSORSAT_GB300_H
#define TENSORSAT_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#if defined(__GNUC__)
#define TSG_API __attribute__((visibility("default")))
#else
#define TSG_API
#endif

typedef int32_t tsg_status;

#define TSG_OK 0
#define TSG_ERR_INVALID_ARGUMENT 1 /* bad ranks, wires, dims or pointers (ValueError upstream) */
#define TSG_ERR_UNSUPPORTED 2      /* valid request outside what the kernels implement */
#define TSG_ERR_TOO_LARGE 3        /* a tensor or index space exceeds the 64-bit / size limits */
#define TSG_ERR_WORKSPACE 4        /* workspace missing, misaligned or smaller than required */
#define TSG_ERR_CUDA 5             /* a CUDA runtime call failed (message has the CUDA error) */
#define TSG_ERR_TIMEOUT 6          /* a bounded device-side wait gave up */

/* Arithmetic of a tree run (tsg_plan_run). */
#define TSG_RING_OR_AND 0 /* uint8 {0,1}: out = OR_k (L AND R); the SAT-bit semiring */
#define TSG_RING_MODP 1   /* uint32 residues mod odd primes in (2^31-2^26, 2^31), one plane each */
#define TSG_RING_U64 2    /* uint64 with wrap-around: the count modulo 2^64 */

#define TSG_MAX_PORTS 64  /* ports per operand of a per-step contraction */
#define TSG_MAX_BITS 62   /* wires of one tree-step index space (out bits + summed bits) */
#define TSG_MAX_PRIMES 4  /* residue planes per TSG_RING_MODP run */

/* Message of the last failing call on this thread ("" if none). Never NULL. */
TSG_API const char* tsg_last_error(void);

/* ABI version of this library (incremented on incompatible changes). */
TSG_API int32_t tsg_abi_version(void);

/* ---------------------------------------------------------------------------------
 * Per-step (box-level) operations. Wires are arbitrary int64 labels; a label may repeat
 * inside lhs_wires, rhs_wires or out_wires (einsum diagonal semantics), and every out
 * wire must occur in lhs or rhs. Dims are given per port; ports carrying the same wire
 * must have equal dims. Wires of lhs/rhs that are absent from out_wires are summed.
 * ------------------------------------------------------------------------------- */

/* out = sign(einsum(lhs, lhs_wires, rhs, rhs_wires -> out_wires)) over uint8 {0,1}
 * tensors; out has shape (dim of out_wires[i])_i. Replaces FinRel._contract2. */
TSG_API tsg_status tsg_contract2_or_and(const uint8_t* lhs_dev, int32_t lhs_rank,
                                const int64_t* lhs_wires, const int64_t* lhs_dims,
                                const uint8_t* rhs_dev, int32_t rhs_rank,
                                const int64_t* rhs_wires, const int64_t* rhs_dims,
                                int32_t out_rank, const int64_t* out_wires,
                                uint8_t* out_dev, void* stream);

/* Same index semantics with uint64 entries and no clamping (counts, wrap mod 2^64). */
TSG_API tsg_status tsg_contract2_count_u64(const uint64_t* lhs_dev, int32_t lhs_rank,
                                   const int64_t* lhs_wires, const int64_t* lhs_dims,
                                   const uint64_t* rhs_dev, int32_t rhs_rank,
                                   const int64_t* rhs_wires, const int64_t* rhs_dims,
                                   int32_t out_rank, const int64_t* out_wires,
                                   uint64_t* out_dev, void* stream);

/* The same index semantics over residues: num_primes (1..4) planes of uint32 residues
 * (plain, 0 <= x < p) lie back to back in lhs, rhs and out (plane q of a tensor at
 * q * its entry count); plane q of out is sum(lhs * rhs) mod primes[q] (any moduli >= 2),
 * each product reduced, so no intermediate overflows. The per-step form of exact model
 * counting modulo several primes, recombined by CRT on the host; counterpart of
 * tsg_contract2_count_u64 beyond 2^64 (FinRel._contract2's einsum,
 * tensorsat/lang/fin_rel.py:255-288, without the clamp). */
TSG_API tsg_status tsg_contract2_modp(const uint32_t* lhs_dev, int32_t lhs_rank,
                              const int64_t* lhs_wires, const int64_t* lhs_dims,
                              const uint32_t* rhs_dev, int32_t rhs_rank,
                              const int64_t* rhs_wires, const int64_t* rhs_dims,
                              int32_t out_rank, const int64_t* out_wires, int32_t num_primes,
                              const uint32_t* primes, uint32_t* out_dev, void* stream);

/* out = sign(rewire(in, out_ports)): permute / duplicate (diagonal) / discard (sum)
 * ports of a uint8 {0,1} tensor. Replaces FinRel._rewire. */
TSG_API tsg_status tsg_rewire_or_and(const uint8_t* in_dev, int32_t rank, const int64_t* dims,
                             int32_t out_rank, const int32_t* out_ports, uint8_t* out_dev,
                             void* stream);

/* out[i] = a[i] | b[i] for i < n (uint8). Replaces FinRel._union. */
TSG_API tsg_status tsg_union_or(const uint8_t* a_dev, const uint8_t* b_dev, uint8_t* out_dev,
                        int64_t n, void* stream);

/* Writes the COPY/spider tensor of `num_ports` ports of dimension `dim`:
 * out[i,...,i] = 1, every other entry 0. Replaces FinRel._spider. */
TSG_API tsg_status tsg_spider_fill(uint8_t* out_dev, int64_t dim, int32_t num_ports, void* stream);

/* ---------------------------------------------------------------------------------
 * Tree executor. A plan is a contraction tree over wires of dimension 2 (bits), with an
 * optional set of sliced wires. Leaves are uint8 {0,1} tensors, packed into one device
 * pool; sliced wires stay inside the leaves and are fixed per slice by the executor.
 *
 * Leaf l: rank leaf_ranks[l] (bits, sliced bits included), element offset
 *   leaf_offsets[l] in the pool, and for each sliced wire j < num_sliced the bit position
 *   leaf_slice_pos[l*num_sliced + j] of that wire inside the leaf index (bit 0 = last,
 *   fastest port), or -1 if the leaf does not carry it. Slice id bit j = value of sliced
 *   wire j.
 * Step s combines operands step_operands[2s] and step_operands[2s+1] (a value v >= 0 is
 *   leaf v; v < 0 is the result of step -v-1, which must precede s). Its index space has
 *   step_out_bits[s] output bits and step_sum_bits[s] summed bits. For operand X in
 *   {lhs, rhs}: step_lhs_pos / step_rhs_pos[s*TSG_MAX_BITS + i] is the bit position inside
 *   X of output bit i (i < out_bits), then of summed bit i-out_bits, or -1 when X does not
 *   carry that wire. Output bit i of step s is bit i of its result tensor. Every
 *   intermediate is consumed exactly once; the last step is the root.
 * ------------------------------------------------------------------------------- */
typedef struct tsg_plan tsg_plan;

TSG_API tsg_status tsg_plan_create(int32_t num_leaves, const int32_t* leaf_ranks,
                           const int64_t* leaf_offsets, int32_t num_sliced,
                           const int32_t* leaf_slice_pos, int32_t num_steps,
                           const int32_t* step_operands, const int32_t* step_out_bits,
                           const int32_t* step_sum_bits, const int32_t* step_lhs_pos,
                           const int32_t* step_rhs_pos, tsg_plan** plan_out);

TSG_API void tsg_plan_destroy(tsg_plan* plan);

/* Bytes of workspace tsg_plan_run needs for `group_size` slices per launch group. */
TSG_API tsg_status tsg_plan_workspace_bytes(const tsg_plan* plan, int32_t ring, int32_t num_primes,
                                    int64_t group_size, int64_t* bytes_out);

/* Root output bits of the plan (the result tensor has 2^bits entries per plane). */
TSG_API tsg_status tsg_plan_root_bits(const tsg_plan* plan, int32_t* bits_out);

/* Number of kernel launches tsg_plan_run issues for the given slice range and group when
 * no step is fused (the OR-AND ring, or fusion off); tsg_plan_launches counts them for a
 * given ring. */
TSG_API tsg_status tsg_plan_launch_count(const tsg_plan* plan, int64_t slice_begin,
                                 int64_t slice_end, int64_t group_size, int64_t* count_out);

/* Number of kernel launches tsg_plan_run issues for these arguments (fused steps issue
 * none of their own). Host only. */
TSG_API tsg_status tsg_plan_launches(const tsg_plan* plan, int32_t ring, int32_t num_primes,
                             int64_t slice_begin, int64_t slice_end, int64_t group_size,
                             int64_t* count_out);

/* Fused steps, allowed (1, the default) or not (0), for plans whose layouts are made after
 * the call (layouts are made per plan, ring and group on first use and kept). A step whose
 * step options carry TSG_STEP_FUSE (tsg_plan_set_step_options; the autotuner sets it
 * where fusing measured faster) and whose large result is read once, as the reused
 * operand of its consumer's tile or streaming form, is not launched: the consumer computes
 * each entry it needs from the step's two operands, so the result never exists in HBM
 * (the structural conditions are in the library's choose_fusion). Results are identical
 * either way; fused plans need less workspace and move fewer bytes, at the price of
 * gathers in the consumer. Process-wide. No counterpart in the reference, which runs one
 * einsum per tree node (tensorsat/_autoray.py:31-62). */
TSG_API tsg_status tsg_set_fusion(int32_t enabled);
TSG_API int32_t tsg_fusion_enabled(void);

/* Per-step kernel options of a plan in one ring (the autotuner's choices): options[s] is
 * a bit set of TSG_STEP_NO_STREAM (run step s on the tile kernel even where the streaming
 * kernel applies), TSG_STEP_NO_FUSE (never compute step s inside its consumer) and
 * TSG_STEP_FUSE (compute step s inside its consumer where the structure allows it; no
 * step is fused without it) and TSG_STEP_PLANE_SPLIT, for every step (num_steps entries);
 * options == NULL clears
 * them. Later runs, workspace sizes and descriptions of that ring follow them; results do
 * not depend on them. Host only.
 * No counterpart in the reference, whose path choice (cotengra's optimize/order kwargs,
 * tensorsat/contractions/cotengra.py:62-64,104-106) has no kernel to choose. */
#define TSG_STEP_NO_STREAM 1
#define TSG_STEP_NO_FUSE 2
#define TSG_STEP_FUSE 4
#define TSG_STEP_PLANE_SPLIT 8 /* MODP tile kernel: one residue plane per block (default:
                                  every plane in one thread) */
TSG_API tsg_status tsg_plan_set_step_options(tsg_plan* plan, int32_t ring,
                                     const int32_t* options);

/* Contracts slices [slice_begin, slice_end) of the plan, `group_size` slices per launch
 * group (a power of two; slice_begin must be a multiple of it, the last group may be
 * partial), and combines the per-slice root tensors into result_dev:
 *   OR_AND: uint8 [2^root_bits], OR over slices;
 *   MODP:   uint32 [num_primes][2^root_bits], sum mod primes[p];
 *   U64:    uint64 [2^root_bits], sum mod 2^64.
 * If accumulate != 0 the result is combined with the existing contents of result_dev,
 * otherwise it is overwritten. leaf_pool_dev holds the uint8 leaves. workspace_dev must
 * be 256-byte aligned and at least tsg_plan_workspace_bytes long. Every launch is
 * bounds-checked on the host first (see tsg_plan_validate). */
TSG_API tsg_status tsg_plan_run(const tsg_plan* plan, int32_t ring, int32_t num_primes,
                        const uint32_t* primes, const uint8_t* leaf_pool_dev,
                        int64_t slice_begin, int64_t slice_end, int64_t group_size,
                        void* workspace_dev, int64_t workspace_bytes, void* result_dev,
                        int32_t accumulate, void* stream);

/* Batched runs of many instances (for example a batch of random CNF instances of uneven
 * sizes, each with its own plan). Instance i contracts all 2^num_sliced slices of plans[i]
 * over its leaf pool leaf_pools[i] in groups of group_sizes[i] and overwrites results[i]
 * (layout as in tsg_plan_run). The instances run one after another on `stream` and share
 * one workspace of at least tsg_batch_workspace_bytes. Every instance's arguments and
 * every launch are checked on the host before the first launch, so a bad instance fails
 * the call with nothing launched. The call neither allocates nor synchronises: it can be
 * captured into a CUDA graph and replayed (make one uncaptured call first, which sets
 * up per-kernel attributes). No counterpart in the reference, which contracts one
 * instance per call (tensorsat/contractions/abc.py:92, Contraction.contract). */
TSG_API tsg_status tsg_batch_workspace_bytes(int32_t num_instances, const tsg_plan* const* plans,
                                     int32_t ring, int32_t num_primes,
                                     const int64_t* group_sizes, int64_t* bytes_out);
TSG_API tsg_status tsg_batch_run(int32_t num_instances, const tsg_plan* const* plans,
                         int32_t ring, int32_t num_primes, const uint32_t* primes,
                         const uint8_t* const* leaf_pools, const int64_t* group_sizes,
                         void* workspace_dev, int64_t workspace_bytes,
                         void* const* results_dev, void* stream);

/* tsg_batch_run over `lanes` (1..32) concurrent lanes: the instances are spread over the
 * lanes (longest estimated work first, each to the least loaded lane), every lane is a
 * stream that forks from `stream` at the call and joins it at the end, and each lane has
 * its own region of the workspace, whose total size tsg_batch_lanes_workspace_bytes
 * reports (the largest workspace of each lane's instances, summed over lanes). Instances
 * on different lanes run concurrently, so the many small launches of small instances
 * overlap on the GPU. Checks every instance and launch before the first launch, like
 * tsg_batch_run; neither allocates device memory nor synchronises, and it can be captured
 * into a CUDA graph (the lanes become parallel branches of the graph). The lane streams
 * are created once per host thread and device. lanes == 1 is tsg_batch_run with the
 * lane workspace rule. No counterpart in the reference (one instance per call). */
TSG_API tsg_status tsg_batch_lanes_workspace_bytes(int32_t num_instances,
                                           const tsg_plan* const* plans, int32_t ring,
                                           int32_t num_primes, const int64_t* group_sizes,
                                           int32_t lanes, int64_t* bytes_out);
TSG_API tsg_status tsg_batch_run_lanes(int32_t num_instances, const tsg_plan* const* plans,
                               int32_t ring, int32_t num_primes, const uint32_t* primes,
                               const uint8_t* const* leaf_pools, const int64_t* group_sizes,
                               int32_t lanes, void* workspace_dev, int64_t workspace_bytes,
                               void* const* results_dev, void* stream);

/* tsg_batch_run_lanes with the instances' small steps packed across instances: each lane's
 * instances whose group holds all their slices are grouped into packs whose workspaces
 * fit side by side in the lane's region (the region holds the lane's largest instance;
 * instances are placed largest first). A pack runs level by level of its members' trees:
 * every step of the level with at most 2^16 output entries (slots included) and 2^5 summed
 * combinations, of every member, goes into shared launches of one packed kernel (up to
 * 240 steps per launch, described in the launch parameters); the level's other steps
 * follow as their own launches; each member ends with its root reduction. Such a pack
 * uses the level-order buffer placement, whose size tsg_batch_packed_workspace_bytes
 * includes. An instance run in several slice groups runs alone, as in tsg_batch_run.
 * Results equal tsg_batch_run's. Checks every launch of every pack before the first,
 * neither allocates nor synchronises, and can be captured into a CUDA graph.
 * *launches_out (if not null) receives the number of kernel launches issued. No
 * counterpart in the reference (one instance per call, one einsum per tree node:
 * tensorsat/contractions/abc.py:92, tensorsat/_autoray.py:31-62). */
TSG_API tsg_status tsg_batch_packed_workspace_bytes(int32_t num_instances,
                                            const tsg_plan* const* plans, int32_t ring,
                                            int32_t num_primes, const int64_t* group_sizes,
                                            int32_t lanes, int64_t* bytes_out);
TSG_API tsg_status tsg_batch_run_packed(int32_t num_instances, const tsg_plan* const* plans,
                                int32_t ring, int32_t num_primes, const uint32_t* primes,
                                const uint8_t* const* leaf_pools, const int64_t* group_sizes,
                                int32_t lanes, void* workspace_dev, int64_t workspace_bytes,
                                void* const* results_dev, void* stream,
                                int64_t* launches_out);

/* Leaf variants of one plan in one run: num_variants (a power of two) copies of the leaf
 * pool lie pool_stride bytes apart (a power of two, at least the plan's pool extent and
 * 16); every tree step is launched once per slice group for all variants together (the
 * variant index is an extra batch axis of the launch, beside the slices), and variant v's
 * result goes to results_dev + v * (result size of tsg_plan_run). All slices are
 * contracted, group_size per launch group and variant; the workspace must hold
 * tsg_plan_variants_workspace_bytes. This is the reference's assignment-search idiom (one
 * wiring, many unit-input diagrams: notebooks/02-random-ksat.ipynb cells 35-36,
 * tensorsat/contractions/abc.py:91-97) with one launch sequence instead of one
 * contraction per variant. */
TSG_API tsg_status tsg_plan_variants_workspace_bytes(const tsg_plan* plan, int32_t ring,
                                             int32_t num_primes, int64_t group_size,
                                             int64_t num_variants, int64_t* bytes_out);
TSG_API tsg_status tsg_plan_run_variants(const tsg_plan* plan, int32_t ring, int32_t num_primes,
                                 const uint32_t* primes, const uint8_t* leaf_pools_dev,
                                 int64_t pool_stride, int64_t num_variants,
                                 int64_t group_size, void* workspace_dev,
                                 int64_t workspace_bytes, void* results_dev,
                                 int32_t accumulate, void* stream);

/* tsg_plan_run that also measures: a CUDA event is recorded on `stream` before the first
 * launch and after every launch, and on return (the call waits for the run to finish)
 * step_ms[s] holds the device time of tree step s summed over the slice groups of the
 * call, step_ms[num_steps] that of the root reductions (caller array of num_steps + 1
 * floats). For profiling: the events add a few microseconds per launch. No counterpart
 * in the reference, which has no device execution to time. */
TSG_API tsg_status tsg_plan_run_timed(const tsg_plan* plan, int32_t ring, int32_t num_primes,
                              const uint32_t* primes, const uint8_t* leaf_pool_dev,
                              int64_t slice_begin, int64_t slice_end, int64_t group_size,
                              void* workspace_dev, int64_t workspace_bytes, void* result_dev,
                              int32_t accumulate, void* stream, float* step_ms);

/* Builds every launch tsg_plan_run would issue for these arguments and checks, on the
 * host, that each operand offset stays inside its leaf or workspace buffer. Touches no
 * device memory and needs no GPU. */
TSG_API tsg_status tsg_plan_validate(const tsg_plan* plan, int32_t ring, int32_t num_primes,
                             const uint32_t* primes, int64_t slice_begin,
                             int64_t slice_end, int64_t group_size);

/* Kernel families of a tree step (tsg_plan_describe). */
#define TSG_KERNEL_GENERAL 0 /* one output entry per thread, bit-scatter offsets */
#define TSG_KERNEL_TILE 1    /* tile kernel: V positions and NE enumerated outputs per thread */
#define TSG_KERNEL_STREAM 2  /* streaming kernel: TMA-staged operands, persistent blocks */
#define TSG_KERNEL_FUSED 3   /* fused kernel: a tile-form step that computes its reused operand
                                from that operand's own two operands (see tsg_set_fusion) */
#define TSG_KERNEL_NONE 4    /* no launch: the step's result is computed inside its consumer */
#define TSG_KERNEL_SUM 5     /* few outputs, many summed combinations: one block per output,
                                its threads split the sum */

/* For every tree step s, the kernel tsg_plan_run launches for it with these arguments
 * (the first slice group of size group_size, 1 <= group_size <= slices), as four int32
 * at kinds[4 s ...]: the family (TSG_KERNEL_*), then the template parameters V (tile
 * kernel: positions per thread, else 0), NE (enumerated output combinations per thread)
 * and NK (summed combinations unrolled at compile time; 0 = a runtime count); a step
 * computed inside its consumer reports TSG_KERNEL_NONE and zeros. Builds and
 * bounds-checks every launch like tsg_plan_validate; touches no device memory and needs no
 * GPU. No counterpart in the reference, which contracts every step with one numpy einsum
 * (tensorsat/lang/fin_rel.py:276,283). */
TSG_API tsg_status tsg_plan_describe(const tsg_plan* plan, int32_t ring, int32_t num_primes,
                             const uint32_t* primes, int64_t group_size, int32_t* kinds);

/* ---------------------------------------------------------------------------------
 * Planner (host only; touches no device and needs no GPU).
 *
 * The dynamic program of subtree reconfiguration over the n (1..20) inputs of one cut
 * subtree: the cheapest binary contraction of the inputs, where the partial result of an
 * input subset m keeps the wires of m that the subtree's root keeps or an input outside
 * m carries, and a step costs 2^(live wires of its two operands together). Wire sets are
 * bitsets of `words` (1..64) 64-bit words: bits[i * words ...] the wires of input i,
 * keep[] the root's wires, live[] the unsliced wires. With max_bits >= 0 a partial result
 * (other than the whole subtree) with more than max_bits live wires is infeasible.
 * Outputs: *best_full the cheapest total cost (INFINITY when infeasible); split[m]
 * (2^n entries) the operand of m's cheapest split that holds m's lowest input;
 * kept[m * words ...] (2^n * words words) the wires m's partial result keeps. Splits are
 * visited in a fixed order and only a strictly cheaper one replaces the best, so results
 * are deterministic. Stands in for the tree search of cotengra's hyper-optimiser
 * (ctg.array_contract_tree), which the reference calls at
 * tensorsat/contractions/cotengra.py:78-85; cotengra itself is not part of this build. */
TSG_API tsg_status tsg_plan_subset_dp(int32_t n, int32_t words, const uint64_t* bits,
                              const uint64_t* keep, const uint64_t* live, int32_t max_bits,
                              double* best_full, uint32_t* split, uint64_t* kept);

/* Synchronizes `stream` and reports whether any kernel of this library recorded a device-
 * side failure since the last call (a bounded wait that gave up: TSG_ERR_TIMEOUT); the
 * record is cleared. Runs launched before the failure are invalid. */
TSG_API tsg_status tsg_take_device_error(void* stream);

/* Enqueues on `stream` a copy of the device-side failure record (0: none) into *host_dst
 * (4 bytes; pinned host memory keeps the copy asynchronous) without synchronizing or
 * clearing it, so a pipelined caller can check a finished run after waiting on its own
 * event; when the copy reads non-zero, tsg_take_device_error reports and clears it. */
TSG_API tsg_status tsg_peek_device_error_async(int32_t* host_dst, void* stream);

/* Limit of every bounded wait inside the streaming kernel (a consumer waiting for staged
 * data, the producer waiting for a free stage), in nanoseconds of the GPU's global timer;
 * between 1 us and the default 2 s. A wait that runs out makes the kernel record
 * TSG_ERR_TIMEOUT (read by tsg_take_device_error) and return; the producer still waits for
 * its own copies in flight (up to 2 s) before its block exits. Applies to launches issued
 * after the call, process-wide. No counterpart in the reference (no device code). */
TSG_API tsg_status tsg_set_wait_limit_ns(uint64_t limit_ns);
TSG_API uint64_t tsg_wait_limit_ns(void);

/* Testing hook: with stages >= 0, the producer warp of every streaming block stops after
 * issuing that many stages (it issues no further copy and arms no further barrier), so
 * the consumers' next wait runs out after tsg_wait_limit_ns and the run reports
 * TSG_ERR_TIMEOUT through tsg_take_device_error; results of such runs are invalid.
 * stages < 0 (the default) turns it off. Process-wide, for launches issued after the
 * call. It exercises the bounded-wait exit path without any device fault. */
TSG_API tsg_status tsg_debug_stall_producer(int64_t stages);

/* ---------------------------------------------------------------------------------
 * Allocation-free variant (no counterpart in the reference).
 *
 * tsg_plan_run with its scratch taken from a 64 MiB array in device global memory that
 * the library itself owns (a file-scope static __device__ array), instead of a caller
 * workspace. It is for callers that cannot allocate device memory themselves: host
 * bindings that only pass pointers to buffers the application already owns (ctypes,
 * cgo, JNI, N-API stubs with no CUDA allocator of their own) and services that must not
 * grow their device memory after start-up. It makes no cudaMalloc / cudaFree call and
 * uses no allocating library routine; the caller still provides the leaf pool and the
 * result buffer.
 *   - Limit: plans whose tsg_plan_workspace_bytes(plan, ring, num_primes, group_size)
 *     exceeds tsg_static_scratch_bytes() (64 MiB) are rejected with TSG_ERR_WORKSPACE
 *     before any device work; lower group_size or use tsg_plan_run.
 *   - The first call on a device resolves the array's device address with
 *     cudaGetSymbolAddress (with that device current) and caches it; make that first
 *     call before any stream capture. The cached address belongs to the device's primary
 *     context, which the CUDA runtime uses: it is not refreshed after cudaDeviceReset or
 *     for a caller that makes another context current, so such callers use tsg_plan_run.
 *   - Every call shares the one array and reuses whatever the previous call left in it:
 *     the executor writes each intermediate before reading it, so nothing needs clearing;
 *     result_dev follows the `accumulate` rule of tsg_plan_run.
 *   - Calls whose work overlaps on the GPU (concurrent streams, or several host threads)
 *     race on the array: serialize them on one stream.
 *   - Every GPU that loads the library holds the 64 MiB until the process exits. */
TSG_API int64_t tsg_static_scratch_bytes(void);

TSG_API tsg_status tsg_plan_run_static(const tsg_plan* plan, int32_t ring, int32_t num_primes,
                               const uint32_t* primes, const uint8_t* leaf_pool_dev,
                               int64_t slice_begin, int64_t slice_end, int64_t group_size,
                               void* result_dev, int32_t accumulate, void* stream);

/* ---------------------------------------------------------------------------------
 * Learned cost model (tensorsat_gb300/costmodel.py): a message-passing network over
 * contraction trees that predicts a tree's device time and ranks candidate trees. Its
 * answers never reach a contraction's result. No counterpart in the reference, whose tree
 * search is cotengra's hyper-optimiser (tensorsat/contractions/cotengra.py:78-85).
 * ------------------------------------------------------------------------------- */

/* out[M x N] = a[M x K] * b[N x K]^T (+ bias[N]) (ReLU if relu != 0), on the tensor cores
 * (tcgen05.mma kind::f16: BF16 a and b, row-major with K contiguous, 16-byte aligned; FP32
 * accumulation in tensor memory); out is FP32 (out_f32 != 0) or BF16, row stride ldo
 * elements. M a multiple of 128, K of 64, N 64 or 128. */
TSG_API tsg_status tsg_cm_gemm_bf16(int64_t m, int64_t n, int64_t k, const void* a_dev,
                            const void* b_dev, const float* bias_dev, int32_t relu,
                            void* out_dev, int64_t ldo, int32_t out_f32, void* stream);

/* out[v] = sum of h[u] over the children u of node v (BF16 rows of `width`; children of v
 * are child[cstart[v] .. cstart[v+1]); out row stride ldo). */
/* Operand staging of tsg_cm_gemm_bf16 for the whole process: 0 (default) loads the A and
 * B tiles with TMA tensor copies (cp.async.bulk.tensor, 128-byte swizzle, one thread
 * issuing copies and MMAs), 1 stages them with the CTA's threads (canonical layout without
 * swizzle). Both give the same products. */
TSG_API tsg_status tsg_cm_set_gemm_mode(int32_t mode);
TSG_API tsg_status tsg_cm_child_sum(const void* h_dev, const int32_t* cstart_dev,
                            const int32_t* child_dev, void* out_dev, int64_t n,
                            int32_t width, int32_t ldo, void* stream);

/* dh[u] += dc[parent[u]] for every node with parent[u] >= 0 (FP32 rows; dc row stride ldc):
 * the transpose of tsg_cm_child_sum, for the backward pass. */
TSG_API tsg_status tsg_cm_parent_add(const float* dc_dev, int32_t ldc, const int32_t* parent_dev,
                             float* dh_dev, int64_t n, int32_t width, void* stream);

/* out[p x q] = a[n x p]^T * b[n x q] (FP32, row-major): weight gradients, a reduction over
 * the n nodes. */
TSG_API tsg_status tsg_cm_gemm_at_b(const float* a_dev, int32_t p, const float* b_dev,
                            int32_t q, int64_t n, float* out_dev, void* stream);

/* One Adam step on n FP32 parameters (moments m, v; step >= 1 for the bias correction). */
TSG_API tsg_status tsg_cm_adam(float* w_dev, const float* g_dev, float* m_dev, float* v_dev,
                       int64_t n, float lr, float beta1, float beta2, float eps, int32_t step,
                       void* stream);

/* Synchronizes `stream` and reports (then clears) a bounded wait of the cost model's
 * kernels that gave up (TSG_ERR_TIMEOUT). */
TSG_API tsg_status tsg_cm_take_error(void* stream);

#ifdef __cplusplus
}
#endif

#endif /* TENSORSAT_GB300_H */
