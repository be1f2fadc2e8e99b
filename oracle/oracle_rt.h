/* oracle_rt.h - CPU restatement of the reference's functional ray-traversal
 * path.  TEST INFRASTRUCTURE ONLY: the parity tests, the smoke check and the
 * CPU-baseline leg of the benchmark call it as the checker; the library never
 * links or calls it.
 *
 * Parity status: the reference (Vulkan-Sim's vulkan_ray_tracing.cc) cannot be
 * built as a whole here (it needs Mesa, the Vulkan SDK, Boost, flex and bison),
 * and it ships no tests or golden vectors for this path.  The path's own
 * functions are compiled in place from the reference tree by oracle/ref_pin/
 * (the decoder header unmodified; the geometry, createTreelets /
 * buildNodeToRootMap / remapBVHToTreeletLayout, traceRay and
 * traceRayWithTreelets as extracted line ranges), and the oracle is pinned
 * against their outputs (tests/golden/), as are the RT-unit replay's
 * treelet-prefetch decision (the decision block of shader.cc's
 * rt_unit::cycle), its warp selection (rt_unit::schedule_next_warp) and its
 * Lee stride prefetcher with the demand-load queue removal (blocks of
 * rt_unit::memory_cycle) and its end-of-run prefetch tally (gpu-sim.cc), each
 * extracted and compiled in a stand-in RT unit.
 * The replay's memory model (cache, latencies, cycle loop) is this project's
 * own: no reference code pins it.
 */
#ifndef ORACLE_RT_H
#define ORACLE_RT_H
#include <stdint.h>

#include "../include/treelet_rt.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct oracle_treelets oracle_treelets;

/* One node decoded by the oracle (kind 0 header, 1 internal, 2 instance
 * leaf, 3 quad leaf) into 62 doubles, in the record layout of
 * oracle/ref_pin/pin_decoders.cpp, which decodes with the reference's own
 * vulkan_acceleration_structure_util.h.  Returns 0 or -1. */
int oracle_decode_node(const uint8_t* blob, uint32_t unit, int kind, double* out);

/* The oracle's ray geometry on n cases (op 0 calculate_idir + ray_box_test,
 * 1 mt_ray_triangle_test, 2 make_transformed_ray, 3 Barycentric), in the case
 * and result layouts of oracle/ref_pin/pin_geometry.cpp, which runs the
 * reference's own functions.  Returns 0 or -1. */
int oracle_geometry(int op, const float* in, uint32_t n, float* out);

/* createTreelets + buildNodeToRootMap over a blob (vulkan_ray_tracing.cc:823-1470,
 * :475-489).  Returns NULL on a condition where the reference asserts; the
 * message is in oracle_last_error(). */
oracle_treelets* oracle_form_treelets(const uint8_t* blob, uint64_t n_bytes, int max_bytes);
void oracle_treelets_free(oracle_treelets* t);
const char* oracle_last_error(void);

/* Sizes: *n_treelets and *n_members. */
void oracle_treelets_sizes(const oracle_treelets* t, uint32_t* n_treelets, uint64_t* n_members);
/* Same layout as rt_treelets_get (any pointer may be NULL). */
void oracle_treelets_get(const oracle_treelets* t, uint64_t n_units, uint32_t* roots, uint64_t* member_first,
                         uint32_t* members, uint16_t* member_bytes, uint32_t* node_root);
/* remapBVHToTreeletLayout (:1473-1509).  Returns 0, or -1 where the reference asserts. */
int oracle_remap(const oracle_treelets* t, int max_bytes, uint32_t stride, uint64_t n_units, uint64_t* new_addr);

/* Traces n rays with traceRay (mode 0, :2309-3076) or traceRayWithTreelets
 * (mode 1, :1522-2307, device_offset = 0; mode 2, the same with a nonzero
 * device_offset, where every child after the first node goes to the
 * other-treelet stack).  `tl` is required for modes 1 and 2 and for treelet
 * traces.
 * visits / treelets / capacity follow rt_trace_buf.  threads <= 1 runs on the
 * calling thread, otherwise contiguous ray ranges per std::thread.
 * Returns 0 or -1 (message in oracle_last_error). */
int oracle_trace(const uint8_t* blob, uint64_t n_bytes, const oracle_treelets* tl, const rt_ray* rays,
                 const uint32_t* flags, uint32_t default_flags, uint64_t n, int mode, rt_hit* hits, uint32_t* visits,
                 uint32_t* treelets, uint32_t capacity, int threads);

/* oracle_trace that also writes, per ray, the largest sizes its stacks
 * reached (peaks[2 r], peaks[2 r + 1]): traceRay's stack and 0, or
 * traceRayWithTreelets' current-treelet and other-treelet stacks.  The
 * reference's lists are unbounded; the tests use these sizes to predict which
 * rays exceed the library's bounded stacks.  peaks may be NULL. */
int oracle_trace_peaks(const uint8_t* blob, uint64_t n_bytes, const oracle_treelets* tl, const rt_ray* rays,
                       const uint32_t* flags, uint32_t default_flags, uint64_t n, int mode, rt_hit* hits,
                       uint32_t* visits, uint32_t* treelets, uint32_t capacity, uint32_t* peaks, int threads);

/* Treelet-prefetch decision of one RT unit (shader.cc:3419-3633 and the
 * second-treelet step :3645-3683).  next_unit holds each resident lane's next
 * access (unit index) or 0xFFFFFFFF.  State and decision use the library's
 * structs (treelet_rt.h). */
int oracle_prefetch_decide(const oracle_treelets* tl, const uint32_t* next_unit, uint32_t lanes,
                           const rt_prefetch_params* p, rt_prefetch_state* state, rt_prefetch_decision* out);

/* The same with two switches: queue_variant 1 runs the copy of the decision
 * that the pipelined treelet queue uses (shader.cc:3780-3932: no second
 * prefetch, only the last prefetched treelet suppressed, heuristic 3 sized at
 * half the treelet), 2 the copy the treelet queue uses (shader.cc:4020-4060:
 * the whole most popular treelet unless it was the last prefetched one, for
 * every heuristic); flush 1 clears the queue before a new treelet's chunks
 * (-flush_prefetch_queue_on_new_treelet; not in the treelet queue's copy). */
int oracle_prefetch_decide_ex(const oracle_treelets* tl, const uint32_t* next_unit, uint32_t lanes,
                              const rt_prefetch_params* p, rt_prefetch_state* state, rt_prefetch_decision* out,
                              uint32_t queue_variant, uint32_t flush);

/* The RT-unit trace replay of rt_unit_replay (treelet_rt.h), restated with
 * the reference's containers: a std::deque prefetch queue erased in place,
 * per-block vectors of prefetch records classified as gpu-cache.cc:1953-2116
 * does, std::map histograms through oracle_prefetch_decide, std::map stride
 * tables.  max_treelet_bytes sizes the metadata (vulkan_ray_tracing.cc:1601-1602).
 * stats: n_rt_units records.  Returns 0 or -1. */
int oracle_unit_replay(const oracle_treelets* tl, int max_treelet_bytes, uint64_t blob_bytes, const rt_hit* hits,
                       const uint32_t* visits, uint32_t n, uint32_t capacity, const rt_unit_config* cfg,
                       rt_unit_stats* stats, int threads);

/* The RT unit's warp selection (rt_unit::schedule_next_warp, shader.cc:4307-4392)
 * over n resident warps in uid order, as the replay uses it: ready[i] is
 * !is_stalled(), next_unit[32 i + lane] the lane's next access (unit index)
 * or 0xFFFFFFFF, last_prefetched a root unit or 0xFFFFFFFF.  Returns the
 * chosen position or -1. */
int oracle_schedule_warp(const oracle_treelets* tl, uint32_t scheduler, uint32_t treelet_prefetch,
                         uint32_t last_prefetched, uint32_t n, const uint8_t* ready, const uint32_t* next_unit);

/* A stream of demand accesses through one Lee MICRO'10 stride prefetcher and
 * its prefetch queue (shader.cc:4779-4828), as the replay drives them: the
 * queue starts with `prefill` entries (request = base = 32 (i + 1)); per
 * event k, pops[k] entries leave the queue front, the queued copies of
 * next_addr[k] are removed and warp_id[k]'s stride tables train on it and may
 * queue two prefetches.  out (uint64), per event: removed, appended, per
 * appended entry (request, base), queue length.  Returns the words written,
 * or -1 when out_cap is too small. */
int64_t oracle_stride_events(uint32_t n, const uint32_t* warp_id, const uint64_t* next_addr, const uint32_t* pops,
                             uint32_t max_queue, uint32_t prefill, uint64_t* out, uint64_t out_cap);

/* The end-of-run tally of one RT unit's prefetch records (gpu-sim.cc:1749-1795)
 * as the replay makes it: n records (block address, class 0-5 numbered as
 * prefetch_request_effectiveness); out[0..4] the count per class, out[5] the
 * unclassified-but-accessed count. */
void oracle_prefetch_tally(uint32_t n, const uint64_t* block, const uint8_t* effectiveness, uint64_t* out);

#ifdef __cplusplus
}
#endif
#endif
