// Traversal kernels.
//
//   trace_plain_kernel    traceRay order (vulkan_ray_tracing.cc:2309-3076)
//   trace_treelet_kernel  traceRayWithTreelets order (vulkan_ray_tracing.cc:1522-2307);
//                         with STAGED = true, each CTA votes every epoch on the
//                         treelet most of its rays need next (the treelet-prefetch
//                         decision of shader.cc:3419-3441 with heuristic ALWAYS),
//                         copies that treelet's image into shared memory with
//                         cp.async.bulk, and serves node reads that fall in a
//                         resident treelet from shared memory.  Staging changes
//                         where a node's bytes come from, never which nodes a
//                         ray visits or in which order.
//
// One thread walks one ray, with its stack(s) in local memory.  Each thread
// keeps the reference's visit order exactly; FP32 arithmetic keeps the
// reference's operation order and is compiled without FMA contraction.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/treelet_rt.h"
#include "device_nodes.cuh"
#include "format.h"
#include "rtmath.h"

namespace rtk {

constexpr uint32_t kNone = 0xFFFFFFFFu;
constexpr uint32_t kTop = 2u, kLeaf = 1u;  // stack entry = unit << 2 | top | leaf

// Device counters, all uint64.
enum Stat { ST_NODE_BYTES = 0, ST_STAGED_BYTES, ST_SMEM_READS, ST_GMEM_READS, ST_STAGINGS, ST_COUNT };
// Status word bits set by kernels (device-wide, not per ray).
constexpr uint32_t kStatusTimeout = 1u;

// What a walk needs of one scene.
struct SceneView {
  const uint4* blob;
  const uint2* meta;      // per unit: x = treelet root unit, y = dense << 10 | slot
  const uint16_t* route;  // per unit: routing bits of the treelet-ordered walk (treelets.h)
  uint32_t n_units;
};

struct TraceArgs {
  const uint4* blob;
  uint32_t n_units;
  // several scenes in one launch: rays [item_begin[k], item_begin[k+1]) use
  // scenes[item_scene[k]]; n_items == 0 means every ray uses blob / meta
  const SceneView* scenes;
  const uint32_t* item_begin;
  const uint32_t* item_scene;
  uint32_t n_items;
  const rt_ray* rays;
  const uint32_t* flags;
  uint32_t default_flags;
  uint32_t n;
  rt_hit* hits;
  uint32_t* visits;
  uint32_t* tl_trace;
  uint32_t cap;
  const uint2* meta;           // per unit: x = treelet root unit, y = dense << 10 | slot
  const uint16_t* route;       // per unit: routing bits of the treelet-ordered walk
  const uint4* pin_image;      // staged: pinned-treelet records (pinned.h), copied to shared memory per CTA
  uint32_t pin_bytes;          // its size (multiple of 128), 0 = nothing pinned
  uint32_t pin_root;           // record of the TLAS root node, 0 = not pinned
  const uint4* images;         // staged image store
  const unsigned long long* image_off;  // per dense treelet, n_treelets + 1
  uint32_t n_treelets;
  unsigned long long* stats;   // ST_COUNT counters
  uint32_t* status;            // kStatus* bits
  uint32_t slots;              // staged treelet slots per CTA
  uint32_t slot_bytes;         // bytes per slot (multiple of 128)
  uint32_t epoch;              // node visits per ray between votes
  uint32_t* queue;             // next ray to hand out (persistent kernels; zeroed per launch)
  uint32_t refill;             // idle lanes of a warp that trigger a refill
  uint32_t min_votes;          // lanes that must want a treelet before a warp stages it
  const uint32_t* hint;        // staged: predicted next treelet per (treelet, direction octant), or null
  uint32_t wait_tries;         // staged: probes of the wait for the pinned image before staging stops
  uint32_t tbuf_off;           // plain walk: byte offset of the trace staging area in dynamic shared
                               // memory (128-aligned base), kNone: trace entries go straight to the rows
  uint32_t ss_off;             // plain walk with SHORT: byte offset of the short stacks, likewise
};

// Trace staging (the plain walk).  A lane writing its ray's trace rows one
// 4-byte entry at a time leaves partly written 32-byte sectors that L2 fills
// from DRAM and writes back again and again (4.5x the entries' bytes
// written, as many read, on bounce rays).  Instead each lane keeps its ray's
// next 8 entries of each row in its warp's 2 KiB staging area ([visit |
// treelet][entry 0..7][lane] words: lanes hit distinct banks) and writes them
// as one whole, aligned sector.  Used when the row capacity is a multiple of
// 8 and the rows start on 32-byte boundaries; the last partial sector is
// written when the ray ends.
constexpr uint32_t kTraceBufWarpBytes = 2048;

extern __shared__ __align__(128) uint8_t rt_dyn_smem[];

// The calling lane's entry 0 of its warp's staging area.
__device__ __forceinline__ uint32_t* trace_buf(uint32_t off) {
  uint8_t* base = rt_dyn_smem + ((128u - ((uint32_t)__cvta_generic_to_shared(rt_dyn_smem) & 127u)) & 127u);
  return reinterpret_cast<uint32_t*>(base + off + (threadIdx.x >> 5) * kTraceBufWarpBytes) + (threadIdx.x & 31u);
}

// Entry n (< capacity) of a ray's visit and treelet rows (either row may be null).
__device__ __forceinline__ void trace_put(const TraceArgs& a, uint32_t* vrow, uint32_t* trow, uint32_t n, uint32_t vis,
                                          uint32_t tl) {
  if (a.tbuf_off == kNone) {
    if (vrow) vrow[n] = vis;
    if (trow) trow[n] = tl;
    return;
  }
  uint32_t* b = trace_buf(a.tbuf_off);
  const uint32_t j = n & 7u;
  if (vrow) b[j * 32] = vis;
  if (trow) b[256 + j * 32] = tl;
  if (j == 7u) {
    if (vrow) {
      uint4* d = reinterpret_cast<uint4*>(vrow + (n - 7u));
      __stcs(d, make_uint4(b[0], b[32], b[64], b[96]));
      __stcs(d + 1, make_uint4(b[128], b[160], b[192], b[224]));
    }
    if (trow) {
      uint4* d = reinterpret_cast<uint4*>(trow + (n - 7u));
      __stcs(d, make_uint4(b[256], b[288], b[320], b[352]));
      __stcs(d + 1, make_uint4(b[384], b[416], b[448], b[480]));
    }
  }
}

// Writes the staged entries of a ray's last partial sector; m = entries
// recorded (at most the capacity).
__device__ __forceinline__ void trace_drain(const TraceArgs& a, uint32_t* vrow, uint32_t* trow, uint32_t m) {
  const uint32_t k = m & 7u;
  if (a.tbuf_off == kNone || k == 0) return;
  const uint32_t* b = trace_buf(a.tbuf_off);
  const uint32_t base = m - k;
  for (uint32_t j = 0; j < k; ++j) {
    if (vrow) vrow[base + j] = b[j * 32];
    if (trow) trow[base + j] = b[256 + j * 32];
  }
}

struct Recorder {
  uint32_t* vrow;
  uint32_t* trow;
  uint32_t cap;
  uint32_t n;
  uint32_t bytes;
  const uint2* meta;
  // TRACED = false: a launch without traces, whose walk only counts.
  template <bool TRACED>
  __device__ __forceinline__ void rec(const TraceArgs& a, uint32_t unit, uint32_t type) {
    if (TRACED && n < cap) trace_put(a, vrow, trow, n, rtf::pack_visit(unit, type), trow ? meta[unit].x : 0u);
    n++;
    bytes += rtf::tx_bytes(type);
  }
};

__device__ __forceinline__ void load_ray(const rt_ray* rays, uint32_t r, rtm::V3& o, float& tmin, rtm::V3& d,
                                         float& tmax) {
  const float4* p = reinterpret_cast<const float4*>(rays + r);
  const float4 a = __ldg(p), b = __ldg(p + 1);
  o = rtm::v3(a.x, a.y, a.z);
  tmin = a.w;
  d = rtm::v3(b.x, b.y, b.z);
  tmax = b.w;
}

// The scene ray r walks.  MULTI = false compiles a launch over one scene,
// whose tables are the launch arguments themselves.
template <bool MULTI>
__device__ __forceinline__ SceneView scene_of(const TraceArgs& a, uint32_t r) {
  if (!MULTI || a.n_items == 0) return SceneView{a.blob, a.meta, a.route, a.n_units};
  uint32_t lo = 0, hi = a.n_items;  // last item with item_begin <= r
  while (hi - lo > 1) {
    const uint32_t mid = (lo + hi) >> 1;
    if (__ldg(a.item_begin + mid) <= r) lo = mid;
    else hi = mid;
  }
  const SceneView* s = a.scenes + __ldg(a.item_scene + lo);
  SceneView v;
  v.blob = reinterpret_cast<const uint4*>(__ldg(reinterpret_cast<const unsigned long long*>(&s->blob)));
  v.meta = reinterpret_cast<const uint2*>(__ldg(reinterpret_cast<const unsigned long long*>(&s->meta)));
  v.route = reinterpret_cast<const uint16_t*>(__ldg(reinterpret_cast<const unsigned long long*>(&s->route)));
  v.n_units = __ldg(&s->n_units);
  return v;
}

// Hit record from the closest leaf / instance (vulkan_ray_tracing.cc:2990-3028).
__device__ __forceinline__ void write_hit(const TraceArgs& a, const SceneView& v, uint32_t r, bool hit, float min_thit, rtm::V3 O,
                                          rtm::V3 D, float tmin, float tmax, uint32_t c_leaf, uint32_t c_inst,
                                          float c_tobj, const Recorder& rec, uint32_t status) {
  rt_hit h;
  h.hit_geometry = 0;
  h.geometry_index = 0;
  h.primitive_index = 0;
  h.instance_index = 0;
  h.world_min_thit = 0.0f;
  h.barycentric[0] = h.barycentric[1] = h.barycentric[2] = 0.0f;
  h.intersection_point[0] = h.intersection_point[1] = h.intersection_point[2] = 0.0f;
  h.closest_leaf = 0;
  h.closest_instance = 0;
  h.reserved = 0;
  if (hit) {
    rtd::Node64 q;
    rtd::load64(v.blob + (uint64_t)c_leaf * 4, 0, q);
    rtd::Instance in;
    rtd::load_instance(v.blob + (uint64_t)c_inst * 4, 0, in);
    const rtm::ObjRay orr = rtm::make_transformed_ray(in.w2o, O, D, tmin, tmax);
    h.hit_geometry = 1;
    h.geometry_index = rtf::geometry_index_of(q.w[1]);
    h.primitive_index = q.w[2];
    h.instance_index = in.instance_id;
    h.world_min_thit = min_thit;
    h.intersection_point[0] = O.x + D.x * min_thit;
    h.intersection_point[1] = O.y + D.y * min_thit;
    h.intersection_point[2] = O.z + D.z * min_thit;
    const rtm::V3 p = rtm::v3(orr.o.x + orr.d.x * c_tobj, orr.o.y + orr.d.y * c_tobj, orr.o.z + orr.d.z * c_tobj);
    const rtm::V3 v0 = rtm::v3(__uint_as_float(q.w[4]), __uint_as_float(q.w[5]), __uint_as_float(q.w[6]));
    const rtm::V3 v1 = rtm::v3(__uint_as_float(q.w[7]), __uint_as_float(q.w[8]), __uint_as_float(q.w[9]));
    const rtm::V3 v2 = rtm::v3(__uint_as_float(q.w[10]), __uint_as_float(q.w[11]), __uint_as_float(q.w[12]));
    const rtm::V3 b = rtm::barycentric(p, v0, v1, v2);
    h.barycentric[0] = b.x;
    h.barycentric[1] = b.y;
    h.barycentric[2] = b.z;
    h.closest_leaf = c_leaf;
    h.closest_instance = c_inst;
  }
  h.n_visits = rec.n;
  h.status = status | (rec.cap && rec.n > rec.cap ? RT_RAY_TRACE_OVERFLOW : 0u);
  a.hits[r] = h;
}

// Object-space ray of one instance (make_transformed_ray).
struct InstCtx {
  uint32_t unit;
  rtm::V3 o, d, idir;
  float tmin, tmax, mult;
};

__device__ __forceinline__ void enter_instance(const rtd::Instance& in, uint32_t unit, rtm::V3 O, rtm::V3 D, float tmin,
                                               float tmax, InstCtx& c) {
  const rtm::ObjRay r = rtm::make_transformed_ray(in.w2o, O, D, tmin, tmax);
  c.unit = unit;
  c.o = r.o;
  c.d = r.d;
  c.tmin = r.tmin;
  c.tmax = r.tmax;
  c.mult = r.mult;
  c.idir = rtm::calculate_idir(r.d);
}

// Adds v summed over the calling warp's active lanes with one atomic.
__device__ __forceinline__ void add_warp_total(unsigned long long* dst, uint32_t v) {
  const uint32_t mask = __activemask();
  const uint32_t sum = __reduce_add_sync(mask, v);
  if ((threadIdx.x & 31u) == (uint32_t)(__ffs(mask) - 1)) atomicAdd(dst, (unsigned long long)sum);
}

// The same for 64-bit values; all 32 lanes must call it.
__device__ __forceinline__ void add_warp_total64(unsigned long long* dst, unsigned long long v) {
#pragma unroll
  for (int s = 16; s > 0; s >>= 1) v += __shfl_xor_sync(0xffffffffu, v, s);
  if ((threadIdx.x & 31u) == 0) atomicAdd(dst, v);
}

// Finds a ray for every idle lane of the warp (one atomic per refill) and
// runs each lane's walker one node visit per iteration.  A lane that finishes
// its ray gets a new one as soon as `refill` lanes of its warp are idle, so
// warps stay full while rays of very different lengths finish (persistent
// threads with dynamic ray fetch).  Every ray's own visit order is unchanged.
template <class W>
__device__ __forceinline__ void run_persistent(const TraceArgs& a, W& w, unsigned long long& bytes_out) {
  const uint32_t lane = threadIdx.x & 31u;
  bool have = false, exhausted = false;
  uint32_t r = 0;
  unsigned long long bytes = 0;
  for (;;) {
    const uint32_t need = __ballot_sync(0xffffffffu, !have);
    if (!exhausted && need && (__popc(need) >= (int)a.refill || need == 0xffffffffu)) {
      const int leader = __ffs(need) - 1;
      uint32_t base = 0;
      if ((int)lane == leader) base = atomicAdd(a.queue, (uint32_t)__popc(need));
      base = __shfl_sync(0xffffffffu, base, leader);
      if (base + (uint32_t)__popc(need) >= a.n) exhausted = true;
      if (!have) {
        const uint32_t rr = base + (uint32_t)__popc(need & ((1u << lane) - 1u));
        if (rr < a.n) {
          r = rr;
          w.init(a, r);
          have = true;
          if (!w.active()) {
            w.finish(a, r);
            bytes += w.rec.bytes;
            have = false;
          }
        }
      }
    }
    if (!__any_sync(0xffffffffu, have)) {
      if (exhausted) break;
      continue;
    }
    if (have) {
      w.step(a, r);
      if (!w.active()) {
        w.finish(a, r);
        bytes += w.rec.bytes;
        have = false;
      }
    }
  }
  bytes_out = bytes;
}

// ----------------------------------------------------------------- plain

// A ray's traceRay walk (vulkan_ray_tracing.cc:2309-3076) as a sequence of
// node visits.  One LIFO stack of unit << 2 | top | leaf entries; `next` is
// the internal node descended next (the first hit internal child, :2570-2578);
// leaves and further children are pushed.  A top-level instance leaf is
// followed by its whole BLAS before the next top-level entry (:2602-2679).
// The warp-synchronous short stack (SHORT): entries 0..kShortStack-1 of each
// ray's stack in its warp's shared memory, entry k of the warp's 32 rays in
// one 128-byte row (lane l in bank l, so a warp's pushes and pops at any mix
// of depths never conflict), the deeper entries in the local-memory stack.
constexpr int kShortStack = 16;
constexpr uint32_t kShortStackWarpBytes = kShortStack * 32 * 4;

// TRACED = false compiles the walk of a launch without traces (no trace
// code at all); TRACED = true writes the rows.  SHORT keeps the bottom of the
// stack in shared memory (rt_tuning.short_stack).
template <int CAP, bool MULTI, bool TRACED, bool SHORT = false>
struct PlainWalker {
  rtm::V3 O, D, idir;
  float tmin, tmax, min_thit, c_tobj;
  bool opaque, terminate, inblas, fast;
  uint32_t next, c_leaf, c_inst, status;
  int sp;
  uint32_t stk[CAP];
  InstCtx ic;
  bool ic_fast;
  Recorder rec;
  SceneView v;

  __device__ __forceinline__ bool active() const { return next != kNone || sp > 0; }


  // entry i of the stack (the short stack's rows for i < kShortStack)
  __device__ __forceinline__ uint32_t* slot(const TraceArgs& a, int i) {
    if (SHORT && i < kShortStack) {
      uint8_t* base = rt_dyn_smem + ((128u - ((uint32_t)__cvta_generic_to_shared(rt_dyn_smem) & 127u)) & 127u);
      return reinterpret_cast<uint32_t*>(base + a.ss_off + (threadIdx.x >> 5) * kShortStackWarpBytes) +
             i * 32 + (threadIdx.x & 31u);
    }
    return stk + i;
  }
  __device__ __forceinline__ void push(const TraceArgs& a, uint32_t e) {
    if (sp < CAP) *slot(a, sp++) = e;
    else status |= RT_RAY_STACK_OVERFLOW;
  }
  __device__ __forceinline__ uint32_t pop(const TraceArgs& a) { return *slot(a, --sp); }

  __device__ __forceinline__ void init(const TraceArgs& a, uint32_t r) {
    v = scene_of<MULTI>(a, r);
    load_ray(a.rays, r, O, tmin, D, tmax);
    const uint32_t flags = a.flags ? a.flags[r] : a.default_flags;
    terminate = flags & rtf::RAY_FLAG_TERMINATE_ON_FIRST_HIT;
    opaque = flags & rtf::RAY_FLAG_OPAQUE;
    rec = Recorder{a.visits ? a.visits + (uint64_t)r * a.cap : nullptr,
                   a.tl_trace ? a.tl_trace + (uint64_t)r * a.cap : nullptr, a.cap, 0u, 0u, v.meta};
    status = 0;
    sp = 0;
    next = kNone;
    inblas = false;
    min_thit = tmax;
    c_leaf = c_inst = 0;
    c_tobj = 0.0f;
    ic.unit = kNone;
    ic_fast = false;
    idir = rtm::calculate_idir(D);
    fast = rtd::finite_ray(O, D, tmin, tmax);
    rec.rec<TRACED>(a, 0, rtf::TX_STRUCTURE);
    const uint4 h0 = __ldg(v.blob), h1 = __ldg(v.blob + 1);
    const uint64_t root_off = (uint64_t)h0.x | ((uint64_t)h0.y << 32);
    const rtm::V3 bmin = rtm::v3(__uint_as_float(h0.z), __uint_as_float(h0.w), __uint_as_float(h1.x));
    const rtm::V3 bmax = rtm::v3(__uint_as_float(h1.y), __uint_as_float(h1.z), __uint_as_float(h1.w));
    float th;
    if (rtm::ray_box_test(bmin, bmax, idir, O, tmin, tmax, th)) push(a, ((uint32_t)(root_off >> 6) << 2) | kTop);
  }

  __device__ __forceinline__ void stop(uint32_t bits) {
    status |= bits;
    sp = 0;
    next = kNone;
  }

  __device__ __forceinline__ void visit_internal(const TraceArgs& a, uint32_t unit, const rtd::Node64& nd) {
    // one box test for both levels (the world ray, or the instance's object
    // ray with the culling distance scaled into object space): lanes at TLAS
    // and BLAS nodes run it together
    const bool f = inblas ? ic_fast : fast;
    const rtm::V3 o = inblas ? ic.o : O, id = inblas ? ic.idir : idir;
    const float t0 = inblas ? ic.tmin : tmin, t1 = inblas ? ic.tmax : tmax;
    const float cull = inblas ? min_thit * ic.mult : min_thit;
    const rtd::ChildHits ch = f ? rtd::test_children<true>(nd, unit, o, id, t0, t1, cull)
                                : rtd::test_children<false>(nd, unit, o, id, t0, t1, cull);
    const uint32_t level = inblas ? 0u : kTop;
    uint32_t c = ch.child_unit, nn = kNone;
#pragma unroll
    for (int i = 0; i < 6; ++i) {
      // the first hit internal child becomes `next`; other hit children are
      // pushed (one predicated store, no branch per child)
      const uint32_t info = ch.info_of(i);
      const bool h = (ch.hit_mask >> i) & 1u, internal = (info >> 2) == rtf::CT_INTERNAL;
      const bool take = h && internal && nn == kNone, store = h && !take, ok = sp < CAP;
      if (store && ok) *slot(a, sp) = (c << 2) | level | (internal ? 0u : kLeaf);
      if (store && !ok) status |= RT_RAY_STACK_OVERFLOW;
      sp += (store && ok) ? 1 : 0;
      nn = take ? c : nn;
      c += info & 3u;
    }
    next = nn;
    if (status & RT_RAY_STACK_OVERFLOW) stop(0);
  }

  // Returns the transaction type of the leaf's second record.
  __device__ __forceinline__ uint32_t visit_leaf(const TraceArgs& a, uint32_t unit, const rtd::Node64& q) {
    if (rtf::leaf_type_of(q.w[1]) == 0) {
      const rtm::V3 v0 = rtm::v3(__uint_as_float(q.w[4]), __uint_as_float(q.w[5]), __uint_as_float(q.w[6]));
      const rtm::V3 v1 = rtm::v3(__uint_as_float(q.w[7]), __uint_as_float(q.w[8]), __uint_as_float(q.w[9]));
      const rtm::V3 v2 = rtm::v3(__uint_as_float(q.w[10]), __uint_as_float(q.w[11]), __uint_as_float(q.w[12]));
      float t = 0.0f;
      const bool hit = rtm::ray_triangle_test(v0, v1, v2, ic.o, ic.d, t);
      const float wt = t / ic.mult;
      if (hit && tmin <= wt && wt <= tmax) {  // :2843-2859
        if (opaque && wt < min_thit) min_thit = t / ic.mult;
        c_leaf = unit;
        c_inst = ic.unit;
        c_tobj = t;
        if (terminate) sp = 0;
        return rtf::TX_QUAD_LEAF_HIT;
      }
      return rtf::TX_QUAD_LEAF;
    }
    status |= RT_RAY_HIT_PROCEDURAL;
    return rtf::TX_PROCEDURAL_LEAF;
  }

  // Returns the unit of the instance's second record (its BLAS header), or
  // kNone when the header lies outside the blob.
  __device__ __forceinline__ uint32_t visit_instance(const TraceArgs& a, uint32_t unit, const rtd::Node64& q) {
    rtd::Instance in;
    rtd::instance_from(q, v.blob + (uint64_t)unit * 4, 0, in);
    const uint64_t hdr = (uint64_t)unit * 64 + in.bvh_address;
    if ((hdr & 63) || hdr / 64 >= v.n_units) {
      stop(RT_RAY_BAD_NODE);
      return kNone;
    }
    const uint4 h0 = __ldg(v.blob + (hdr >> 4));
    const uint64_t broot = hdr + ((uint64_t)h0.x | ((uint64_t)h0.y << 32));
    enter_instance(in, unit, O, D, tmin, tmax, ic);
    ic_fast = rtd::finite_ray(ic.o, ic.d, ic.tmin, ic.tmax);
    push(a, (uint32_t)(broot >> 6) << 2);
    inblas = true;
    if (status & RT_RAY_STACK_OVERFLOW) stop(0);
    return (uint32_t)(hdr >> 6);
  }

  // One node visit (the caller checks active() first).  The node to visit is
  // found first and its first 64 bytes loaded once for every kind, so a
  // warp's lanes at internal nodes, leaves and instance leaves issue one load.
  __device__ __forceinline__ void step(const TraceArgs& a) {
    uint32_t unit, kind;  // 0 internal node, 1 primitive leaf, 2 instance leaf
    for (;;) {
      if (next != kNone) {
        unit = next;
        kind = 0;
        break;
      }
      if (inblas) {
        if (sp > 0 && !(*slot(a, sp - 1) & kTop)) {
          const uint32_t e = pop(a);
          if (e & kLeaf) {
            unit = e >> 2;
            kind = 1;
            break;
          }
          next = e >> 2;
          continue;
        }
        inblas = false;
        continue;
      }
      if (sp == 0) return;
      const uint32_t e = pop(a);
      if (!(e & kLeaf)) {
        next = e >> 2;
        continue;
      }
      unit = e >> 2;
      kind = 2;
      break;
    }
    if (unit + (kind == 2 ? 1u : 0u) >= v.n_units) return stop(RT_RAY_BAD_NODE);
    rtd::Node64 q;
    rtd::load64(v.blob + (uint64_t)unit * 4, 0, q);
    // a visit records one or two transactions; two call sites for all kinds
    // keep the recording code (staged through shared memory) out of every
    // branch
    rec.rec<TRACED>(a, unit, kind == 0 ? rtf::TX_INTERNAL : (kind == 1 ? rtf::TX_LEAF_DESC : rtf::TX_INSTANCE_LEAF));
    uint32_t unit2 = unit, type2 = rtf::TX_STRUCTURE;
    if (kind == 0) {
      visit_internal(a, unit, q);
      unit2 = kNone;
    } else if (kind == 1) {
      type2 = visit_leaf(a, unit, q);
    } else {
      unit2 = visit_instance(a, unit, q);
    }
    if (unit2 != kNone) rec.rec<TRACED>(a, unit2, type2);
  }

  // (the walk keeps its own rows in the recorder; the ray index is not needed)
  __device__ __forceinline__ void step(const TraceArgs& a, uint32_t) { step(a); }

  __device__ __forceinline__ void finish(const TraceArgs& a, uint32_t r) {
    const bool bad = status & (RT_RAY_STACK_OVERFLOW | RT_RAY_BAD_NODE);
    if (TRACED) trace_drain(a, rec.vrow, rec.trow, min(rec.n, rec.cap));
    write_hit(a, v, r, !bad && (min_thit < tmax), min_thit, O, D, tmin, tmax, c_leaf, c_inst, c_tobj, rec, status);
  }
};

// The plain walk keeps its stack inside the walker, whose fields the compiler
// then leaves in local memory: 48 registers and five 256-thread CTAs per SM
// (the launch bound holds it there: with the trace staging the compiler
// would take 54 registers and fit four CTAs, 2-8% slower untraced and 7%
// slower traced on bounce rays).
// Its fields in registers (90, or capped at 51-85 with spills) measured
// 40-45% slower, while the treelet walks gained from them (below).
template <int CAP, bool MULTI, bool TRACED, bool SHORT = false>
__global__ void __launch_bounds__(256, 5) trace_plain_kernel(TraceArgs a) {
  PlainWalker<CAP, MULTI, TRACED, SHORT> w;
  unsigned long long bytes = 0;
  run_persistent(a, w, bytes);
  if (a.stats) add_warp_total64(a.stats + ST_NODE_BYTES, bytes);
}

}  // namespace rtk
