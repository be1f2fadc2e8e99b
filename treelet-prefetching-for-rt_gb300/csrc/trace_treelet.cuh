// Treelet-ordered traversal (traceRayWithTreelets, vulkan_ray_tracing.cc:1522-2307)
// and its shared-memory staged variant.
#pragma once
#include "pinned.h"
#include "trace_kernels.cuh"

namespace rtk {

constexpr uint32_t kSlotBitsDev = 10;
// Stack entry of the treelet-ordered walk, low word:
//   unit << 3 | top | leaf          node in global memory
//   soff << 3 | kEPin | top | leaf  node held as a pinned record in shared memory
// high word: the instance leaf a bottom-level node belongs to.
constexpr uint32_t kEShift = 3, kEPin = 4;
constexpr uint32_t kRouteOther = 6, kRouteInst = 12;  // route bits (treelets.h)

// A ray's treelet-ordered walk.  Two LIFO stacks as in the reference
// (push_front / pop_front on std::list, :1708-1709): `cu` holds nodes of the
// current treelet, `ot` the rest (:1821-1856).  Both live in one local
// array (cu at [0, CAP), ot at [CAP, 2 CAP)), so that a push goes to either
// with one predicated store instead of a branch per child.  Which stack a child goes to
// is read from the per-node route bits (treelets.h): a node popped from `cu`
// is in the current treelet, and a node popped from `ot` becomes the current
// treelet root, so the reference's addrToTreeletID comparison is fixed per
// node and precomputed.  The staged location of a node (dense treelet << 10 |
// 64-byte slot in that treelet's image) is read from the node table when a
// warp has a staged slot; pinned nodes are named by their record.
//
// Fields a step rarely needs live in the tail of the stack array, in local
// memory, instead of registers (kColdWords 64-bit words after the 2 CAP stack
// entries): the world direction, the closest hit and, in the unstaged walk,
// the world origin and inverse direction, which only TLAS nodes and instance
// entries read.  The trace rows are found from the ray index, which the
// kernel's loop holds anyway, instead of from the tail (two local loads per
// recorded transaction before).  Fewer live registers let the treelet
// walk run four CTAs per SM at 64 registers: +5% on bounce rays, +2% on
// primary rays; the staged walk, with its pinned-record state, measured best
// with the world ray in registers at three CTAs per SM.
constexpr int kColdWords = 7;

// SLAB = true keeps the other-treelet stack in a per-ray slab of global
// memory (`ot`, CAP entries) instead of the local array, so that a ray can
// stop between treelets and go on later in another thread: the treelet-queued
// walk (trace_queued.cuh).  The local array then holds only the current
// stack and the cold tail.
// TRACED = false compiles the walk of a launch without traces (no trace code
// at all).
template <int CAP, bool STAGED, bool MULTI, bool SLAB = false, bool TRACED = true>
struct Walker {
  static constexpr bool kColdWorld = !STAGED;
  static constexpr int kOtLocal = SLAB ? 0 : CAP;  // other-stack entries in the local array
  rtm::V3 O, idir;  // world ray (registers only when !kColdWorld)
  float tmin, tmax, min_thit;
  bool terminate, fast, ic_fast;  // FAST min/max allowed for the world / object ray
  uint32_t status;
  unsigned long long* stk;  // CAP + kOtLocal + kColdWords entries, a local array of the kernel
  unsigned long long* ot;   // SLAB: the ray's other-treelet stack in global memory
  int ncu, not_;            // entries on cu and on ot
  // The top of `cu` when it was pushed by the previous node visit: the node
  // the walk pops next, kept in a register instead of a local-memory round
  // trip (0 = none; no stack entry is 0, a blob's unit 0 is its TLAS header).
  unsigned long long nxt;
  InstCtx ic;
  // Visit recording: the counts in registers, the trace rows in the cold tail.
  struct Counts {
    uint32_t cap, n, bytes;
  } rec;
  SceneView v;
  uint32_t smem_reads, gmem_reads;
  uint32_t pin_base;  // shared address of the pinned records, 0 = none
  uint32_t pin_root;  // record of the TLAS root node, 0 = not pinned

  __device__ __forceinline__ bool active() const { return nxt != 0 || (ncu | not_) != 0; }

  __device__ __forceinline__ void clear() {
    nxt = 0;
    ncu = not_ = 0;
  }

  // ---- the cold tail: stk[CAP + kOtLocal + k]
  __device__ __forceinline__ unsigned long long& cold(int k) const { return stk[CAP + kOtLocal + k]; }
  // ---- entry i of the other-treelet stack
  __device__ __forceinline__ unsigned long long& ot_at(int i) const { return SLAB ? ot[i] : stk[CAP + i]; }
  static __device__ __forceinline__ unsigned long long pack(float a, float b) {
    return (unsigned long long)__float_as_uint(a) | ((unsigned long long)__float_as_uint(b) << 32);
  }
  static __device__ __forceinline__ float lo(unsigned long long w) { return __uint_as_float((uint32_t)w); }
  static __device__ __forceinline__ float hi(unsigned long long w) { return __uint_as_float((uint32_t)(w >> 32)); }
  __device__ __forceinline__ void set_dir(rtm::V3 d) {
    cold(0) = pack(d.x, d.y);
    cold(1) = pack(d.z, 0.0f);
  }
  __device__ __forceinline__ rtm::V3 dir() const {
    const unsigned long long a = cold(0), b = cold(1);
    return rtm::v3(lo(a), hi(a), lo(b));
  }
  __device__ __forceinline__ void set_hit(uint32_t leaf, uint32_t inst, float tobj) {
    cold(2) = (unsigned long long)leaf | ((unsigned long long)inst << 32);
    cold(3) = pack(tobj, 0.0f);
  }
  __device__ __forceinline__ void set_world(rtm::V3 o, rtm::V3 id) {
    if (kColdWorld) {
      cold(4) = pack(o.x, o.y);
      cold(5) = pack(o.z, id.x);
      cold(6) = pack(id.y, id.z);
    } else {
      O = o;
      idir = id;
    }
  }
  __device__ __forceinline__ rtm::V3 world_o() const {
    if (!kColdWorld) return O;
    const unsigned long long a = cold(4), b = cold(5);
    return rtm::v3(lo(a), hi(a), lo(b));
  }
  __device__ __forceinline__ rtm::V3 world_idir() const {
    if (!kColdWorld) return idir;
    const unsigned long long b = cold(5), c = cold(6);
    return rtm::v3(hi(b), lo(c), hi(c));
  }
  // one visit of the trace (the reference's MemoryTransactionRecord)
  // The rows are written entry by entry: staging them through shared memory
  // as the plain walk does measured 15-30% slower here (eight inlined
  // copies of the staging code in the traced walk).
  __device__ __forceinline__ void record(const TraceArgs& a, uint32_t r, uint32_t unit, uint32_t type) {
    if (TRACED && rec.n < rec.cap) {
      const uint64_t at = (uint64_t)r * a.cap + rec.n;
      if (a.visits) a.visits[at] = rtf::pack_visit(unit, type);
      if (a.tl_trace) a.tl_trace[at] = v.meta[unit].x;
    }
    rec.n++;
    rec.bytes += rtf::tx_bytes(type);
  }

  // Staged location (dense treelet << 10 | slot) of the node the ray visits
  // next, i.e. its first pending access; kNone for a pinned node.
  __device__ __forceinline__ uint32_t next_loc() const {
    unsigned long long e;
    if (nxt) e = nxt;
    else if (ncu > 0) e = stk[ncu - 1];
    else if (not_ > 0) e = ot_at(not_ - 1);
    else return kNone;
    if ((uint32_t)e & kEPin) return kNone;
    const uint32_t unit = (uint32_t)e >> kEShift;
    return unit < v.n_units ? __ldg(reinterpret_cast<const uint32_t*>(v.meta) + 2ull * unit + 1) : kNone;
  }

  __device__ __forceinline__ void push(bool same, uint32_t code, uint32_t inst) {
    const unsigned long long e = (unsigned long long)code | ((unsigned long long)inst << 32);
    // same treelet: e becomes nxt and the previous nxt (if any) goes to cu;
    // else e goes to ot.  One predicated store instead of a branch per child
    // (treelet walk +5% on bounce rays, staged walk +4%).
    const bool store = !same || nxt != 0;
    const int cnt = same ? ncu : not_;
    const bool ok = cnt < CAP;
    if (store && ok) {
      if (SLAB) *(same ? stk + cnt : ot + cnt) = same ? nxt : e;
      else stk[same ? cnt : CAP + cnt] = same ? nxt : e;
    }
    if (store && !ok) status |= RT_RAY_STACK_OVERFLOW;
    ncu += (same && store && ok) ? 1 : 0;
    not_ += (!same && ok) ? 1 : 0;
    nxt = same ? e : nxt;
  }

  __device__ __forceinline__ void bad_node() {
    status |= RT_RAY_BAD_NODE;
    clear();
  }

  __device__ __forceinline__ void init(const TraceArgs& a, uint32_t r) {
    v = scene_of<MULTI>(a, r);
    rtm::V3 o, D;
    load_ray(a.rays, r, o, tmin, D, tmax);
    const uint32_t flags = a.flags ? a.flags[r] : a.default_flags;
    terminate = flags & rtf::RAY_FLAG_TERMINATE_ON_FIRST_HIT;
    rec = Counts{a.cap, 0u, 0u};
    status = 0;
    clear();
    min_thit = tmax;
    set_hit(0, 0, 0.0f);
    set_dir(D);
    ic.unit = kNone;
    smem_reads = gmem_reads = 0;
    const rtm::V3 id = rtm::calculate_idir(D);
    set_world(o, id);
    fast = rtd::finite_ray(o, D, tmin, tmax);
    ic_fast = false;
    record(a, r, 0, rtf::TX_STRUCTURE);
    const uint4 h0 = __ldg(v.blob), h1 = __ldg(v.blob + 1);
    const uint64_t root_off = (uint64_t)h0.x | ((uint64_t)h0.y << 32);
    const rtm::V3 bmin = rtm::v3(__uint_as_float(h0.z), __uint_as_float(h0.w), __uint_as_float(h1.x));
    const rtm::V3 bmax = rtm::v3(__uint_as_float(h1.y), __uint_as_float(h1.z), __uint_as_float(h1.w));
    float th;
    if (rtm::ray_box_test(bmin, bmax, id, o, tmin, tmax, th)) {
      // current_treelet_root starts as the TLAS header, unit 0 (:1707)
      const uint32_t code = ((uint32_t)(root_off >> 6) << kEShift) | kTop;
      const uint32_t unit = code >> kEShift;
      const uint32_t root = unit < v.n_units ? __ldg(&v.meta[unit].x) : kNone;
      push(root == 0u, pin_root ? ((pin_root << kEShift) | kEPin | kTop) : code, 0);
    }
  }

  // ---- the treelet-queued walk (SLAB): a ray's state between two treelets,
  // 64 bytes: the ray (origin, tmin, direction, tmax), then min_thit, status
  // (bit 31: terminate on first hit), transactions and bytes recorded, the
  // closest leaf, its instance, its object-space t, and the other-treelet
  // stack's size.  The current-treelet stack is empty between treelets.
  static constexpr uint32_t kTerminateBit = 0x80000000u;

  __device__ __forceinline__ void save_ray(uint4* st) const {
    const rtm::V3 o = world_o(), d = dir();
    st[0] = make_uint4(__float_as_uint(o.x), __float_as_uint(o.y), __float_as_uint(o.z), __float_as_uint(tmin));
    st[1] = make_uint4(__float_as_uint(d.x), __float_as_uint(d.y), __float_as_uint(d.z), __float_as_uint(tmax));
  }

  __device__ __forceinline__ void suspend(uint4* st) const {
    const unsigned long long h = cold(2);
    st[2] = make_uint4(__float_as_uint(min_thit), status | (terminate ? kTerminateBit : 0u), rec.n, rec.bytes);
    st[3] = make_uint4((uint32_t)h, (uint32_t)(h >> 32), (uint32_t)cold(3), (uint32_t)not_);
  }

  __device__ __forceinline__ void resume(const TraceArgs& a, uint32_t r, const uint4* st) {
    v = scene_of<MULTI>(a, r);
    const uint4 q0 = st[0], q1 = st[1], q2 = st[2], q3 = st[3];
    const rtm::V3 o = rtm::v3(__uint_as_float(q0.x), __uint_as_float(q0.y), __uint_as_float(q0.z));
    const rtm::V3 D = rtm::v3(__uint_as_float(q1.x), __uint_as_float(q1.y), __uint_as_float(q1.z));
    tmin = __uint_as_float(q0.w);
    tmax = __uint_as_float(q1.w);
    min_thit = __uint_as_float(q2.x);
    status = q2.y & ~kTerminateBit;
    terminate = (q2.y & kTerminateBit) != 0;
    rec = Counts{a.cap, q2.z, q2.w};
    cold(2) = (unsigned long long)q3.x | ((unsigned long long)q3.y << 32);
    cold(3) = (unsigned long long)q3.z;
    nxt = 0;
    ncu = 0;
    not_ = (int)q3.w;
    set_dir(D);
    ic.unit = kNone;
    ic_fast = false;
    smem_reads = gmem_reads = 0;
    set_world(o, rtm::calculate_idir(D));
    fast = rtd::finite_ray(o, D, tmin, tmax);
  }

  // True while the walk is inside its current treelet: the next pop would
  // come from the current-treelet stack.
  __device__ __forceinline__ bool in_treelet() const { return nxt != 0 || ncu > 0; }

  // Visits one node; `lookup(unit, meta)` returns the shared-memory address
  // of a node staged in a warp slot, else 0.
  template <class Lookup>
  __device__ __forceinline__ void step(const TraceArgs& a, uint32_t r, Lookup&& lookup) {
    const bool from_cu = nxt != 0 || ncu > 0;  // :1748-1754
    unsigned long long e = nxt;
    if (!nxt) {
      e = SLAB ? (from_cu ? stk[ncu - 1] : ot[not_ - 1]) : stk[from_cu ? ncu - 1 : CAP + not_ - 1];
      ncu -= from_cu ? 1 : 0;
      not_ -= from_cu ? 0 : 1;
    }
    nxt = 0;
    const uint32_t code = (uint32_t)e, inst = (uint32_t)(e >> 32);
    const bool top = code & kTop, leaf = code & kLeaf, pinned = STAGED && (code & kEPin);
    const uint32_t rsh = from_cu ? 0u : 1u;  // which route bit applies
    uint32_t unit, rbits, saddr = 0;
    if (pinned) {
      saddr = pin_base + (code >> kEShift) * 16u;
      unit = rtd::ld_shared_u32(saddr + (leaf ? 0u : rtp::IN_UNIT));
      ++smem_reads;
    } else {
      unit = code >> kEShift;
      if (unit + ((top && leaf) ? 1u : 0u) >= v.n_units) return bad_node();
      if (STAGED) {
        saddr = lookup(unit, v.meta);
        if (saddr) ++smem_reads;
        else ++gmem_reads;
      }
    }
    const uint4* g = v.blob + (uint64_t)unit * 4;
    // the first 64 bytes (or the whole pinned record of an instance leaf), for
    // every kind of node at once, so the warp's lanes issue one load
    rtd::Node64 nd;
    if (STAGED) {
      // one generic load for lanes reading shared memory and lanes reading
      // global memory, instead of both load paths for a mixed warp
      const uint4* src = saddr ? reinterpret_cast<const uint4*>(__cvta_shared_to_generic(saddr)) : g;
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        const uint4 w = src[k];
        nd.w[4 * k + 0] = w.x;
        nd.w[4 * k + 1] = w.y;
        nd.w[4 * k + 2] = w.z;
        nd.w[4 * k + 3] = w.w;
      }
    } else {
      rtd::load64(g, 0, nd);
    }
    // The instance context, once for every kind of node: an instance leaf
    // enters its own instance; a BLAS node needs its instance's object ray,
    // recomputed when the walk comes back from another instance's nodes
    // (make_transformed_ray is deterministic, so recomputing gives the
    // reference's stored objectRay).  Lanes of all kinds switch together.
    rtd::Instance in;
    uint32_t enter = kNone;
    if (top && leaf) {
      if (pinned) {
#pragma unroll
        for (int k = 0; k < 12; ++k) in.w2o.m[k / 3][k % 3] = __uint_as_float(nd.w[rtp::IL_W2O / 4 + k]);
      } else {
        rtd::instance_from(nd, g, saddr, in);
      }
      enter = unit;
    } else if (!top && inst != ic.unit) {
      rtd::load_instance(v.blob + (uint64_t)inst * 4, 0, in);
      enter = inst;
    }
    if (enter != kNone) {
      enter_instance(in, enter, world_o(), dir(), tmin, tmax, ic);
      ic_fast = rtd::finite_ray(ic.o, ic.d, ic.tmin, ic.tmax);
    }
    if (!leaf) {  // internal node, top (:1758-1869) or bottom (:1954-2070)
      record(a, r, unit, rtf::TX_INTERNAL);
      uint32_t soff01 = 0, soff23 = 0, soff45 = 0;
      if (pinned) {  // route bits in bytes 16..17, child records in the tail
        const uint4 t = rtd::ld_shared_v4(saddr + rtp::IN_UNIT);
        rbits = nd.w[rtp::IN_ROUTE / 4] & 0xffffu;
        soff01 = t.y;
        soff23 = t.z;
        soff45 = t.w;
      } else {
        rbits = __ldg(v.route + unit);
      }
      // one box test for both levels, so lanes at TLAS and BLAS nodes run it together
      const bool f = top ? fast : ic_fast;
      const rtm::V3 o = top ? world_o() : ic.o, id = top ? world_idir() : ic.idir;
      const float t0 = top ? tmin : ic.tmin, t1 = top ? tmax : ic.tmax;
      const float cull = top ? min_thit : min_thit * ic.mult;
      const rtd::ChildHits ch = f ? rtd::test_children<true>(nd, unit, o, id, t0, t1, cull)
                                  : rtd::test_children<false>(nd, unit, o, id, t0, t1, cull);
      const uint32_t hit = ch.hit_mask;
      const uint64_t info = ch.info;
      const uint32_t same = rbits >> (rsh * kRouteOther);
      const uint32_t level = top ? kTop : 0u;
      uint32_t c = ch.child_unit;
#pragma unroll
      for (int i = 0; i < 6; ++i) {
        const uint32_t ci = (uint32_t)(info >> (8 * i)) & 0x3fu;
        if ((hit >> i) & 1u) {
          const uint32_t lf = ((ci >> 2) != rtf::CT_INTERNAL) ? kLeaf : 0u;
          const uint32_t sw = i < 2 ? soff01 : (i < 4 ? soff23 : soff45);
          const uint32_t so = (sw >> (16 * (i & 1))) & 0xffffu;
          const uint32_t cc = so ? ((so << kEShift) | kEPin | level | lf) : ((c << kEShift) | level | lf);
          push((same >> i) & 1u, cc, inst);
        }
        c += ci & 3u;
      }
    } else if (top) {  // instance leaf (:1870-1953)
      record(a, r, unit, rtf::TX_INSTANCE_LEAF);
      uint32_t hdr_unit, broot_unit, broot_soff = 0;
      if (pinned) {  // the 64-byte record: units, route bits, BLAS root record, rows
        hdr_unit = nd.w[rtp::IL_HDR_UNIT / 4];
        broot_unit = nd.w[rtp::IL_BROOT_UNIT / 4];
        rbits = nd.w[rtp::IL_ROUTE / 4] & 0xffffu;
        broot_soff = nd.w[rtp::IL_ROUTE / 4] >> 16;
      } else {
        rbits = __ldg(v.route + unit);
        const uint64_t hdr = (uint64_t)unit * 64 + in.bvh_address;
        if ((hdr & 63) || hdr / 64 >= v.n_units) return bad_node();
        hdr_unit = (uint32_t)(hdr >> 6);
        const uint4 h0 = __ldg(v.blob + (hdr >> 4));
        const uint64_t broot = hdr + ((uint64_t)h0.x | ((uint64_t)h0.y << 32));
        broot_unit = (uint32_t)(broot >> 6);
      }
      record(a, r, hdr_unit, rtf::TX_STRUCTURE);
      const uint32_t cc = broot_soff ? ((broot_soff << kEShift) | kEPin) : (broot_unit << kEShift);
      push((rbits >> (kRouteInst + rsh)) & 1u, cc, unit);
    } else {  // primitive leaf (:2071-2196)
      record(a, r, unit, rtf::TX_LEAF_DESC);
      const rtd::Node64& q = nd;
      if (rtf::leaf_type_of(q.w[1]) == 0) {
        const rtm::V3 v0 = rtm::v3(__uint_as_float(q.w[4]), __uint_as_float(q.w[5]), __uint_as_float(q.w[6]));
        const rtm::V3 v1 = rtm::v3(__uint_as_float(q.w[7]), __uint_as_float(q.w[8]), __uint_as_float(q.w[9]));
        const rtm::V3 v2 = rtm::v3(__uint_as_float(q.w[10]), __uint_as_float(q.w[11]), __uint_as_float(q.w[12]));
        float t = 0.0f;
        const bool hit = rtm::ray_triangle_test(v0, v1, v2, ic.o, ic.d, t);
        const float wt = t / ic.mult;
        if (hit && tmin <= wt && wt <= tmax && wt < min_thit) {  // :2127-2141
          min_thit = t / ic.mult;
          set_hit(unit, inst, t);
          record(a, r, unit, rtf::TX_QUAD_LEAF_HIT);
          if (terminate) clear();
        } else {
          record(a, r, unit, rtf::TX_QUAD_LEAF);
        }
      } else {
        status |= RT_RAY_HIT_PROCEDURAL;
        record(a, r, unit, rtf::TX_PROCEDURAL_LEAF);
      }
    }
    if (status & RT_RAY_STACK_OVERFLOW) clear();
  }

  __device__ __forceinline__ void step(const TraceArgs& a, uint32_t r) {
    step(a, r, [](uint32_t, const uint2*) -> uint32_t { return 0u; });
  }

  __device__ __forceinline__ void finish(const TraceArgs& a, uint32_t r) {
    const bool bad = status & (RT_RAY_STACK_OVERFLOW | RT_RAY_BAD_NODE);
    const unsigned long long h = cold(2);
    const Recorder counts{nullptr, nullptr, rec.cap, rec.n, rec.bytes, v.meta};
    write_hit(a, v, r, !bad && (min_thit < tmax), min_thit, world_o(), dir(), tmin, tmax, (uint32_t)h,
              (uint32_t)(h >> 32), lo(cold(3)), counts, status);
  }
};

// The walker's stacks are a separate local array so that its fields stay in
// registers (+5% over the walker with its stacks inside, whose fields the
// compiler left in local memory); with its rarely used fields in the stack's
// cold tail it fits four 256-thread CTAs per SM at 64 registers.
constexpr int kTreeletMinBlocks = 4;

template <int CAP, bool MULTI, bool TRACED>
__global__ void __launch_bounds__(256, kTreeletMinBlocks) trace_treelet_kernel(TraceArgs a) {
  unsigned long long stack[2 * CAP + kColdWords];
  Walker<CAP, false, MULTI, false, TRACED> w;
  w.stk = stack;
  w.pin_base = 0;
  w.pin_root = 0;
  unsigned long long bytes = 0;
  run_persistent(a, w, bytes);
  if (a.stats) add_warp_total64(a.stats + ST_NODE_BYTES, bytes);
}

// ------------------------------------------------------------------ staged

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}

// One non-blocking probe of the phase with the given parity.
__device__ __forceinline__ bool mbar_test(uint64_t* bar, uint32_t parity) {
  uint32_t done;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(done)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return done != 0;
}

// Bounded wait for the phase with the given parity; false if it gave up.
// The first of the max_tries probes does not block (test_wait), the others
// may suspend the thread for a while each (try_wait).
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, uint32_t max_tries) {
  const uint32_t addr = smem_u32(bar);
  if (max_tries == 0) return false;
  if (mbar_test(bar, parity)) return true;
  for (uint32_t i = 1; i < max_tries; ++i) {
    uint32_t done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(addr), "r"(parity)
        : "memory");
    if (done) return true;
  }
  return false;
}

// Global -> shared bulk copy completing on `bar`.  The fence orders this
// thread's earlier generic-proxy accesses before the async-proxy writes.
__device__ __forceinline__ void bulk_copy_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(smem_u32(dst)),
      "l"(src), "r"(bytes), "r"(smem_u32(bar))
      : "memory");
}

constexpr int kMaxSlots = 8;  // slots per warp
constexpr uint32_t kWaitTries = 1u << 22;
// Three 256-thread CTAs per SM, 85 registers a thread as the treelet walk:
// measured against one 512-thread CTA per SM (108 registers, no spills),
// +3% on primary rays and +2% on bounce rays.
constexpr int kStagedMaxThreads = 256;
constexpr int kStagedMinBlocks = 3;
constexpr uint32_t kPinChunk = 32768;  // bytes per bulk copy of the pinned image

// Per-warp staging state in shared memory.
struct WarpStage {
  uint64_t bar;
  uint32_t resident[kMaxSlots];  // dense treelet id per slot, or kNone
  uint32_t units[kMaxSlots];     // 64-byte units of that treelet held in the slot
  uint32_t pending_slot, pending_id, pending_units, phase, victim, disabled;
};

// The staged walk.  Persistent warps with ray refill (as run_persistent).
//
// Pinned treelets: at launch each CTA copies the pinned image (the treelets
// most rays visit, decoded into records, pinned.h) into shared memory with
// cp.async.bulk and keeps it for the whole launch; every node read that names
// a record is served from it.
//
// Warp slots: every `epoch` node visits a warp votes: each lane names the
// treelet of its next access, __match_any_sync counts equal names, and the
// most popular treelet that is not resident (ties to the lowest treelet, i.e.
// the lowest root address, as the RT unit's decision in shader.cc:3424-3441)
// is copied with cp.async.bulk into the warp's least recently filled slot,
// provided at least `min_votes` lanes want it.  A slot holds the first
// slot_bytes of the treelet's image (the whole image when it fits).  Node
// reads that fall in a resident slot are served from shared memory.  A slot
// is read only by its own warp; __syncwarp orders the slot's reads before it
// is refilled.  SLOTS = false compiles the warp slots out (a.slots == 0).
template <int CAP, bool SLOTS, bool TRACED>
__global__ void __launch_bounds__(kStagedMaxThreads, kStagedMinBlocks) trace_staged_kernel(TraceArgs a) {
  extern __shared__ __align__(128) uint8_t dyn_smem[];
  __shared__ WarpStage ws[kStagedMaxThreads / 32];
  __shared__ uint64_t pin_bar;
  __shared__ uint32_t pin_ok;
  uint8_t* const smem0 = dyn_smem + ((128u - (smem_u32(dyn_smem) & 127u)) & 127u);
  const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
  const uint32_t slots = a.slots;
  uint8_t* const my_slots = smem0 + a.pin_bytes + (size_t)warp * slots * a.slot_bytes;
  const uint32_t slot_base = smem_u32(my_slots);
  WarpStage& st = ws[warp];
  if (threadIdx.x == 0) {
    pin_ok = 0;
    if (a.pin_bytes) {
      mbar_init(&pin_bar, 1);
      mbar_expect_tx(&pin_bar, a.pin_bytes);
      for (uint32_t off = 0; off < a.pin_bytes; off += kPinChunk)
        bulk_copy_g2s(smem0 + off, reinterpret_cast<const uint8_t*>(a.pin_image) + off,
                      min(kPinChunk, a.pin_bytes - off), &pin_bar);
      pin_ok = mbar_wait(&pin_bar, 0, a.wait_tries) ? 1u : 0u;
      if (!pin_ok) atomicOr(a.status, kStatusTimeout);
    }
  }
  if (lane == 0) {
    mbar_init(&st.bar, 1);
    for (int s = 0; s < kMaxSlots; ++s) {
      st.resident[s] = kNone;
      st.units[s] = 0;
    }
    st.pending_slot = kNone;
    st.pending_id = kNone;
    st.pending_units = 0;
    st.phase = 0;
    st.victim = 0;
    st.disabled = 0;
  }
  __syncthreads();
  // the node's location is read only while some slot of the warp is resident
  auto lookup = [&](uint32_t unit, const uint2* meta) -> uint32_t {
    bool any = false;
    for (uint32_t s = 0; s < slots; ++s) any |= st.resident[s] != kNone;
    if (!any) return 0u;
    const uint32_t loc = __ldg(reinterpret_cast<const uint32_t*>(meta) + 2ull * unit + 1);
    if (loc == kNone) return 0u;
    const uint32_t d = loc >> kSlotBitsDev, u = loc & ((1u << kSlotBitsDev) - 1u);
    for (uint32_t s = 0; s < slots; ++s)
      if (st.resident[s] == d && u < st.units[s]) return slot_base + s * a.slot_bytes + u * 64u;
    return 0u;
  };
  unsigned long long stack[2 * CAP + kColdWords];
  Walker<CAP, true, false, false, TRACED> w;  // staged launches trace one scene
  w.stk = stack;
  w.pin_base = pin_ok ? smem_u32(smem0) : 0u;
  w.pin_root = pin_ok ? a.pin_root : 0u;
  bool have = false, exhausted = false;
  uint32_t r = 0, it = 0;
  unsigned long long bytes = 0, staged = 0, stagings = 0, sreads = 0, greads = 0;
  for (;; ++it) {
    // --- refill idle lanes (as run_persistent)
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
    // --- staging: land a finished copy, then vote for the next one
    if (SLOTS && slots > 0 && (it % a.epoch) == 0) {
      if (lane == 0 && st.pending_slot != kNone && mbar_test(&st.bar, st.phase)) {
        st.resident[st.pending_slot] = st.pending_id;
        st.units[st.pending_slot] = st.pending_units;
        st.phase ^= 1u;
        st.pending_slot = kNone;
      }
      __syncwarp();
      if (st.pending_slot == kNone && !st.disabled) {
        const uint32_t nl = (have && w.active()) ? w.next_loc() : kNone;
        uint32_t key = nl == kNone ? kNone : (nl >> kSlotBitsDev);
        if (a.hint && key != kNone) {
          // vote for the treelet predicted to follow the one the ray enters next
          const rtm::V3 wd = w.dir();
          const uint32_t oct = (wd.x > 0.0f ? 1u : 0u) | (wd.y > 0.0f ? 2u : 0u) | (wd.z > 0.0f ? 4u : 0u);
          key = __ldg(a.hint + (size_t)key * 8 + oct);
          if (key >= a.n_treelets) key = kNone;
        }
        if (key != kNone)
          for (uint32_t s = 0; s < slots; ++s)
            if (st.resident[s] == key) key = kNone;  // already resident
        const uint32_t peers = __match_any_sync(0xffffffffu, key);
        unsigned long long v =
            key == kNone ? 0ull : (((unsigned long long)__popc(peers) << 32) | (unsigned long long)(~key));
#pragma unroll
        for (int s = 16; s > 0; s >>= 1) {
          const unsigned long long o = __shfl_xor_sync(0xffffffffu, v, s);
          v = o > v ? o : v;
        }
        const uint32_t votes = (uint32_t)(v >> 32);
        if (votes > 0 && votes >= a.min_votes && lane == 0) {
          const uint32_t d = ~(uint32_t)(v & 0xffffffffu);
          const unsigned long long off = a.image_off[d];
          uint32_t nb = (uint32_t)(a.image_off[d + 1] - off);
          if (nb > a.slot_bytes) nb = a.slot_bytes;
          if (nb > 0) {
            const uint32_t s = st.victim;
            st.victim = (s + 1 == slots) ? 0 : s + 1;
            st.resident[s] = kNone;
            st.units[s] = 0;
            mbar_expect_tx(&st.bar, nb);
            bulk_copy_g2s(my_slots + (size_t)s * a.slot_bytes, reinterpret_cast<const uint8_t*>(a.images) + off, nb,
                          &st.bar);
            st.pending_slot = s;
            st.pending_id = d;
            st.pending_units = nb / 64u;
            staged += nb;
            stagings += 1;
          }
        }
      }
      __syncwarp();
    }
    // --- one node visit per lane
    if (have) {
      if (SLOTS) w.step(a, r, lookup);
      else w.step(a, r);
      if (!w.active()) {
        w.finish(a, r);
        bytes += w.rec.bytes;
        sreads += w.smem_reads;
        greads += w.gmem_reads;
        have = false;
      }
    }
  }
  // copies still in flight must land before the CTA's shared memory goes away
  if (lane == 0 && st.pending_slot != kNone) {
    if (!mbar_wait(&st.bar, st.phase, kWaitTries)) atomicOr(a.status, kStatusTimeout);
  }
  if (threadIdx.x == 0 && a.pin_bytes && !pin_ok) {
    if (!mbar_wait(&pin_bar, 0, kWaitTries)) atomicOr(a.status, kStatusTimeout);
  }
  __syncwarp();
  if (a.stats) {
    add_warp_total64(a.stats + ST_NODE_BYTES, bytes);
    add_warp_total64(a.stats + ST_SMEM_READS, sreads);
    add_warp_total64(a.stats + ST_GMEM_READS, greads);
    add_warp_total64(a.stats + ST_STAGED_BYTES, staged);
    add_warp_total64(a.stats + ST_STAGINGS, stagings);
  }
  if (a.stats && threadIdx.x == 0 && pin_ok && blockIdx.x == 0) {
    // the pinned image counts once as staged bytes (copied by every CTA)
    atomicAdd(a.stats + ST_STAGED_BYTES, (unsigned long long)a.pin_bytes * gridDim.x);
    atomicAdd(a.stats + ST_STAGINGS, (unsigned long long)gridDim.x);
  }
}

}  // namespace rtk
