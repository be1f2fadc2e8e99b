// Treelet-ordered traversal (traceRayWithTreelets, vulkan_ray_tracing.cc:1522-2307)
// and its shared-memory staged variant.
#pragma once
#include "trace_kernels.cuh"

namespace rtk {

constexpr uint32_t kSlotBitsDev = 10;

// A ray's treelet-ordered walk.  Two LIFO stacks as in the reference
// (push_front / pop_front on std::list, :1708-1709): `cur` holds nodes of the
// current treelet, `oth` the rest (:1821-1856).  An entry packs the node
// (unit << 2 | top | leaf) and, for bottom-level nodes, the instance leaf it
// belongs to.  The staged location of a node (dense treelet << 10 | 64-byte
// slot in that treelet's image) is read from the node table when needed, not
// kept on the stacks.
template <int CAP, bool STAGED>
struct Walker {
  rtm::V3 O, D, idir;
  float tmin, tmax, min_thit, c_tobj;
  bool terminate, fast, ic_fast;  // FAST min/max allowed for the world / object ray
  uint32_t c_leaf, c_inst, current_root, status;
  int cn, on;
  unsigned long long cu[CAP], ot[CAP];
  InstCtx ic;
  Recorder rec;
  SceneView v;
  uint32_t smem_reads, gmem_reads;

  __device__ __forceinline__ bool active() const { return cn > 0 || on > 0; }

  // Staged location (dense treelet << 10 | slot) of the node the ray visits
  // next, i.e. its first pending access.
  __device__ __forceinline__ uint32_t next_loc() const {
    unsigned long long e;
    if (cn > 0) e = cu[cn - 1];
    else if (on > 0) e = ot[on - 1];
    else return kNone;
    const uint32_t unit = (uint32_t)e >> 2;
    return unit < v.n_units ? __ldg(reinterpret_cast<const uint32_t*>(v.meta) + 2ull * unit + 1) : kNone;
  }

  // addrToTreeletID(child) == current_treelet_root ? current : other.
  __device__ __forceinline__ void route(const TraceArgs& a, uint32_t code, uint32_t inst) {
    const uint32_t unit = code >> 2;
    const uint32_t root = unit < v.n_units ? __ldg(reinterpret_cast<const uint32_t*>(v.meta) + 2ull * unit) : kNone;
    const unsigned long long e = (unsigned long long)code | ((unsigned long long)inst << 32);
    if (root == current_root) {
      if (cn < CAP) cu[cn++] = e;
      else status |= RT_RAY_STACK_OVERFLOW;
    } else {
      if (on < CAP) ot[on++] = e;
      else status |= RT_RAY_STACK_OVERFLOW;
    }
  }

  __device__ __forceinline__ void init(const TraceArgs& a, uint32_t r) {
    v = scene_of(a, r);
    load_ray(a.rays, r, O, tmin, D, tmax);
    const uint32_t flags = a.flags ? a.flags[r] : a.default_flags;
    terminate = flags & rtf::RAY_FLAG_TERMINATE_ON_FIRST_HIT;
    rec = Recorder{a.visits ? a.visits + (uint64_t)r * a.cap : nullptr,
                   a.tl_trace ? a.tl_trace + (uint64_t)r * a.cap : nullptr, a.cap, 0u, 0u, v.meta};
    status = 0;
    cn = on = 0;
    min_thit = tmax;
    c_leaf = c_inst = 0;
    c_tobj = 0.0f;
    current_root = 0;  // the TLAS header (:1707)
    ic.unit = kNone;
    smem_reads = gmem_reads = 0;
    idir = rtm::calculate_idir(D);
    fast = rtd::finite_ray(O, D, tmin, tmax);
    ic_fast = false;
    rec.rec(0, rtf::TX_STRUCTURE);
    const uint4 h0 = __ldg(v.blob), h1 = __ldg(v.blob + 1);
    const uint64_t root_off = (uint64_t)h0.x | ((uint64_t)h0.y << 32);
    const rtm::V3 bmin = rtm::v3(__uint_as_float(h0.z), __uint_as_float(h0.w), __uint_as_float(h1.x));
    const rtm::V3 bmax = rtm::v3(__uint_as_float(h1.y), __uint_as_float(h1.z), __uint_as_float(h1.w));
    float th;
    if (rtm::ray_box_test(bmin, bmax, idir, O, tmin, tmax, th)) route(a, ((uint32_t)(root_off >> 6) << 2) | kTop, 0);
  }

  __device__ __forceinline__ void ensure_instance(const TraceArgs& a, uint32_t inst) {
    if (ic.unit == inst) return;
    rtd::Instance in;
    rtd::load_instance(v.blob + (uint64_t)inst * 4, 0, in);
    enter_instance(in, inst, O, D, tmin, tmax, ic);
    ic_fast = rtd::finite_ray(ic.o, ic.d, ic.tmin, ic.tmax);
  }

  // Visits one node; `lookup(unit, meta)` returns its shared-memory address
  // when it is staged, else 0.
  template <class Lookup>
  __device__ __forceinline__ void step(const TraceArgs& a, Lookup&& lookup) {
    unsigned long long e;
    if (cn == 0) {  // :1748-1754
      --on;
      e = ot[on];
      current_root = (uint32_t)e >> 2;
    } else {
      --cn;
      e = cu[cn];
    }
    const uint32_t code = (uint32_t)e, inst = (uint32_t)(e >> 32);
    const uint32_t unit = code >> 2;
    const bool top = code & kTop, leaf = code & kLeaf;
    if (unit + ((top && leaf) ? 1u : 0u) >= v.n_units) {
      status |= RT_RAY_BAD_NODE;
      cn = on = 0;
      return;
    }
    uint32_t saddr = 0;
    if (STAGED) {
      saddr = lookup(unit, v.meta);
      if (saddr) ++smem_reads;
      else ++gmem_reads;
    }
    const uint4* g = v.blob + (uint64_t)unit * 4;
    if (!leaf) {  // internal node, top (:1758-1869) or bottom (:1954-2070)
      rec.rec(unit, rtf::TX_INTERNAL);
      rtd::Node64 nd;
      rtd::load64(g, saddr, nd);
      rtd::ChildHits ch;
      if (top) {
        ch = fast ? rtd::test_children<true>(nd, unit, O, idir, tmin, tmax, min_thit)
                  : rtd::test_children<false>(nd, unit, O, idir, tmin, tmax, min_thit);
      } else {
        ensure_instance(a, inst);
        const float cull = min_thit * ic.mult;
        ch = ic_fast ? rtd::test_children<true>(nd, unit, ic.o, ic.idir, ic.tmin, ic.tmax, cull)
                     : rtd::test_children<false>(nd, unit, ic.o, ic.idir, ic.tmin, ic.tmax, cull);
      }
      const uint32_t level = top ? kTop : 0u;
      uint32_t c = ch.child_unit;
#pragma unroll
      for (int i = 0; i < 6; ++i) {
        const uint32_t info = ch.info_of(i);
        if ((ch.hit_mask >> i) & 1u) {
          const uint32_t lf = ((info >> 2) != rtf::CT_INTERNAL) ? kLeaf : 0u;
          route(a, (c << 2) | level | lf, inst);
        }
        c += info & 3u;
      }
    } else if (top) {  // instance leaf (:1870-1953)
      rec.rec(unit, rtf::TX_INSTANCE_LEAF);
      rtd::Instance in;
      rtd::load_instance(g, saddr, in);
      const uint64_t hdr = (uint64_t)unit * 64 + in.bvh_address;
      if ((hdr & 63) || hdr / 64 >= v.n_units) {
        status |= RT_RAY_BAD_NODE;
        cn = on = 0;
        return;
      }
      rec.rec((uint32_t)(hdr >> 6), rtf::TX_STRUCTURE);
      const uint4 h0 = __ldg(v.blob + (hdr >> 4));
      const uint64_t broot = hdr + ((uint64_t)h0.x | ((uint64_t)h0.y << 32));
      enter_instance(in, unit, O, D, tmin, tmax, ic);
      ic_fast = rtd::finite_ray(ic.o, ic.d, ic.tmin, ic.tmax);
      route(a, (uint32_t)(broot >> 6) << 2, unit);
    } else {  // primitive leaf (:2071-2196)
      rec.rec(unit, rtf::TX_LEAF_DESC);
      rtd::Node64 q;
      rtd::load64(g, saddr, q);
      if (rtf::leaf_type_of(q.w[1]) == 0) {
        ensure_instance(a, inst);
        const rtm::V3 v0 = rtm::v3(__uint_as_float(q.w[4]), __uint_as_float(q.w[5]), __uint_as_float(q.w[6]));
        const rtm::V3 v1 = rtm::v3(__uint_as_float(q.w[7]), __uint_as_float(q.w[8]), __uint_as_float(q.w[9]));
        const rtm::V3 v2 = rtm::v3(__uint_as_float(q.w[10]), __uint_as_float(q.w[11]), __uint_as_float(q.w[12]));
        float t = 0.0f;
        const bool hit = rtm::ray_triangle_test(v0, v1, v2, ic.o, ic.d, t);
        const float wt = t / ic.mult;
        if (hit && tmin <= wt && wt <= tmax && wt < min_thit) {  // :2127-2141
          min_thit = t / ic.mult;
          c_tobj = t;
          c_leaf = unit;
          c_inst = inst;
          rec.rec(unit, rtf::TX_QUAD_LEAF_HIT);
          if (terminate) cn = on = 0;
        } else {
          rec.rec(unit, rtf::TX_QUAD_LEAF);
        }
      } else {
        status |= RT_RAY_HIT_PROCEDURAL;
        rec.rec(unit, rtf::TX_PROCEDURAL_LEAF);
      }
    }
    if (status & RT_RAY_STACK_OVERFLOW) cn = on = 0;
  }

  __device__ __forceinline__ void step(const TraceArgs& a) {
    step(a, [](uint32_t, const uint2*) -> uint32_t { return 0u; });
  }

  __device__ __forceinline__ void finish(const TraceArgs& a, uint32_t r) {
    const bool bad = status & (RT_RAY_STACK_OVERFLOW | RT_RAY_BAD_NODE);
    write_hit(a, v, r, !bad && (min_thit < tmax), min_thit, O, D, tmin, tmax, c_leaf, c_inst, c_tobj, rec, status);
  }
};

template <int CAP>
__global__ void __launch_bounds__(256) trace_treelet_kernel(TraceArgs a) {
  Walker<CAP, false> w;
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
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, uint32_t max_tries) {
  const uint32_t addr = smem_u32(bar);
  for (uint32_t i = 0; i < max_tries; ++i) {
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

// Per-warp staging state in shared memory.
struct WarpStage {
  uint64_t bar;
  uint32_t resident[kMaxSlots];  // dense treelet id per slot, or kNone
  uint32_t units[kMaxSlots];     // 64-byte units of that treelet held in the slot
  uint32_t pending_slot, pending_id, pending_units, phase, victim, disabled;
};

// The staged walk.  Persistent warps with ray refill (as run_persistent).
// Every `epoch` node visits a warp votes: each lane names the treelet of its
// next access, __match_any_sync counts equal names, and the most popular
// treelet that is not resident (ties to the lowest treelet, i.e. the lowest
// root address, as the RT unit's decision in shader.cc:3424-3441) is copied
// with cp.async.bulk into the warp's least recently filled slot, provided at
// least `min_votes` lanes want it.  A slot holds the first slot_bytes of the
// treelet's image (the whole image when it fits).  Node reads that fall in a
// resident slot are served from shared memory.  A slot is read only by its
// own warp; __syncwarp orders the slot's reads before it is refilled.
template <int CAP>
__global__ void __launch_bounds__(256) trace_staged_kernel(TraceArgs a) {
  extern __shared__ __align__(128) uint8_t dyn_smem[];
  __shared__ WarpStage ws[8];
  uint8_t* const smem0 = dyn_smem + ((128u - (smem_u32(dyn_smem) & 127u)) & 127u);
  const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
  const uint32_t slots = a.slots;
  uint8_t* const my_slots = smem0 + (size_t)warp * slots * a.slot_bytes;
  const uint32_t slot_base = smem_u32(my_slots);
  WarpStage& st = ws[warp];
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
  __syncwarp();
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
  Walker<CAP, true> w;
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
    if (slots > 0 && (it % a.epoch) == 0) {
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
          const uint32_t oct = (w.D.x > 0.0f ? 1u : 0u) | (w.D.y > 0.0f ? 2u : 0u) | (w.D.z > 0.0f ? 4u : 0u);
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
      w.step(a, lookup);
      if (!w.active()) {
        w.finish(a, r);
        bytes += w.rec.bytes;
        sreads += w.smem_reads;
        greads += w.gmem_reads;
        have = false;
      }
    }
  }
  // a copy still in flight must land before the warp's shared memory goes away
  if (lane == 0 && st.pending_slot != kNone) {
    if (!mbar_wait(&st.bar, st.phase, kWaitTries)) atomicOr(a.status, kStatusTimeout);
  }
  __syncwarp();
  if (a.stats) {
    add_warp_total64(a.stats + ST_NODE_BYTES, bytes);
    add_warp_total64(a.stats + ST_SMEM_READS, sreads);
    add_warp_total64(a.stats + ST_GMEM_READS, greads);
    add_warp_total64(a.stats + ST_STAGED_BYTES, staged);
    add_warp_total64(a.stats + ST_STAGINGS, stagings);
  }
}

}  // namespace rtk
