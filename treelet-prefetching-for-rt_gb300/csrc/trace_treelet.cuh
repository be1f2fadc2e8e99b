// Treelet-ordered traversal (traceRayWithTreelets, vulkan_ray_tracing.cc:1522-2307)
// with optional shared-memory staging of treelets.
#pragma once
#include "trace_kernels.cuh"

namespace rtk {

constexpr uint32_t kSlotBitsDev = 10;

// A ray's treelet-ordered walk.  Two LIFO stacks as in the reference
// (push_front / pop_front on std::list): `cur` for nodes in the current
// treelet, `oth` for the rest.  An entry carries the node (unit << 2 | top |
// leaf), the instance leaf it belongs to (bottom-level entries) and the
// node's staged location.
template <int CAP>
struct Walker {
  rtm::V3 O, D, idir;
  float tmin, tmax, min_thit, c_tobj;
  bool terminate;
  uint32_t c_leaf, c_inst, current_root, status;
  int cn, on;
  uint32_t cu_code[CAP], cu_inst[CAP], cu_loc[CAP];
  uint32_t ot_code[CAP], ot_inst[CAP], ot_loc[CAP];
  InstCtx ic;
  Recorder rec;
  uint32_t smem_reads, gmem_reads;

  __device__ __forceinline__ bool active() const { return cn > 0 || on > 0; }

  // Unit index of the node the ray visits next (its first pending access).
  __device__ __forceinline__ uint32_t next_loc() const {
    if (cn > 0) return cu_loc[cn - 1];
    if (on > 0) return ot_loc[on - 1];
    return kNone;
  }

  __device__ __forceinline__ void route(const TraceArgs& a, uint32_t code, uint32_t inst) {
    const uint32_t unit = code >> 2;
    uint2 m = make_uint2(kNone, kNone);
    if (unit < a.n_units) m = __ldg(a.meta + unit);
    if (m.x == current_root) {
      if (cn < CAP) {
        cu_code[cn] = code;
        cu_inst[cn] = inst;
        cu_loc[cn] = m.y;
        ++cn;
      } else {
        status |= RT_RAY_STACK_OVERFLOW;
      }
    } else {
      if (on < CAP) {
        ot_code[on] = code;
        ot_inst[on] = inst;
        ot_loc[on] = m.y;
        ++on;
      } else {
        status |= RT_RAY_STACK_OVERFLOW;
      }
    }
  }

  __device__ __forceinline__ void init(const TraceArgs& a, uint32_t r) {
    load_ray(a.rays, r, O, tmin, D, tmax);
    const uint32_t flags = a.flags ? a.flags[r] : a.default_flags;
    terminate = flags & rtf::RAY_FLAG_TERMINATE_ON_FIRST_HIT;
    rec = Recorder{a.visits ? a.visits + (uint64_t)r * a.cap : nullptr,
                   a.tl_trace ? a.tl_trace + (uint64_t)r * a.cap : nullptr, a.cap, 0u, 0u, a.meta};
    status = 0;
    cn = on = 0;
    min_thit = tmax;
    c_leaf = c_inst = 0;
    c_tobj = 0.0f;
    current_root = 0;  // the TLAS header (:1707)
    ic.unit = kNone;
    smem_reads = gmem_reads = 0;
    idir = rtm::calculate_idir(D);
    rec.rec(0, rtf::TX_STRUCTURE);
    const uint4 h0 = __ldg(a.blob), h1 = __ldg(a.blob + 1);
    const uint64_t root_off = (uint64_t)h0.x | ((uint64_t)h0.y << 32);
    const rtm::V3 bmin = rtm::v3(__uint_as_float(h0.z), __uint_as_float(h0.w), __uint_as_float(h1.x));
    const rtm::V3 bmax = rtm::v3(__uint_as_float(h1.y), __uint_as_float(h1.z), __uint_as_float(h1.w));
    float th;
    if (rtm::ray_box_test(bmin, bmax, idir, O, tmin, tmax, th)) route(a, ((uint32_t)(root_off >> 6) << 2) | kTop, 0);
  }

  __device__ __forceinline__ void ensure_instance(const TraceArgs& a, uint32_t inst) {
    if (ic.unit == inst) return;
    rtd::Instance in;
    rtd::load_instance(a.blob + (uint64_t)inst * 4, 0, in);
    enter_instance(in, inst, O, D, tmin, tmax, ic);
  }

  // Visits one node.  `saddr` is its shared-memory address when staged, else 0.
  template <class Lookup>
  __device__ __forceinline__ void step(const TraceArgs& a, Lookup&& lookup) {
    uint32_t code, inst, loc;
    if (cn == 0) {  // :1748-1754
      --on;
      code = ot_code[on];
      inst = ot_inst[on];
      loc = ot_loc[on];
      current_root = code >> 2;
    } else {
      --cn;
      code = cu_code[cn];
      inst = cu_inst[cn];
      loc = cu_loc[cn];
    }
    const uint32_t unit = code >> 2;
    const bool top = code & kTop, leaf = code & kLeaf;
    if (unit + ((top && leaf) ? 1u : 0u) >= a.n_units) {
      status |= RT_RAY_BAD_NODE;
      cn = on = 0;
      return;
    }
    const uint32_t saddr = lookup(loc);
    if (saddr) ++smem_reads;
    else ++gmem_reads;
    const uint4* g = a.blob + (uint64_t)unit * 4;
    if (!leaf) {  // internal node, top (:1758-1869) or bottom (:1954-2070)
      rec.rec(unit, rtf::TX_INTERNAL);
      rtd::Node64 nd;
      rtd::load64(g, saddr, nd);
      rtd::ChildHits ch;
      if (top) {
        ch = rtd::test_children(nd, unit, O, idir, tmin, tmax, min_thit);
      } else {
        ensure_instance(a, inst);
        ch = rtd::test_children(nd, unit, ic.o, ic.idir, ic.tmin, ic.tmax, min_thit * ic.mult);
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
      if ((hdr & 63) || hdr / 64 >= a.n_units) {
        status |= RT_RAY_BAD_NODE;
        cn = on = 0;
        return;
      }
      rec.rec((uint32_t)(hdr >> 6), rtf::TX_STRUCTURE);
      const uint4 h0 = __ldg(a.blob + (hdr >> 4));
      const uint64_t broot = hdr + ((uint64_t)h0.x | ((uint64_t)h0.y << 32));
      enter_instance(in, unit, O, D, tmin, tmax, ic);
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
        if (hit && tmin <= wt && wt <= tmax && wt < min_thit) {
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

  __device__ __forceinline__ void finish(const TraceArgs& a, uint32_t r) {
    const bool bad = status & (RT_RAY_STACK_OVERFLOW | RT_RAY_BAD_NODE);
    write_hit(a, r, !bad && (min_thit < tmax), min_thit, O, D, tmin, tmax, c_leaf, c_inst, c_tobj, rec, status);
  }
};

template <int CAP>
__global__ void __launch_bounds__(256) trace_treelet_kernel(TraceArgs a) {
  const uint32_t r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= a.n) return;
  Walker<CAP> w;
  w.init(a, r);
  auto no_stage = [](uint32_t) -> uint32_t { return 0u; };
  while (w.active()) w.step(a, no_stage);
  w.finish(a, r);
  if (a.stats) add_warp_total(a.stats + ST_NODE_BYTES, w.rec.bytes);
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

__device__ __forceinline__ void bulk_copy_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(smem_u32(dst)),
      "l"(src), "r"(bytes), "r"(smem_u32(bar))
      : "memory");
}

constexpr int kHashSize = 512;   // vote table entries (>= 2 x threads per CTA)
constexpr int kMaxSlots = 32;
constexpr uint32_t kWaitTries = 1u << 22;

struct StagedShared {
  uint64_t bar;
  uint32_t resident[kMaxSlots];  // dense treelet id per slot, or kNone
  uint32_t pending_slot, pending_id, phase, disabled, victim;
  uint32_t hkey[kHashSize];
  uint32_t hcnt[kHashSize];
  unsigned long long best[8];
  unsigned long long staged_bytes, stagings;
};

// One CTA = the rays of one RT unit.  Each epoch: finish the previous copy,
// vote on the treelet the most rays access next, start copying it into a
// slot, then let every ray walk up to `epoch` nodes.
template <int CAP>
__global__ void __launch_bounds__(256) trace_staged_kernel(TraceArgs a) {
  extern __shared__ __align__(128) uint8_t dyn_smem[];
  __shared__ StagedShared sh;
  // slots start on a 128-byte boundary (the launch adds 128 bytes of room)
  uint8_t* const slot_mem = dyn_smem + ((128u - (smem_u32(dyn_smem) & 127u)) & 127u);
  const uint32_t tid = threadIdx.x;
  const uint32_t r = blockIdx.x * blockDim.x + tid;
  const bool mine = r < a.n;
  Walker<CAP> w;
  if (mine) w.init(a, r);
  else w.cn = w.on = 0;
  const uint32_t slots = a.slots;
  if (tid == 0) {
    mbar_init(&sh.bar, 1);
    sh.pending_slot = kNone;
    sh.pending_id = kNone;
    sh.phase = 0;
    sh.disabled = 0;
    sh.victim = 0;
    sh.staged_bytes = 0;
    sh.stagings = 0;
  }
  for (uint32_t s = tid; s < kMaxSlots; s += blockDim.x) sh.resident[s] = kNone;
  const uint32_t slot_base = smem_u32(slot_mem);
  auto lookup = [&](uint32_t loc) -> uint32_t {
    if (loc == kNone) return 0u;
    const uint32_t d = loc >> kSlotBitsDev;
    for (uint32_t s = 0; s < slots; ++s)
      if (sh.resident[s] == d) return slot_base + s * a.slot_bytes + (loc & ((1u << kSlotBitsDev) - 1u)) * 64u;
    return 0u;
  };
  __syncthreads();
  for (;;) {
    // 1. complete the copy started last epoch; clear the vote table
    if (tid == 0 && sh.pending_slot != kNone) {
      if (mbar_wait(&sh.bar, sh.phase, kWaitTries)) {
        sh.resident[sh.pending_slot] = sh.pending_id;
        sh.phase ^= 1u;
      } else {
        sh.disabled = 1;
        atomicOr(a.status, kStatusTimeout);
      }
      sh.pending_slot = kNone;
      sh.pending_id = kNone;
    }
    for (int h = tid; h < kHashSize; h += blockDim.x) {
      sh.hkey[h] = kNone;
      sh.hcnt[h] = 0;
    }
    __syncthreads();
    // 2. vote: each active ray's next access -> its treelet
    const uint32_t nl = w.active() ? w.next_loc() : kNone;
    const uint32_t key = nl == kNone ? kNone : (nl >> kSlotBitsDev);
    const uint32_t peers = __match_any_sync(0xffffffffu, key);
    if (key != kNone && (tid & 31u) == (uint32_t)(__ffs(peers) - 1)) {
      uint32_t h = (key * 2654435761u) & (kHashSize - 1);
      for (int probe = 0; probe < kHashSize; ++probe) {
        const uint32_t old = atomicCAS(&sh.hkey[h], kNone, key);
        if (old == kNone || old == key) {
          atomicAdd(&sh.hcnt[h], (uint32_t)__popc(peers));
          break;
        }
        h = (h + 1) & (kHashSize - 1);
      }
    }
    __syncthreads();
    // argmax over (count, lowest id), skipping resident treelets
    unsigned long long bestv = 0;
    for (int h = tid; h < kHashSize; h += blockDim.x) {
      const uint32_t k = sh.hkey[h];
      if (k == kNone) continue;
      bool res = false;
      for (uint32_t s = 0; s < slots; ++s) res |= (sh.resident[s] == k);
      if (res) continue;
      const unsigned long long v = ((unsigned long long)sh.hcnt[h] << 32) | (unsigned long long)(~k);
      bestv = v > bestv ? v : bestv;
    }
#pragma unroll
    for (int s = 16; s > 0; s >>= 1) {
      const unsigned long long o = __shfl_xor_sync(0xffffffffu, bestv, s);
      bestv = o > bestv ? o : bestv;
    }
    if ((tid & 31u) == 0) sh.best[tid >> 5] = bestv;
    __syncthreads();
    if (tid == 0) {
      unsigned long long b = 0;
      for (uint32_t k = 0; k < (blockDim.x + 31) / 32; ++k) b = sh.best[k] > b ? sh.best[k] : b;
      const uint32_t cnt = (uint32_t)(b >> 32);
      if (cnt > 0 && !sh.disabled && slots > 0) {
        const uint32_t d = ~(uint32_t)(b & 0xffffffffu);
        const unsigned long long off = a.image_off[d];
        const uint32_t bytes = (uint32_t)(a.image_off[d + 1] - off);
        if (bytes > 0 && bytes <= a.slot_bytes) {
          const uint32_t s = sh.victim;
          sh.victim = (s + 1 == slots) ? 0 : s + 1;
          sh.resident[s] = kNone;
          mbar_expect_tx(&sh.bar, bytes);
          bulk_copy_g2s(slot_mem + (size_t)s * a.slot_bytes, reinterpret_cast<const uint8_t*>(a.images) + off, bytes,
                        &sh.bar);
          sh.pending_slot = s;
          sh.pending_id = d;
          sh.staged_bytes += bytes;
          sh.stagings += 1;
        }
      }
    }
    __syncthreads();
    // 3. walk
    for (uint32_t k = 0; k < a.epoch && w.active(); ++k) w.step(a, lookup);
    if (!__syncthreads_or(w.active() ? 1 : 0)) break;
  }
  // a copy still in flight must land before the CTA's shared memory goes away
  if (tid == 0 && sh.pending_slot != kNone) {
    if (!mbar_wait(&sh.bar, sh.phase, kWaitTries)) atomicOr(a.status, kStatusTimeout);
  }
  if (mine) {
    w.finish(a, r);
    if (a.stats) {
      add_warp_total(a.stats + ST_NODE_BYTES, w.rec.bytes);
      add_warp_total(a.stats + ST_SMEM_READS, w.smem_reads);
      add_warp_total(a.stats + ST_GMEM_READS, w.gmem_reads);
    }
  }
  if (tid == 0 && a.stats) {
    atomicAdd(a.stats + ST_STAGED_BYTES, sh.staged_bytes);
    atomicAdd(a.stats + ST_STAGINGS, sh.stagings);
  }
  __syncthreads();
}

}  // namespace rtk
