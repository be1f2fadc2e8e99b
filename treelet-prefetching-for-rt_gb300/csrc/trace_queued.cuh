// Treelet-queued staged traversal: rays wait in per-treelet queues, and each
// treelet is staged into shared memory with cp.async.bulk before the rays
// queued on it traverse it.
//
// traceRayWithTreelets (vulkan_ray_tracing.cc:1522-2307) walks one treelet at
// a time: it drains the current-treelet stack, then pops the other-treelet
// stack and makes that node the current treelet root (:1748-1754).  A ray's
// walk therefore splits into stints, one per treelet, and between two stints
// its whole state is the ray, the closest hit so far and the other-treelet
// stack.  Here that state lives in global memory (Walker<..., SLAB>), so a
// ray can stop at the end of a stint and go on later in any thread:
//
//   round 0     every ray starts at the TLAS root treelet (one queue);
//   round k     the rays that are left are binned by the treelet of their
//               next node (a counting sort: histogram, scan, scatter), so
//               that the rays queued on one treelet sit next to each other;
//               a warp takes 32 queued rays, copies the treelet of its first
//               ray into its shared-memory slot (cp.async.bulk, mbarrier,
//               bounded wait) and runs each ray's stint, reading that
//               treelet's nodes from the slot;
//   last round  after `queue_rounds` binned rounds the rays still walking
//               finish their walks one node visit per iteration with
//               per-lane refill (their late stints fall on small, scattered
//               treelets that queues cannot batch).
//
// The most waiting treelets come first within a round only in the sense that
// every queue is drained once per round; the RT unit's choice of the most
// popular treelet (shader.cc:3419-3441) becomes "every treelet with waiting
// rays, each staged once per warp that serves it".  Each ray's own visit
// order is the reference's exactly, so hit records and access traces equal
// the treelet-order walk's bit for bit; only when a ray's work runs changes.
#pragma once
#include "trace_treelet.cuh"

namespace rtk {

constexpr uint32_t kBinScanItems = 4096;  // bins per block of bin_scan_kernel (1024 threads x 4)
constexpr uint32_t kQueueSlotMax = 8192;  // bytes of a warp's staging slot

struct QueueArgs {
  uint4* state;              // per ray: 4 x uint4 (Walker::save_ray / suspend)
  unsigned long long* slab;  // per ray: CAP entries of its other-treelet stack
  const uint32_t* in_ray;    // this round's queued rays, grouped by treelet (null in round 0: all rays in order)
  const uint32_t* in_key;    // the treelet (dense id) each queued ray needs next
  const uint32_t* n_in;      // queued rays (null in round 0: the launch's n)
  uint32_t* take;            // hand-out counter of this round
  uint32_t* out_ray;         // rays still walking after this round, unsorted
  uint32_t* out_key;
  uint32_t* n_out;
  uint32_t* hist;            // rays per bin for the next round
  uint32_t n_bins;           // treelets + 1 (the last bin: a node outside every image)
  uint32_t slot_bytes;       // per-warp staging slot (multiple of 128, holds the largest image)
};

// Bin of the node on top of the ray's other-treelet stack: the dense id of
// its treelet, or the last bin.
template <class W>
__device__ __forceinline__ uint32_t next_bin(const TraceArgs& a, const QueueArgs& q, const W& w) {
  const unsigned long long e = w.ot_at(w.not_ - 1);
  const uint32_t unit = (uint32_t)e >> kEShift;
  const uint32_t loc = unit < w.v.n_units ? __ldg(reinterpret_cast<const uint32_t*>(w.v.meta) + 2ull * unit + 1) : kNone;
  const uint32_t d = loc == kNone ? kNone : loc >> kSlotBitsDev;
  return d < q.n_bins - 1 ? d : q.n_bins - 1;
}

// Adds 1 per lane to counter[key] with one atomic per distinct key of the
// calling lanes; returns this lane's old value + its rank among equal keys.
__device__ __forceinline__ uint32_t add_grouped(uint32_t* counter, uint32_t key, uint32_t mask) {
  const uint32_t lane = threadIdx.x & 31u;
  const uint32_t peers = __match_any_sync(mask, key);
  const int leader = __ffs(peers) - 1;
  uint32_t base = 0;
  if ((int)lane == leader) base = atomicAdd(counter + key, (uint32_t)__popc(peers));
  base = __shfl_sync(peers, base, leader);
  return base + (uint32_t)__popc(peers & ((1u << lane) - 1u));
}

// One binned round (FINAL = false) or the last round (FINAL = true).
template <int CAP, bool FINAL>
__global__ void __launch_bounds__(kStagedMaxThreads, kStagedMinBlocks) trace_queued_kernel(TraceArgs a, QueueArgs q) {
  extern __shared__ __align__(128) uint8_t dyn_smem[];
  __shared__ uint64_t bars[kStagedMaxThreads / 32];
  __shared__ uint32_t slot_key[kStagedMaxThreads / 32], slot_units[kStagedMaxThreads / 32];
  uint8_t* const smem0 = dyn_smem + ((128u - (smem_u32(dyn_smem) & 127u)) & 127u);
  const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
  uint8_t* const slot = smem0 + (size_t)warp * q.slot_bytes;
  const uint32_t slot_base = smem_u32(slot);
  uint32_t phase = 0;         // lane 0: parity of the slot's next mbarrier phase
  bool inflight = false;      // lane 0: a copy whose wait gave up is still landing
  bool staging = !FINAL && q.slot_bytes > 0;
  if (lane == 0) {
    mbar_init(&bars[warp], 1);
    slot_key[warp] = kNone;
    slot_units[warp] = 0;
  }
  __syncwarp();
  const bool round0 = q.in_ray == nullptr;
  const uint32_t n_in = q.n_in ? *q.n_in : a.n;
  // nodes of the warp's staged treelet come from its slot
  auto lookup = [&](uint32_t unit, const uint2* meta) -> uint32_t {
    const uint32_t key = slot_key[warp];
    if (FINAL || key == kNone) return 0u;
    const uint32_t loc = __ldg(reinterpret_cast<const uint32_t*>(meta) + 2ull * unit + 1);
    if (loc == kNone || (loc >> kSlotBitsDev) != key) return 0u;
    const uint32_t u = loc & ((1u << kSlotBitsDev) - 1u);
    return u < slot_units[warp] ? slot_base + u * 64u : 0u;
  };
  unsigned long long stack[CAP + kColdWords];
  Walker<CAP, true, false, true> w;
  w.stk = stack;
  w.pin_base = 0;
  w.pin_root = 0;
  unsigned long long bytes = 0, staged = 0, stagings = 0, sreads = 0, greads = 0;

  if (FINAL) {
    // every ray still walking goes to its end, one node visit per iteration,
    // idle lanes refilled from the list (as run_persistent)
    bool have = false, exhausted = false;
    uint32_t r = 0;
    for (;;) {
      const uint32_t need = __ballot_sync(0xffffffffu, !have);
      if (!exhausted && need && (__popc(need) >= (int)a.refill || need == 0xffffffffu)) {
        const int leader = __ffs(need) - 1;
        uint32_t base = 0;
        if ((int)lane == leader) base = atomicAdd(q.take, (uint32_t)__popc(need));
        base = __shfl_sync(0xffffffffu, base, leader);
        if (base + (uint32_t)__popc(need) >= n_in) exhausted = true;
        if (!have) {
          const uint32_t p = base + (uint32_t)__popc(need & ((1u << lane) - 1u));
          if (p < n_in) {
            r = q.in_ray[p];
            w.ot = q.slab + (size_t)r * CAP;
            w.resume(a, r, q.state + 4ull * r);
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
        w.step(a, r, lookup);
        if (!w.active()) {
          w.finish(a, r);
          bytes += w.rec.bytes;
          sreads += w.smem_reads;
          greads += w.gmem_reads;
          have = false;
        }
      }
    }
  } else {
    for (;;) {
      uint32_t base = 0;
      if (lane == 0) base = atomicAdd(q.take, 32u);
      base = __shfl_sync(0xffffffffu, base, 0);
      if (base >= n_in) break;
      const uint32_t p = base + lane;
      const bool valid = p < n_in;
      const uint32_t r = valid ? (round0 ? p : q.in_ray[p]) : 0u;
      const uint32_t key = valid ? (round0 ? kNone : q.in_key[p]) : kNone;
      // stage the first queued ray's treelet (round 0: the TLAS root treelet,
      // found after the lanes' first push) unless the slot already holds it
      if (valid) {
        w.ot = q.slab + (size_t)r * CAP;
        if (round0) {
          w.init(a, r);
          w.save_ray(q.state + 4ull * r);
        } else {
          w.resume(a, r, q.state + 4ull * r);
        }
      }
      const bool live = valid && w.active();
      uint32_t want = key;
      if (round0 && live) {
        // the node the ray visits first (nxt, or the top of the other stack)
        const unsigned long long e = w.nxt ? w.nxt : w.ot_at(w.not_ - 1);
        const uint32_t loc = __ldg(reinterpret_cast<const uint32_t*>(a.meta) + 2ull * ((uint32_t)e >> kEShift) + 1);
        want = loc == kNone ? kNone : loc >> kSlotBitsDev;
      }
      const uint32_t first = __ballot_sync(0xffffffffu, live && want != kNone);
      if (staging && first) {
        const uint32_t t = __shfl_sync(0xffffffffu, want, __ffs(first) - 1);
        // stage it when at least min_votes of the chunk's rays are queued on it
        const uint32_t votes = __popc(__ballot_sync(0xffffffffu, live && want == t));
        if (t != slot_key[warp] && t < a.n_treelets && votes >= a.min_votes) {
          // every lane is done with the slot's previous treelet (the
          // __syncwarp closing the last chunk); lane 0 refills it
          uint32_t ok = 1;
          if (lane == 0) {
            const unsigned long long off = a.image_off[t];
            uint32_t nb = (uint32_t)(a.image_off[t + 1] - off);
            if (nb > q.slot_bytes) nb = q.slot_bytes;
            slot_key[warp] = kNone;
            if (nb > 0) {
              mbar_expect_tx(&bars[warp], nb);
              bulk_copy_g2s(slot, reinterpret_cast<const uint8_t*>(a.images) + off, nb, &bars[warp]);
              if (mbar_wait(&bars[warp], phase, kWaitTries)) {
                phase ^= 1u;
                slot_key[warp] = t;
                slot_units[warp] = nb / 64u;
                staged += nb;
                stagings += 1;
              } else {
                // this warp stops staging; the copy is waited for at exit
                inflight = true;
                ok = 0;
                atomicOr(a.status, kStatusTimeout);
              }
            }
          }
          staging = __shfl_sync(0xffffffffu, ok, 0) != 0;
          __syncwarp();  // the slot's key and contents before any lane reads them
        }
      }
      // each ray's stint: node visits while it stays in its current treelet
      bool go = live;
      while (__any_sync(0xffffffffu, go)) {
        if (go) {
          w.step(a, r, lookup);
          go = w.in_treelet();
        }
      }
      const bool cont = live && w.active();
      if (valid && !cont) {
        w.finish(a, r);
        bytes += w.rec.bytes;
      }
      if (valid) {
        sreads += w.smem_reads;
        greads += w.gmem_reads;
      }
      // rays that go on: state out, queued for the next round
      const uint32_t cmask = __ballot_sync(0xffffffffu, cont);
      if (cont) {
        w.suspend(q.state + 4ull * r);
        const uint32_t bin = next_bin(a, q, w);
        const int leader = __ffs(cmask) - 1;
        uint32_t o = 0;
        if ((int)lane == leader) o = atomicAdd(q.n_out, (uint32_t)__popc(cmask));
        o = __shfl_sync(cmask, o, leader) + (uint32_t)__popc(cmask & ((1u << lane) - 1u));
        q.out_ray[o] = r;
        q.out_key[o] = bin;
        add_grouped(q.hist, bin, cmask);
      }
      __syncwarp();
    }
  }
  // a copy still in flight after a wait that gave up must land before the
  // CTA's shared memory goes away
  if (!FINAL && lane == 0 && inflight) {
    if (!mbar_wait(&bars[warp], phase, kWaitTries)) atomicOr(a.status, kStatusTimeout);
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

// Exclusive scan of the bins, kBinScanItems per block: the offsets within
// the block into `offset`, the block's total into block_sum; the histogram is
// zeroed for the next round.
__global__ void __launch_bounds__(1024) bin_scan_kernel(uint32_t* hist, uint32_t* offset, uint32_t* block_sum,
                                                        uint32_t n_bins) {
  __shared__ uint32_t warp_sum[32];
  const uint32_t i0 = blockIdx.x * kBinScanItems + threadIdx.x * 4u;
  uint32_t v[4], s = 0;
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    v[k] = i0 + k < n_bins ? hist[i0 + k] : 0u;
    s += v[k];
  }
  const uint32_t lane = threadIdx.x & 31u, wid = threadIdx.x >> 5;
  uint32_t x = s;  // inclusive scan of the threads' sums within the warp
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    const uint32_t y = __shfl_up_sync(0xffffffffu, x, d);
    if ((int)lane >= d) x += y;
  }
  if (lane == 31) warp_sum[wid] = x;
  __syncthreads();
  if (wid == 0) {
    uint32_t t = warp_sum[lane];
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
      const uint32_t y = __shfl_up_sync(0xffffffffu, t, d);
      if ((int)lane >= d) t += y;
    }
    warp_sum[lane] = t;  // inclusive over warps
  }
  __syncthreads();
  uint32_t run = x - s + (wid ? warp_sum[wid - 1] : 0u);
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    if (i0 + k < n_bins) {
      offset[i0 + k] = run;
      hist[i0 + k] = 0;
    }
    run += v[k];
  }
  if (threadIdx.x == 1023) block_sum[blockIdx.x] = warp_sum[31];
}

// Exclusive scan of the block totals (one block; n_blocks <= 4096).
__global__ void __launch_bounds__(1024) bin_scan_top_kernel(uint32_t* block_sum, uint32_t n_blocks) {
  __shared__ uint32_t warp_sum[32];
  const uint32_t i0 = threadIdx.x * 4u;
  uint32_t v[4], s = 0;
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    v[k] = i0 + k < n_blocks ? block_sum[i0 + k] : 0u;
    s += v[k];
  }
  const uint32_t lane = threadIdx.x & 31u, wid = threadIdx.x >> 5;
  uint32_t x = s;
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    const uint32_t y = __shfl_up_sync(0xffffffffu, x, d);
    if ((int)lane >= d) x += y;
  }
  if (lane == 31) warp_sum[wid] = x;
  __syncthreads();
  if (wid == 0) {
    uint32_t t = warp_sum[lane];
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
      const uint32_t y = __shfl_up_sync(0xffffffffu, t, d);
      if ((int)lane >= d) t += y;
    }
    warp_sum[lane] = t;
  }
  __syncthreads();
  uint32_t run = x - s + (wid ? warp_sum[wid - 1] : 0u);
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    if (i0 + k < n_blocks) block_sum[i0 + k] = run;
    run += v[k];
  }
}

// Places every ray still walking at its bin's next free position: the rays
// queued on one treelet become contiguous.  offset[] serves as the bins'
// cursors (one atomic per distinct bin of a warp).
__global__ void __launch_bounds__(256) bin_scatter_kernel(const uint32_t* out_ray, const uint32_t* out_key,
                                                          const uint32_t* n_out, uint32_t* offset,
                                                          const uint32_t* block_sum, uint32_t* in_ray,
                                                          uint32_t* in_key) {
  const uint32_t n = *n_out;
  for (uint32_t i0 = blockIdx.x * blockDim.x; i0 < n; i0 += gridDim.x * blockDim.x) {
    const uint32_t i = i0 + threadIdx.x;
    const bool ok = i < n;
    const uint32_t mask = __ballot_sync(0xffffffffu, ok);
    if (!ok) continue;
    const uint32_t key = out_key[i];
    const uint32_t pos = block_sum[key / kBinScanItems] + add_grouped(offset, key, mask);
    in_ray[pos] = out_ray[i];
    in_key[pos] = key;
  }
}

}  // namespace rtk
