// Treelet-prefetch decision of an RT unit (src/gpgpu-sim/shader.cc:3419-3683,
// or the copies the pipelined treelet queue, :3780-3932, and the treelet
// queue, :4020-4060, run) as a batched kernel: one CTA per RT unit.
//
// The reference builds std::map<treelet root, count> over the first pending
// access of every resident lane, takes the first maximum in ascending root
// order, applies the heuristic, and queues the treelet's members as 32-byte
// requests unless it was the last (or last second) treelet prefetched.  Here
// the lanes' roots are sorted in shared memory (bitonic), runs give the
// counts, and thread 0 applies the same heuristic arithmetic (IEEE double for
// the popularity share, as in the reference).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/treelet_rt.h"

namespace rtk {

constexpr int kMaxLanes = 1024;

struct PrefetchArgs {
  const uint32_t* next_unit;
  uint32_t n_groups, lanes;
  rt_prefetch_params p;
  rt_prefetch_state* state;
  rt_prefetch_decision* out;
  const uint2* meta;                 // unit -> root
  uint32_t n_units;
  const uint32_t* roots;             // dense -> root unit (ascending)
  const unsigned long long* member_first;  // dense -> first member, n + 1
  const uint16_t* member_bytes;
  uint32_t n_treelets;
};

__device__ __forceinline__ uint32_t dense_of_root(const PrefetchArgs& a, uint32_t root) {
  uint32_t lo = 0, hi = a.n_treelets;
  while (lo < hi) {
    const uint32_t mid = (lo + hi) >> 1;
    if (a.roots[mid] < root) lo = mid + 1;
    else hi = mid;
  }
  return (lo < a.n_treelets && a.roots[lo] == root) ? lo : kNone;
}

__global__ void __launch_bounds__(512) prefetch_decide_kernel(PrefetchArgs a) {
  __shared__ uint32_t keys[kMaxLanes];
  __shared__ uint32_t nkeys;
  const uint32_t g = blockIdx.x;
  const uint32_t tid = threadIdx.x;
  uint32_t padded = 1;
  while (padded < a.lanes) padded <<= 1;
  for (uint32_t l = tid; l < padded; l += blockDim.x) {
    uint32_t k = kNone;
    if (l < a.lanes) {
      const uint32_t u = a.next_unit[(uint64_t)g * a.lanes + l];
      if (u != kNone && u < a.n_units) k = a.meta[u].x;
    }
    keys[l] = k;
  }
  __syncthreads();
  // bitonic sort ascending (kNone sorts last)
  for (uint32_t size = 2; size <= padded; size <<= 1) {
    for (uint32_t stride = size >> 1; stride > 0; stride >>= 1) {
      for (uint32_t i = tid; i < padded; i += blockDim.x) {
        const uint32_t j = i ^ stride;
        if (j > i) {
          const bool up = (i & size) == 0;
          const uint32_t x = keys[i], y = keys[j];
          if ((x > y) == up) {
            keys[i] = y;
            keys[j] = x;
          }
        }
      }
      __syncthreads();
    }
  }
  if (tid != 0) return;
  // runs: first maximum in ascending order; distinct count; total
  uint32_t total = 0, distinct = 0, best = kNone, best_cnt = 0;
  {
    uint32_t i = 0;
    while (i < padded && keys[i] != kNone) {
      uint32_t j = i;
      while (j < padded && keys[j] == keys[i]) ++j;
      const uint32_t c = j - i;
      total += c;
      ++distinct;
      if (best == kNone || c > best_cnt) {  // strict >: the lowest root wins ties
        best = keys[i];
        best_cnt = c;
      }
      i = j;
    }
    nkeys = i;
  }
  rt_prefetch_state st = a.state[g];
  const uint32_t copy = a.p.variant & 3u;
  const bool pipelined = copy == RT_PREFETCH_PIPELINED_QUEUE;
  const bool flush = (a.p.variant & RT_PREFETCH_FLUSH_ON_NEW_TREELET) != 0;
  rt_prefetch_decision d;
  d.treelet = best;
  d.count = best == kNone ? 0u : best_cnt;
  d.total = total;
  d.submitted = 0;
  d.first_member = 0;
  d.n_members = 0;
  d.chunks = 0;
  d.second_treelet = kNone;
  bool submit = false;
  int num_nodes = 0;
  uint32_t bd = kNone;
  int n_nodes = 0;
  if (best != kNone) {
    bd = dense_of_root(a, best);
    if (bd != kNone) n_nodes = (int)(a.member_first[bd + 1] - a.member_first[bd]);
  }
  uint64_t queue = st.queue_len;
  if (copy == RT_PREFETCH_TREELET_QUEUE) {
    // the treelet queue's copy: the whole treelet whatever the heuristic,
    // unless it was the last one prefetched; an empty histogram names no
    // treelet (an empty member list) and is recorded as the last one
    if (st.last_prefetched != best && (uint64_t)n_nodes + queue <= a.p.max_queue) {
      uint32_t chunks = 0;
      if (bd != kNone)
        for (int j = 0; j < n_nodes; ++j) chunks += (a.member_bytes[a.member_first[bd] + j] + 31u) / 32u;
      queue += chunks;
      d.submitted = best != kNone ? 1u : 0u;
      d.n_members = (uint32_t)n_nodes;
      d.chunks = chunks;
      st.last_prefetched = best;
    }
    st.queue_len = (uint32_t)queue;
    a.state[g] = st;
    a.out[g] = d;
    return;
  }
  if (a.p.heuristic == RT_PREFETCH_ALWAYS) {
    submit = true;
  } else if (best != kNone) {
    const double pct = (double)best_cnt / (double)total;
    if (a.p.heuristic == RT_PREFETCH_POPULARITY) {
      if (pct >= a.p.threshold) {
        st.last_rejected = kNone;
        submit = true;
      } else {
        if (st.last_rejected != best) st.last_rejected = best;
      }
    } else {
      // the pipelined queue's copy sizes LATTER at half the treelet
      const double share = (pipelined && a.p.heuristic == RT_PREFETCH_LATTER) ? 0.5 : pct;
      num_nodes = (int)(((double)n_nodes * share) + 0.5);
      submit = true;
    }
  }
  if (submit && best != kNone && bd != kNone) {
    if (st.last_prefetched != best && (pipelined || st.last_prefetched_second != best)) {
      const bool partial = a.p.heuristic == RT_PREFETCH_PARTIAL || a.p.heuristic == RT_PREFETCH_LATTER;
      const int num = partial ? num_nodes : n_nodes;
      if ((uint64_t)num + queue <= a.p.max_queue) {
        if (flush) queue = 0;
        const int j0 = a.p.heuristic == RT_PREFETCH_LATTER ? n_nodes - num : 0;
        const int j1 = a.p.heuristic == RT_PREFETCH_LATTER ? n_nodes : num;
        uint32_t chunks = 0;
        for (int j = j0; j < j1; ++j) chunks += (a.member_bytes[a.member_first[bd] + j] + 31u) / 32u;
        queue += chunks;
        d.submitted = 1;
        d.first_member = (uint32_t)j0;
        d.n_members = (uint32_t)(j1 - j0);
        d.chunks = chunks;
        st.last_prefetched = best;
      }
    }
  }
  if (a.p.second_prefetch && !pipelined && queue == 0 && total > 0 && distinct > 1 && st.last_prefetched == best &&
      best != kNone) {
    // next most popular treelet other than the last prefetched one
    uint32_t second = kNone, scnt = 0;
    uint32_t i = 0;
    while (i < nkeys) {
      uint32_t j = i;
      while (j < nkeys && keys[j] == keys[i]) ++j;
      const uint32_t c = j - i;
      if (keys[i] != st.last_prefetched && (second == kNone || c > scnt)) {
        second = keys[i];
        scnt = c;
      }
      i = j;
    }
    if (second != kNone && st.last_prefetched_second != second) {
      const uint32_t sd = dense_of_root(a, second);
      uint32_t chunks = 0;
      if (sd != kNone)
        for (unsigned long long j = a.member_first[sd]; j < a.member_first[sd + 1]; ++j)
          chunks += (a.member_bytes[j] + 31u) / 32u;
      queue += chunks;
      d.chunks += chunks;
      d.second_treelet = second;
      st.last_prefetched_second = second;
    }
  }
  st.queue_len = (uint32_t)queue;
  a.state[g] = st;
  a.out[g] = d;
}

}  // namespace rtk
