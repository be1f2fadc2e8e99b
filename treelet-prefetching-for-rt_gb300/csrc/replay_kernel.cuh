// RT-unit trace replay (rt_unit_replay): one CUDA thread runs one RT unit's
// model over the visit traces of its warps.  The model is the one described
// at rt_unit_replay in treelet_rt.h; this file is its GPU form.
//
// Per unit, in a slice of one device scratch buffer:
//   lines     sectored L1 (128 B lines, 4 x 32 B sectors, LRU stamps)
//   sectors   open-addressing map keyed by 32 B sector: prefetch records of
//             the sector still unclassified, per-class counts of classified
//             ones, and the state of the sector's most recently evicted
//             prefetch record.  A prefetch record is only ever classified
//             through the sector it filled or, once evicted, as the sector's
//             most recently evicted one, so the classification needs these
//             counts and no record list
//   queued    open-addressing map: live queued prefetch requests per address
//             (so a demand request scans the prefetch queue only when it can
//             match)
//   pq        the prefetch queue: a ring of (address, base) with tombstones
//   warps     resident warps in admission order, per lane a trace cursor
//   stride    the Lee stride tables of warp ids 0 .. max_warps-1
//   keys      the lanes' next-access treelets, sorted when they change
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/treelet_rt.h"
#include "format.h"

namespace rtr {

constexpr uint32_t kNone = 0xFFFFFFFFu;
constexpr uint32_t kChunkCap = 32 * 4;     // a round: 32 lanes x 128 B
constexpr uint32_t kMaxResident = 16;
constexpr uint32_t kMetaRing = 4096;       // > miss latency: metadata fills in flight
constexpr uint32_t kStrideEntries = 33;    // a stride table grows while it has <= 32 entries
constexpr uint32_t kTimeCap = 0xF0000000u; // cycles are 32-bit

struct Line {
  unsigned long long block;
  uint32_t lru;
  uint32_t flags;  // bit k: sector k valid; bit 4+k: filled by a prefetch; bit 8+k: that record unclassified
  uint32_t ready[4];
};

struct SectorEntry {
  unsigned long long key;  // sector + 1, 0 = empty
  uint32_t n_unclassified;
  uint32_t count[4];       // RT_PF_TOO_LATE .. RT_PF_TOO_EARLY
  uint32_t evicted;        // 0 none, 1 most recent evicted record unclassified, 2 classified
};

struct QueuedEntry {
  unsigned long long key;  // address + 1, 0 = empty
  uint32_t count;
  uint32_t pad;
};

struct Request {
  unsigned long long addr, base;
  uint32_t first, pad;
};

struct WarpSlot {
  uint32_t gid, wid, in_flight, all_sent, ready, ilat, issued;
  uint32_t live;  // lanes with transactions left
  uint32_t ptr[32], end[32];
};

struct StrideTable {
  uint32_t has, n;
  unsigned long long last;
  int stride[kStrideEntries];
  uint32_t count[kStrideEntries];
};

struct MetaReturn {
  uint32_t t, pad;
  unsigned long long base;
};

struct ReplayArgs {
  const rt_hit* hits;
  const uint32_t* visits;
  uint32_t n, capacity;
  rt_unit_config cfg;
  rt_unit_stats* stats;
  // scene
  const uint2* meta;
  uint32_t n_units;
  const uint32_t* roots;
  const unsigned long long* member_first;
  const uint32_t* members;
  const uint16_t* member_bytes;
  uint32_t n_treelets;
  unsigned long long meta_base, meta_size;
  // scratch
  uint8_t* scratch;
  unsigned long long unit_bytes;
  uint32_t sec_log2, queued_log2, pq_cap;
  uint32_t cycle_cap;  // per unit: the model's own bound on its cycles (or max_cycles)
  unsigned long long off_lines, off_sec, off_queued, off_pq, off_dead, off_chunk, off_warps, off_stride, off_meta,
      off_keys;
};

__device__ __forceinline__ uint32_t hash_slot(unsigned long long key, uint32_t log2) {
  return (uint32_t)((key * 0x9E3779B97F4A7C15ull) >> (64 - log2));
}

__device__ __forceinline__ uint32_t tx_size(uint32_t type) { return type == 2 ? 128u : (type == 3 ? 8u : 64u); }
__device__ __forceinline__ uint32_t intersection_latency(uint32_t type) {
  return (type == 0 || type == 3) ? 2u : 4u;  // 2,4,4,2,4,4,4
}

struct Unit {
  const ReplayArgs& a;
  const rt_unit_config& cfg;
  rt_unit_stats st;
  Line* lines;
  SectorEntry* sec;
  QueuedEntry* queued;
  unsigned long long* pq;  // pairs (addr, base)
  uint8_t* dead;
  Request* chunk;
  WarpSlot* warps;
  StrideTable* stride;
  MetaReturn* metaret;
  uint32_t* keys;
  // prefetch queue ring
  uint32_t pq_head, pq_tail, pq_live;
  // chunk queue of the warp being served
  uint32_t ch_head, ch_tail, serving;
  // resident warps in order (slot ids)
  uint32_t order[kMaxResident], n_res, free_mask;
  // metadata
  uint32_t mr_head, mr_tail;
  unsigned long long most_recent_metadata;
  // decision
  rt_prefetch_state ds;
  uint32_t n_keys, best, best_cnt, total, distinct;
  bool hist_dirty;
  bool full;

  __device__ Unit(const ReplayArgs& args, uint32_t u) : a(args), cfg(args.cfg) {
    uint8_t* base = a.scratch + (unsigned long long)u * a.unit_bytes;
    lines = reinterpret_cast<Line*>(base + a.off_lines);
    sec = reinterpret_cast<SectorEntry*>(base + a.off_sec);
    queued = reinterpret_cast<QueuedEntry*>(base + a.off_queued);
    pq = reinterpret_cast<unsigned long long*>(base + a.off_pq);
    dead = base + a.off_dead;
    chunk = reinterpret_cast<Request*>(base + a.off_chunk);
    warps = reinterpret_cast<WarpSlot*>(base + a.off_warps);
    stride = reinterpret_cast<StrideTable*>(base + a.off_stride);
    metaret = reinterpret_cast<MetaReturn*>(base + a.off_meta);
    keys = reinterpret_cast<uint32_t*>(base + a.off_keys);
    st = rt_unit_stats{};
    pq_head = pq_tail = pq_live = 0;
    ch_head = ch_tail = 0;
    serving = kNone;
    n_res = 0;
    free_mask = (1u << cfg.max_warps) - 1u;
    mr_head = mr_tail = 0;
    most_recent_metadata = 0;
    ds = rt_prefetch_state{kNone, kNone, kNone, 0};
    n_keys = 0;
    best = kNone;
    best_cnt = total = distinct = 0;
    hist_dirty = true;
    full = false;
  }

  // ------------------------------------------------------------ tables
  __device__ SectorEntry* sector_entry(unsigned long long sector, bool create) {
    const unsigned long long key = sector + 1;
    const uint32_t mask = (1u << a.sec_log2) - 1u;
    uint32_t i = hash_slot(key, a.sec_log2);
    for (uint32_t probe = 0; probe <= mask; ++probe, i = (i + 1) & mask) {
      SectorEntry& e = sec[i];
      if (e.key == key) return &e;
      if (e.key == 0) {
        if (!create) return nullptr;
        e.key = key;
        return &e;
      }
    }
    full = true;
    return nullptr;
  }

  __device__ QueuedEntry* queued_entry(unsigned long long addr, bool create) {
    const unsigned long long key = addr + 1;
    const uint32_t mask = (1u << a.queued_log2) - 1u;
    uint32_t i = hash_slot(key, a.queued_log2);
    for (uint32_t probe = 0; probe <= mask; ++probe, i = (i + 1) & mask) {
      QueuedEntry& e = queued[i];
      if (e.key == key) return &e;
      if (e.key == 0) {
        if (!create) return nullptr;
        e.key = key;
        return &e;
      }
    }
    full = true;
    return nullptr;
  }

  __device__ void classify(unsigned long long sector, uint32_t cls) {
    SectorEntry* e = sector_entry(sector, false);
    if (!e) return;
    e->n_unclassified--;
    e->count[cls]++;
  }

  // ------------------------------------------------------------ cache
  __device__ Line* find(unsigned long long block) {
    Line* set = lines + (size_t)(block & (cfg.l1_sets - 1)) * cfg.l1_ways;
    for (uint32_t w = 0; w < cfg.l1_ways; ++w)
      if ((set[w].flags & 0x80000000u) && set[w].block == block) return &set[w];
    return nullptr;
  }

  __device__ Line* allocate(unsigned long long block, uint32_t t) {
    Line* set = lines + (size_t)(block & (cfg.l1_sets - 1)) * cfg.l1_ways;
    Line* v = nullptr;
    for (uint32_t w = 0; w < cfg.l1_ways && !v; ++w)
      if (!(set[w].flags & 0x80000000u)) v = &set[w];
    if (!v) {
      for (uint32_t w = 0; w < cfg.l1_ways; ++w)
        if (!v || set[w].lru < v->lru) v = &set[w];
      for (uint32_t k = 0; k < 4; ++k)
        if ((v->flags >> k) & (v->flags >> (4 + k)) & 1u) {
          SectorEntry* e = sector_entry(v->block * 4 + k, false);
          if (e) e->evicted = ((v->flags >> (8 + k)) & 1u) ? 1u : 2u;
        }
    }
    v->block = block;
    v->flags = 0x80000000u;
    v->lru = t;
    return v;
  }

  __device__ uint32_t demand(unsigned long long addr, uint32_t t) {
    const unsigned long long sector = addr >> 5, block = addr >> 7;
    const uint32_t k = (uint32_t)((addr >> 5) & 3);
    st.demand_requests++;
    Line* l = find(block);
    if (l && ((l->flags >> k) & 1u)) {
      l->lru = t;
      const bool pf_uncl = (l->flags >> (4 + k)) & (l->flags >> (8 + k)) & 1u;
      if (l->ready[k] <= t) {
        st.demand_hits++;
        if (pf_uncl) {
          classify(sector, RT_PF_TIMELY);
          l->flags &= ~(1u << (8 + k));
        }
        return t + cfg.hit_latency;
      }
      st.demand_hit_reserved++;
      if (pf_uncl) {
        classify(sector, RT_PF_LATE);
        l->flags &= ~(1u << (8 + k));
      }
      return l->ready[k];
    }
    st.demand_misses++;
    SectorEntry* e = sector_entry(sector, false);
    if (e && e->evicted == 1u) {
      e->n_unclassified--;
      e->count[RT_PF_TOO_EARLY]++;
      e->evicted = 2u;
    }
    if (!l) l = allocate(block, t);
    l->lru = t;
    l->flags = (l->flags | (1u << k)) & ~((1u << (4 + k)) | (1u << (8 + k)));
    l->ready[k] = t + cfg.miss_latency;
    return t + cfg.miss_latency;
  }

  __device__ bool is_metadata(unsigned long long base) const {
    return cfg.load_metadata && base >= a.meta_base && base <= a.meta_base + (unsigned long long)a.n_treelets * a.meta_size;
  }

  __device__ void prefetch(unsigned long long addr, unsigned long long base, uint32_t t) {
    const unsigned long long sector = addr >> 5, block = addr >> 7;
    const uint32_t k = (uint32_t)((addr >> 5) & 3);
    st.prefetch_issued++;
    SectorEntry* e = sector_entry(sector, true);
    if (e) e->n_unclassified++;
    Line* l = find(block);
    if (l && ((l->flags >> k) & 1u)) {
      l->lru = t;
      // a fresh record is unclassified, so the TOO_LATE rule of
      // gpu-cache.cc:2101-2116 never applies to it
      if (l->ready[k] <= t) st.prefetch_present++;
      else st.prefetch_merged++;
      return;
    }
    st.prefetch_filled++;
    if (!l) l = allocate(block, t);
    l->lru = t;
    l->flags |= (1u << k) | (1u << (4 + k)) | (1u << (8 + k));
    l->ready[k] = t + cfg.miss_latency;
    if (is_metadata(base)) {
      if (mr_tail - mr_head < kMetaRing) {
        metaret[mr_tail % kMetaRing] = MetaReturn{t + cfg.miss_latency, 0u, base};
        ++mr_tail;
      } else {
        full = true;
      }
    }
  }

  // ------------------------------------------------------------ prefetch queue
  __device__ void pq_push(unsigned long long addr, unsigned long long base) {
    st.prefetch_queued++;
    if (pq_tail - pq_head >= a.pq_cap) {  // ring full (live + erased entries)
      full = true;
      return;
    }
    const uint32_t i = pq_tail % a.pq_cap;
    pq[2 * i] = addr;
    pq[2 * i + 1] = base;
    dead[i] = 0;
    ++pq_tail;
    ++pq_live;
    QueuedEntry* q = queued_entry(addr, true);
    if (q) q->count++;
  }

  __device__ void pq_drop_dead() {
    while (pq_head != pq_tail && dead[pq_head % a.pq_cap]) ++pq_head;
  }

  // Erases queued prefetches of `addr`, stepping past the entry that follows
  // each erased one (shader.cc:4657-4668 as written).
  __device__ void remove_queued(unsigned long long addr) {
    QueuedEntry* q = queued_entry(addr, false);
    if (!q || q->count == 0) return;
    bool skip = false;
    for (uint32_t p = pq_head; p != pq_tail; ++p) {
      const uint32_t i = p % a.pq_cap;
      if (dead[i]) continue;
      if (skip) {
        skip = false;
        continue;
      }
      if (pq[2 * i] == addr) {
        dead[i] = 1;
        --pq_live;
        q->count--;
        st.prefetch_removed++;
        skip = true;
      }
    }
    pq_drop_dead();
  }

  __device__ uint32_t dense_of(uint32_t root) const {
    uint32_t lo = 0, hi = a.n_treelets;
    while (lo < hi) {
      const uint32_t mid = (lo + hi) >> 1;
      if (__ldg(a.roots + mid) < root) lo = mid + 1;
      else hi = mid;
    }
    return (lo < a.n_treelets && __ldg(a.roots + lo) == root) ? lo : kNone;
  }

  __device__ void push_member(unsigned long long j, bool with_metadata) {
    const uint32_t m = __ldg(a.members + j);
    if (with_metadata && cfg.load_metadata) {
      const uint32_t d = dense_of(m);  // treelet_addr_to_metadata_idx: 0 for a member that is no root
      const unsigned long long ma = a.meta_base + (unsigned long long)(d == kNone ? 0u : d) * a.meta_size;
      for (unsigned long long i = 0; i < a.meta_size / 32; ++i) {
        pq_push(ma + i * 32, ma);
        st.metadata_queued++;
      }
    }
    const unsigned long long addr = (unsigned long long)m * 64;
    const uint32_t b = __ldg(a.member_bytes + j);
    for (uint32_t i = 0; i < (b + 31) / 32; ++i) pq_push(addr + 32ull * i, addr);
  }

  // ------------------------------------------------------------ decision
  __device__ uint32_t lane_root(const WarpSlot& w, uint32_t lane) const {
    const uint32_t r = w.gid * 32 + lane;
    const uint32_t unit = __ldg(a.visits + (unsigned long long)r * a.capacity + w.ptr[lane]) >> 3;
    return unit < a.n_units ? __ldg(&a.meta[unit].x) : kNone;
  }

  __device__ void rebuild_histogram() {
    n_keys = 0;
    for (uint32_t o = 0; o < n_res; ++o) {
      const WarpSlot& w = warps[order[o]];
      for (uint32_t l = 0; l < 32; ++l)
        if (w.ptr[l] < w.end[l]) {
          const uint32_t k = lane_root(w, l);
          if (k != kNone) keys[n_keys++] = k;
        }
    }
    // shell sort (Ciura gaps)
    const uint32_t gaps[8] = {701, 301, 132, 57, 23, 10, 4, 1};
    for (uint32_t g = 0; g < 8; ++g) {
      const uint32_t gap = gaps[g];
      for (uint32_t i = gap; i < n_keys; ++i) {
        const uint32_t v = keys[i];
        uint32_t j = i;
        while (j >= gap && keys[j - gap] > v) {
          keys[j] = keys[j - gap];
          j -= gap;
        }
        keys[j] = v;
      }
    }
    best = kNone;
    best_cnt = 0;
    total = n_keys;
    distinct = 0;
    for (uint32_t i = 0; i < n_keys;) {
      uint32_t j = i;
      while (j < n_keys && keys[j] == keys[i]) ++j;
      ++distinct;
      if (best == kNone || j - i > best_cnt) {  // first maximum in ascending root order
        best = keys[i];
        best_cnt = j - i;
      }
      i = j;
    }
    hist_dirty = false;
  }

  // The RT unit's decision (shader.cc:3419-3683; as prefetch_decide_kernel).
  __device__ void decide() {
    if (hist_dirty) rebuild_histogram();
    st.decisions++;
    const rt_prefetch_params& p = cfg.decision;
    bool submit = false;
    int num_nodes = 0, n_nodes = 0;
    const uint32_t bd = best == kNone ? kNone : dense_of(best);
    if (bd != kNone) n_nodes = (int)(__ldg(a.member_first + bd + 1) - __ldg(a.member_first + bd));
    if (p.heuristic == RT_PREFETCH_ALWAYS) {
      submit = true;
    } else if (best != kNone) {
      const double pct = (double)best_cnt / (double)total;
      if (p.heuristic == RT_PREFETCH_POPULARITY) {
        if (pct >= p.threshold) {
          ds.last_rejected = kNone;
          submit = true;
        } else if (ds.last_rejected != best) {
          ds.last_rejected = best;
        }
      } else {
        num_nodes = (int)(((double)n_nodes * pct) + 0.5);
        submit = true;
      }
    }
    unsigned long long queue = pq_live;
    if (submit && best != kNone && bd != kNone && ds.last_prefetched != best && ds.last_prefetched_second != best) {
      const bool partial = p.heuristic == RT_PREFETCH_PARTIAL || p.heuristic == RT_PREFETCH_LATTER;
      const int num = partial ? num_nodes : n_nodes;
      if ((unsigned long long)num + queue <= p.max_queue) {
        const int j0 = p.heuristic == RT_PREFETCH_LATTER ? n_nodes - num : 0;
        const int j1 = p.heuristic == RT_PREFETCH_LATTER ? n_nodes : num;
        const unsigned long long mf = __ldg(a.member_first + bd);
        for (int j = j0; j < j1; ++j) {
          queue += (__ldg(a.member_bytes + mf + j) + 31u) / 32u;
          push_member(mf + j, true);
        }
        ds.last_prefetched = best;
        st.treelets_prefetched++;
      }
    }
    if (p.second_prefetch && queue == 0 && total > 0 && distinct > 1 && ds.last_prefetched == best && best != kNone) {
      uint32_t second = kNone, scnt = 0;
      for (uint32_t i = 0; i < n_keys;) {
        uint32_t j = i;
        while (j < n_keys && keys[j] == keys[i]) ++j;
        if (keys[i] != ds.last_prefetched && (second == kNone || j - i > scnt)) {
          second = keys[i];
          scnt = j - i;
        }
        i = j;
      }
      if (second != kNone && ds.last_prefetched_second != second) {
        const uint32_t sd = dense_of(second);
        if (sd != kNone)
          for (unsigned long long j = __ldg(a.member_first + sd); j < __ldg(a.member_first + sd + 1); ++j)
            push_member(j, false);
        ds.last_prefetched_second = second;
        st.treelets_prefetched++;
      }
    }
  }

  // ------------------------------------------------------------ stride (Lee MICRO'10)
  __device__ void stride_prefetch(uint32_t wid, unsigned long long next_addr) {
    StrideTable& s = stride[wid];
    if (!s.has) {
      s.last = next_addr;
    } else if (s.n <= 32) {
      const int d = (int)(uint32_t)(next_addr - s.last);
      uint32_t i = 0;
      while (i < s.n && s.stride[i] < d) ++i;
      if (i < s.n && s.stride[i] == d) {
        s.count[i]++;
      } else {
        for (uint32_t k = s.n; k > i; --k) {
          s.stride[k] = s.stride[k - 1];
          s.count[k] = s.count[k - 1];
        }
        s.stride[i] = d;
        s.count[i] = 1;
        s.n++;
      }
    }
    s.has = 1;  // the table lookup below creates the warp's (empty) table
    int largest = 0;
    uint32_t largest_count = 0;
    for (uint32_t i = 0; i < s.n; ++i)
      if (s.count[i] > largest_count) {
        largest = s.stride[i];
        largest_count = s.count[i];
      }
    const unsigned long long pa = next_addr + (unsigned long long)(long long)largest;
    if (cfg.decision.max_queue <= pq_live) {
      pq_push(pa, pa);
      pq_push(pa + 32, pa);
    }
  }

  // ------------------------------------------------------------ warps
  __device__ bool warp_ready(const WarpSlot& w) const { return !w.in_flight && w.live != 0; }

  __device__ uint32_t matching_lanes(const WarpSlot& w) const {
    if (ds.last_prefetched == kNone) return 0;
    uint32_t c = 0;
    for (uint32_t l = 0; l < 32; ++l)
      if (w.ptr[l] < w.end[l] && lane_root(w, l) == ds.last_prefetched) ++c;
    return c;
  }

  // rt_unit::schedule_next_warp (shader.cc:4307-4392)
  __device__ uint32_t schedule() const {
    const bool treelet = cfg.prefetcher == RT_UNIT_PF_TREELET;
    if (treelet && cfg.scheduler == RT_UNIT_SCHED_OMR) {
      for (uint32_t o = 0; o < n_res; ++o)
        if (warp_ready(warps[order[o]]) && matching_lanes(warps[order[o]]) > 0) return order[o];
    } else if (treelet && cfg.scheduler == RT_UNIT_SCHED_PMR) {
      uint32_t b = kNone, bc = 0;
      for (uint32_t o = 0; o < n_res; ++o)
        if (warp_ready(warps[order[o]])) {
          const uint32_t c = matching_lanes(warps[order[o]]);
          if (c > bc) {
            b = order[o];
            bc = c;
          }
        }
      if (b != kNone) return b;
    }
    for (uint32_t o = 0; o < n_res; ++o)
      if (warp_ready(warps[order[o]])) return order[o];
    return kNone;
  }

  __device__ void start_round(uint32_t slot) {
    WarpSlot& w = warps[slot];
    uint32_t ilat = 0, issued = 0;
    ch_head = ch_tail = 0;
    for (uint32_t l = 0; l < 32; ++l) {
      if (w.ptr[l] >= w.end[l]) continue;
      issued |= 1u << l;
      const uint32_t v = __ldg(a.visits + (unsigned long long)(w.gid * 32 + l) * a.capacity + w.ptr[l]);
      const unsigned long long addr = (unsigned long long)(v >> 3) * 64;
      const uint32_t size = tx_size(v & 7);
      ilat = max(ilat, intersection_latency(v & 7));
      bool dup = false;  // an (address, size) pair already in this round
      for (uint32_t l2 = 0; l2 < l && !dup; ++l2) {
        if (!((issued >> l2) & 1u)) continue;
        const uint32_t v2 = __ldg(a.visits + (unsigned long long)(w.gid * 32 + l2) * a.capacity + w.ptr[l2]);
        dup = (v2 >> 3) == (v >> 3) && tx_size(v2 & 7) == size;
      }
      if (dup) continue;
      for (uint32_t i = 0; i < (size + 31) / 32; ++i) chunk[ch_tail++] = Request{addr + 32ull * i, addr, i == 0 ? 1u : 0u, 0u};
    }
    w.issued = issued;
    w.in_flight = 1;
    w.all_sent = 0;
    w.ready = 0;
    w.ilat = ilat;
    serving = slot;
  }

  __device__ void send_demand(uint32_t t) {
    const Request r = chunk[ch_head++];
    if (cfg.prefetcher == RT_UNIT_PF_TREELET || cfg.prefetcher == RT_UNIT_PF_STRIDE) remove_queued(r.addr);
    WarpSlot& w = warps[serving];
    if (cfg.prefetcher == RT_UNIT_PF_STRIDE && r.first) stride_prefetch(w.wid, r.addr);
    const uint32_t ret = demand(r.addr, t);
    w.ready = max(w.ready, ret);
    if (ch_head == ch_tail) {
      w.all_sent = 1;
      w.ready += w.ilat;
      serving = kNone;
    }
  }

  __device__ bool prefetch_issuable() const {
    const unsigned long long base = pq[2 * (pq_head % a.pq_cap) + 1];
    if (!cfg.wait_metadata || is_metadata(base)) return true;
    // shader.cc:4469-4476: the metadata of the treelet the request's base node belongs to
    const unsigned long long unit = base >> 6;
    const uint32_t root = (base % 64 == 0 && unit < a.n_units) ? __ldg(&a.meta[unit].x) : kNone;
    const uint32_t d = root == kNone ? kNone : dense_of(root);
    return most_recent_metadata == a.meta_base + (unsigned long long)(d == kNone ? 0u : d) * a.meta_size;
  }

  __device__ void run(uint32_t u) {
    const uint32_t n_warps = (a.n + 31) / 32;
    uint32_t next_gid = u, local = 0;
    const uint32_t tcap = a.cycle_cap;
    for (uint32_t k = 0; k < cfg.max_warps; ++k) stride[k].has = stride[k].n = 0;
    for (uint32_t t = 0;; ++t) {
      // rounds whose data is back, warps that are done
      uint32_t keep = 0;
      for (uint32_t o = 0; o < n_res; ++o) {
        WarpSlot& w = warps[order[o]];
        if (w.in_flight && w.all_sent && w.ready <= t) {
          for (uint32_t l = 0; l < 32; ++l)
            if ((w.issued >> l) & 1u) {
              if (++w.ptr[l] >= w.end[l]) w.live &= ~(1u << l);
              st.transactions++;
            }
          w.issued = 0;
          w.in_flight = 0;
          hist_dirty = true;
        }
        if (!w.in_flight && !warp_ready(w)) {
          st.warps++;
          free_mask |= 1u << order[o];
          hist_dirty = true;
        } else {
          order[keep++] = order[o];
        }
      }
      n_res = keep;
      while (n_res < cfg.max_warps && next_gid < n_warps) {
        const uint32_t slot = __ffs(free_mask) - 1;
        free_mask &= ~(1u << slot);
        WarpSlot& w = warps[slot];
        w.gid = next_gid;
        w.wid = local++ % cfg.max_warps;
        w.in_flight = w.all_sent = 0;
        w.ready = w.ilat = w.issued = w.live = 0;
        for (uint32_t l = 0; l < 32; ++l) {
          const uint32_t r = next_gid * 32 + l;
          w.ptr[l] = 0;
          w.end[l] = r < a.n ? min(a.hits[r].n_visits, a.capacity) : 0u;
          if (w.end[l]) w.live |= 1u << l;
        }
        order[n_res++] = slot;
        next_gid += cfg.n_rt_units;
        hist_dirty = true;
      }
      if (n_res == 0) {
        st.cycles = t;
        break;
      }
      if (t >= tcap) {
        st.cycles = t;
        st.status |= 2;
        break;
      }
      while (mr_head != mr_tail && metaret[mr_head % kMetaRing].t <= t) {
        most_recent_metadata = metaret[mr_head % kMetaRing].base;
        ++mr_head;
      }
      if (cfg.prefetcher == RT_UNIT_PF_TREELET && t % cfg.prefetch_delay == 0) decide();
      if (ch_head != ch_tail) {
        send_demand(t);
      } else {
        const uint32_t s = schedule();
        if (s != kNone) {
          start_round(s);
          send_demand(t);
        } else if (cfg.prefetcher != RT_UNIT_PF_NONE && pq_live > 0 && prefetch_issuable()) {
          const uint32_t i = pq_head % a.pq_cap;
          const unsigned long long addr = pq[2 * i], base = pq[2 * i + 1];
          dead[i] = 1;
          --pq_live;
          QueuedEntry* q = queued_entry(addr, false);
          if (q) q->count--;
          pq_drop_dead();
          prefetch(addr, base, t);
        }
      }
    }
    // final tally (gpu-sim.cc:1749-1790)
    const uint32_t n_sec = 1u << a.sec_log2;
    for (uint32_t i = 0; i < n_sec; ++i) {
      const SectorEntry& e = sec[i];
      if (!e.key) continue;
      const uint32_t classified = e.count[0] + e.count[1] + e.count[2] + e.count[3];
      if (classified) {
        st.unclassified_but_accessed += e.n_unclassified;
        for (uint32_t c = 0; c < 4; ++c) st.effectiveness[c] += e.count[c];
      } else {
        st.effectiveness[RT_PF_NEVER_USED] += e.n_unclassified;
      }
    }
    if (full) st.status |= 1;
  }
};

__global__ void __launch_bounds__(64) unit_replay_kernel(ReplayArgs a) {
  const uint32_t u = blockIdx.x * blockDim.x + threadIdx.x;
  if (u >= a.cfg.n_rt_units) return;
  Unit unit(a, u);
  unit.run(u);
  a.stats[u] = unit.st;
}

}  // namespace rtr
