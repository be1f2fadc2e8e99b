// RT-unit trace replay (rt_unit_replay): one warp runs one RT unit's model
// over the visit traces of its warps.  The model is the one described at
// rt_unit_replay in treelet_rt.h; this file is its GPU form.
//
// The model advances one cycle at a time and sends at most one 32-byte
// request per cycle, so a unit is a sequential loop.  The warp works the
// parts of a cycle that have lanes in them: the L1 set (one lane per way),
// the resident warps (one lane per warp), a round's 32 lanes (one lane per
// RT lane, identical requests merged with __match_any_sync), the sorted
// histogram of next treelets, and the prefetch-queue scans.  Lane 0 keeps
// the unit's counters and makes the single-request updates.
//
// Per unit, in shared memory: the unit's scalar state, the resident warps
// (per RT lane a trace cursor), the current round's requests, the histogram
// keys, the stride tables and, when they fit, the L1 lines.  In a slice of
// one device scratch buffer:
//   lines     sectored L1 (128 B lines, 4 x 32 B sectors, LRU stamps), when
//             they do not fit in shared memory
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
//   metaret   metadata fills in flight
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/treelet_rt.h"
#include "format.h"

namespace rtr {

constexpr uint32_t kNone = 0xFFFFFFFFu;
constexpr uint32_t kFull = 0xFFFFFFFFu;
constexpr uint32_t kChunkCap = 32 * 4;     // a round: 32 lanes x 128 B
constexpr uint32_t kMaxResident = 16;
constexpr uint32_t kMaxKeys = 32 * kMaxResident;
constexpr uint32_t kMetaRing = 4096;       // > miss latency: metadata fills in flight
constexpr uint32_t kStrideEntries = 33;    // a stride table grows while it has <= 32 entries
constexpr uint32_t kTimeCap = 0xF0000000u; // cycles are 32-bit
constexpr uint32_t kLineValid = 0x80000000u;
constexpr uint32_t kSmemLinesMax = 1536;   // lines kept in shared memory (48 KiB)

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

// The unit's scalar state (shared memory; lane 0 writes, __syncwarp, all read).
struct UnitState {
  rt_unit_stats st;
  unsigned long long most_recent_metadata;
  rt_prefetch_state ds;
  uint32_t pq_head, pq_tail, pq_live;
  uint32_t ch_head, ch_tail, serving;
  uint32_t order[kMaxResident], n_res, free_mask;
  uint32_t mr_head, mr_tail;
  // histogram summary of the lanes' next treelets
  uint32_t n_keys, best, best_cnt, total, distinct, best_dense, best_nodes, second, hist_dirty;
  uint32_t full, next_gid, local;
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
  uint32_t cycle_cap;     // per unit: the model's own bound on its cycles (or max_cycles)
  uint32_t lines_shared;  // 1: the L1 lines live in shared memory
  unsigned long long off_lines, off_sec, off_queued, off_pq, off_dead, off_meta;
};

// Dynamic shared memory of one unit (one warp per CTA).
struct UnitShared {
  UnitState s;
  WarpSlot warps[kMaxResident];
  Request chunk[kChunkCap];
  uint32_t keys[kMaxKeys];
  StrideTable stride[kMaxResident];
};

__device__ __forceinline__ uint32_t hash_slot(unsigned long long key, uint32_t log2) {
  return (uint32_t)((key * 0x9E3779B97F4A7C15ull) >> (64 - log2));
}

__device__ __forceinline__ uint32_t tx_size(uint32_t type) { return type == 2 ? 128u : (type == 3 ? 8u : 64u); }
__device__ __forceinline__ uint32_t intersection_latency(uint32_t type) {
  return (type == 0 || type == 3) ? 2u : 4u;  // 2,4,4,2,4,4,4
}

__device__ __forceinline__ uint32_t lanemask_lt() {
  return (1u << (threadIdx.x & 31u)) - 1u;
}

__device__ __forceinline__ unsigned long long warp_max64(unsigned long long v) {
#pragma unroll
  for (int s = 16; s > 0; s >>= 1) {
    const unsigned long long o = __shfl_xor_sync(kFull, v, s);
    v = o > v ? o : v;
  }
  return v;
}

__device__ __forceinline__ unsigned long long warp_min64(unsigned long long v) {
#pragma unroll
  for (int s = 16; s > 0; s >>= 1) {
    const unsigned long long o = __shfl_xor_sync(kFull, v, s);
    v = o < v ? o : v;
  }
  return v;
}

__device__ __forceinline__ uint32_t warp_sum(uint32_t v) { return __reduce_add_sync(kFull, v); }

struct WUnit {
  const ReplayArgs& a;
  const rt_unit_config& cfg;
  const uint32_t lane;
  UnitShared& sh;
  UnitState& S;
  Line* lines;
  SectorEntry* sec;
  QueuedEntry* queued;
  unsigned long long* pq;  // pairs (addr, base)
  uint8_t* dead;
  MetaReturn* metaret;

  __device__ WUnit(const ReplayArgs& args, uint32_t u, UnitShared& shm, Line* smem_lines)
      : a(args), cfg(args.cfg), lane(threadIdx.x & 31u), sh(shm), S(shm.s) {
    uint8_t* base = a.scratch + (unsigned long long)u * a.unit_bytes;
    lines = a.lines_shared ? smem_lines : reinterpret_cast<Line*>(base + a.off_lines);
    sec = reinterpret_cast<SectorEntry*>(base + a.off_sec);
    queued = reinterpret_cast<QueuedEntry*>(base + a.off_queued);
    pq = reinterpret_cast<unsigned long long*>(base + a.off_pq);
    dead = base + a.off_dead;
    metaret = reinterpret_cast<MetaReturn*>(base + a.off_meta);
  }

  // ------------------------------------------------------------ tables (lane 0)
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
    S.full = 1;
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
    S.full = 1;
    return nullptr;
  }

  __device__ void classify(unsigned long long sector, uint32_t cls) {
    SectorEntry* e = sector_entry(sector, false);
    if (!e) return;
    e->n_unclassified--;
    e->count[cls]++;
  }

  // ------------------------------------------------------------ cache (warp)
  __device__ Line* set_of(unsigned long long block) const {
    return lines + (size_t)(block & (cfg.l1_sets - 1)) * cfg.l1_ways;
  }

  // Way holding `block`, or -1 (one lane per way).
  __device__ int find_way(unsigned long long block) const {
    const Line* set = set_of(block);
    const bool m = lane < cfg.l1_ways && (set[lane].flags & kLineValid) && set[lane].block == block;
    const uint32_t b = __ballot_sync(kFull, m);
    return b ? __ffs(b) - 1 : -1;
  }

  // An unused way first, else the least recently used, lowest way on ties.
  __device__ int victim_way(unsigned long long block) const {
    const Line* set = set_of(block);
    const uint32_t inv = __ballot_sync(kFull, lane < cfg.l1_ways && !(set[lane].flags & kLineValid));
    if (inv) return __ffs(inv) - 1;
    const unsigned long long k = lane < cfg.l1_ways ? (((unsigned long long)set[lane].lru << 5) | lane) : ~0ull;
    return (int)(warp_min64(k) & 31u);
  }

  // Lane 0: installs `block` in way `w`, recording evicted prefetched sectors.
  __device__ Line* install(unsigned long long block, int w, uint32_t t) {
    Line* v = set_of(block) + w;
    if (v->flags & kLineValid) {
      for (uint32_t k = 0; k < 4; ++k)
        if ((v->flags >> k) & (v->flags >> (4 + k)) & 1u) {
          SectorEntry* e = sector_entry(v->block * 4 + k, false);
          if (e) e->evicted = ((v->flags >> (8 + k)) & 1u) ? 1u : 2u;
        }
    }
    v->block = block;
    v->flags = kLineValid;
    v->lru = t;
    return v;
  }

  // A demand request; returns the cycle its data is there (uniform).
  __device__ uint32_t demand(unsigned long long addr, uint32_t t) {
    const unsigned long long block = addr >> 7;
    const int way = find_way(block);
    Line* set = set_of(block);
    const uint32_t k = (uint32_t)((addr >> 5) & 3);
    const bool sector_valid = way >= 0 && ((set[way].flags >> k) & 1u);
    const int vic = (way < 0) ? victim_way(block) : -1;
    uint32_t ret = 0;
    if (lane == 0) {
      const unsigned long long sector = addr >> 5;
      S.st.demand_requests++;
      if (sector_valid) {
        Line* l = set + way;
        l->lru = t;
        const bool pf_uncl = (l->flags >> (4 + k)) & (l->flags >> (8 + k)) & 1u;
        if (l->ready[k] <= t) {
          S.st.demand_hits++;
          if (pf_uncl) {
            classify(sector, RT_PF_TIMELY);
            l->flags &= ~(1u << (8 + k));
          }
          ret = t + cfg.hit_latency;
        } else {
          S.st.demand_hit_reserved++;
          if (pf_uncl) {
            classify(sector, RT_PF_LATE);
            l->flags &= ~(1u << (8 + k));
          }
          ret = l->ready[k];
        }
      } else {
        S.st.demand_misses++;
        SectorEntry* e = sector_entry(sector, false);
        if (e && e->evicted == 1u) {
          e->n_unclassified--;
          e->count[RT_PF_TOO_EARLY]++;
          e->evicted = 2u;
        }
        Line* l = way >= 0 ? set + way : install(block, vic, t);
        l->lru = t;
        l->flags = (l->flags | (1u << k)) & ~((1u << (4 + k)) | (1u << (8 + k)));
        l->ready[k] = t + cfg.miss_latency;
        ret = t + cfg.miss_latency;
      }
    }
    __syncwarp();
    return __shfl_sync(kFull, ret, 0);
  }

  __device__ bool is_metadata(unsigned long long base) const {
    return cfg.load_metadata && base >= a.meta_base && base <= a.meta_base + (unsigned long long)a.n_treelets * a.meta_size;
  }

  __device__ void prefetch(unsigned long long addr, unsigned long long base, uint32_t t) {
    const unsigned long long block = addr >> 7;
    const int way = find_way(block);
    Line* set = set_of(block);
    const uint32_t k = (uint32_t)((addr >> 5) & 3);
    const bool sector_valid = way >= 0 && ((set[way].flags >> k) & 1u);
    const int vic = (way < 0) ? victim_way(block) : -1;
    if (lane == 0) {
      S.st.prefetch_issued++;
      SectorEntry* e = sector_entry(addr >> 5, true);
      if (e) e->n_unclassified++;
      if (sector_valid) {
        Line* l = set + way;
        l->lru = t;
        // a fresh record is unclassified, so the TOO_LATE rule of
        // gpu-cache.cc:2101-2116 never applies to it
        if (l->ready[k] <= t) S.st.prefetch_present++;
        else S.st.prefetch_merged++;
      } else {
        S.st.prefetch_filled++;
        Line* l = way >= 0 ? set + way : install(block, vic, t);
        l->lru = t;
        l->flags |= (1u << k) | (1u << (4 + k)) | (1u << (8 + k));
        l->ready[k] = t + cfg.miss_latency;
        if (is_metadata(base)) {
          if (S.mr_tail - S.mr_head < kMetaRing) {
            metaret[S.mr_tail % kMetaRing] = MetaReturn{t + cfg.miss_latency, 0u, base};
            ++S.mr_tail;
          } else {
            S.full = 1;
          }
        }
      }
    }
    __syncwarp();
  }

  // ------------------------------------------------------------ prefetch queue
  __device__ void pq_push(unsigned long long addr, unsigned long long base) {  // lane 0
    S.st.prefetch_queued++;
    if (S.pq_tail - S.pq_head >= a.pq_cap) {  // ring full (live + erased entries)
      S.full = 1;
      return;
    }
    const uint32_t i = S.pq_tail % a.pq_cap;
    pq[2 * i] = addr;
    pq[2 * i + 1] = base;
    dead[i] = 0;
    ++S.pq_tail;
    ++S.pq_live;
    QueuedEntry* q = queued_entry(addr, true);
    if (q) q->count++;
  }

  __device__ void pq_drop_dead() {  // lane 0
    while (S.pq_head != S.pq_tail && dead[S.pq_head % a.pq_cap]) ++S.pq_head;
  }

  // Erases queued prefetches of `addr`, stepping past the entry that follows
  // each erased one (shader.cc:4657-4668 as written).  Lanes read 32 queue
  // entries at a time; lane 0 walks their live ones in order.
  __device__ void remove_queued(unsigned long long addr) {
    uint32_t scan = 0;
    QueuedEntry* q = nullptr;
    if (lane == 0) {
      q = queued_entry(addr, false);
      scan = (q && q->count) ? 1u : 0u;
    }
    scan = __shfl_sync(kFull, scan, 0);
    if (!scan) return;
    const uint32_t head = S.pq_head, tail = S.pq_tail;
    bool skip = false;
    for (uint32_t p0 = head; p0 != tail; p0 += (tail - p0 < 32u ? tail - p0 : 32u)) {
      const uint32_t p = p0 + lane;
      const bool in = p - head < tail - head;
      const uint32_t i = p % a.pq_cap;
      const bool live = in && !dead[i];
      const bool match = live && pq[2 * i] == addr;
      const uint32_t lm = __ballot_sync(kFull, live), mm = __ballot_sync(kFull, match);
      __syncwarp();
      if (lane == 0) {
        for (uint32_t m = lm; m; m &= m - 1) {
          const uint32_t b = __ffs(m) - 1;
          if (skip) {
            skip = false;
            continue;
          }
          if ((mm >> b) & 1u) {
            dead[(p0 + b) % a.pq_cap] = 1;
            --S.pq_live;
            q->count--;
            S.st.prefetch_removed++;
            skip = true;
          }
        }
      }
      __syncwarp();
    }
    if (lane == 0) pq_drop_dead();
    __syncwarp();
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

  __device__ void push_member(unsigned long long j, bool with_metadata) {  // lane 0
    const uint32_t m = __ldg(a.members + j);
    if (with_metadata && cfg.load_metadata) {
      const uint32_t d = dense_of(m);  // treelet_addr_to_metadata_idx: 0 for a member that is no root
      const unsigned long long ma = a.meta_base + (unsigned long long)(d == kNone ? 0u : d) * a.meta_size;
      for (unsigned long long i = 0; i < a.meta_size / 32; ++i) {
        pq_push(ma + i * 32, ma);
        S.st.metadata_queued++;
      }
    }
    const unsigned long long addr = (unsigned long long)m * 64;
    const uint32_t b = __ldg(a.member_bytes + j);
    for (uint32_t i = 0; i < (b + 31) / 32; ++i) pq_push(addr + 32ull * i, addr);
  }

  // ------------------------------------------------------------ decision
  __device__ uint32_t lane_root(const WarpSlot& w, uint32_t l) const {
    const uint32_t r = w.gid * 32 + l;
    const uint32_t unit = __ldg(a.visits + (unsigned long long)r * a.capacity + w.ptr[l]) >> 3;
    return unit < a.n_units ? __ldg(&a.meta[unit].x) : kNone;
  }

  // Run summary of the sorted keys, skipping `skip_key`: (count << 32 | ~key)
  // of the first maximum in ascending key order, and the number of runs.
  __device__ unsigned long long best_run(uint32_t skip_key, uint32_t* runs) const {
    const uint32_t n = S.n_keys;
    unsigned long long best = 0;
    uint32_t nr = 0;
    for (uint32_t i = lane; i < n; i += 32) {
      const uint32_t k = sh.keys[i];
      if (i > 0 && sh.keys[i - 1] == k) continue;
      ++nr;
      if (k == skip_key) continue;
      uint32_t lo = i + 1, hi = n;  // end of the run
      while (lo < hi) {
        const uint32_t mid = (lo + hi) >> 1;
        if (sh.keys[mid] == k) lo = mid + 1;
        else hi = mid;
      }
      const unsigned long long v = ((unsigned long long)(lo - i) << 32) | (unsigned long long)(~k);
      best = v > best ? v : best;
    }
    if (runs) *runs = warp_sum(nr);
    return warp_max64(best);
  }

  __device__ void rebuild_histogram() {
    uint32_t n = 0;
    for (uint32_t o = 0; o < S.n_res; ++o) {
      const WarpSlot& w = sh.warps[S.order[o]];
      const uint32_t k = (w.ptr[lane] < w.end[lane]) ? lane_root(w, lane) : kNone;
      const uint32_t b = __ballot_sync(kFull, k != kNone);
      if (k != kNone) sh.keys[n + __popc(b & lanemask_lt())] = k;
      n += __popc(b);
    }
    uint32_t P = 1;
    while (P < n) P <<= 1;
    for (uint32_t i = n + lane; i < P; i += 32) sh.keys[i] = kNone;
    __syncwarp();
    for (uint32_t size = 2; size <= P; size <<= 1)
      for (uint32_t stride = size >> 1; stride > 0; stride >>= 1) {
        for (uint32_t i = lane; i < P; i += 32) {
          const uint32_t j = i ^ stride;
          if (j > i) {
            const bool up = (i & size) == 0;
            const uint32_t x = sh.keys[i], y = sh.keys[j];
            if ((x > y) == up) {
              sh.keys[i] = y;
              sh.keys[j] = x;
            }
          }
        }
        __syncwarp();
      }
    if (lane == 0) S.n_keys = n;
    __syncwarp();
    uint32_t runs = 0;
    const unsigned long long b = best_run(kNone, &runs);
    unsigned long long b2 = 0;
    if (cfg.decision.second_prefetch && n) b2 = best_run(~(uint32_t)(b & 0xffffffffu), nullptr);
    if (lane == 0) {
      S.second = b2 ? ~(uint32_t)(b2 & 0xffffffffu) : kNone;
      S.total = n;
      S.distinct = runs;
      S.best = n ? ~(uint32_t)(b & 0xffffffffu) : kNone;
      S.best_cnt = (uint32_t)(b >> 32);
      S.best_dense = S.best == kNone ? kNone : dense_of(S.best);
      S.best_nodes = S.best_dense == kNone
                         ? 0u
                         : (uint32_t)(__ldg(a.member_first + S.best_dense + 1) - __ldg(a.member_first + S.best_dense));
      S.hist_dirty = 0;
    }
    __syncwarp();
  }

  // The RT unit's decision (shader.cc:3419-3683; as prefetch_decide_kernel).
  __device__ void decide() {
    if (S.hist_dirty) rebuild_histogram();
    const rt_prefetch_params& p = cfg.decision;
    if (lane == 0) {
      S.st.decisions++;
      const uint32_t best = S.best;
      bool submit = false;
      int num_nodes = 0;
      const int n_nodes = (int)S.best_nodes;
      const uint32_t bd = S.best_dense;
      if (p.heuristic == RT_PREFETCH_ALWAYS) {
        submit = true;
      } else if (best != kNone) {
        const double pct = (double)S.best_cnt / (double)S.total;
        if (p.heuristic == RT_PREFETCH_POPULARITY) {
          if (pct >= p.threshold) {
            S.ds.last_rejected = kNone;
            submit = true;
          } else if (S.ds.last_rejected != best) {
            S.ds.last_rejected = best;
          }
        } else {
          num_nodes = (int)(((double)n_nodes * pct) + 0.5);
          submit = true;
        }
      }
      unsigned long long queue = S.pq_live;
      if (submit && best != kNone && bd != kNone && S.ds.last_prefetched != best && S.ds.last_prefetched_second != best) {
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
          S.ds.last_prefetched = best;
          S.st.treelets_prefetched++;
        }
      }
      if (p.second_prefetch && queue == 0 && S.total > 0 && S.distinct > 1 && S.ds.last_prefetched == best &&
          best != kNone) {
        // the first maximum among treelets other than the last prefetched one,
        // which is `best` here (kept with the histogram)
        const uint32_t second = S.second;
        if (second != kNone && S.ds.last_prefetched_second != second) {
          const uint32_t sd = dense_of(second);
          if (sd != kNone)
            for (unsigned long long j = __ldg(a.member_first + sd); j < __ldg(a.member_first + sd + 1); ++j)
              push_member(j, false);
          S.ds.last_prefetched_second = second;
          S.st.treelets_prefetched++;
        }
      }
    }
    __syncwarp();
  }

  // ------------------------------------------------------------ stride (Lee MICRO'10), lane 0
  __device__ void stride_prefetch(uint32_t wid, unsigned long long next_addr) {
    StrideTable& s = sh.stride[wid];
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
    if (cfg.decision.max_queue <= S.pq_live) {
      pq_push(pa, pa);
      pq_push(pa + 32, pa);
    }
  }

  // ------------------------------------------------------------ warps
  __device__ uint32_t matching_lanes(uint32_t slot) const {
    const WarpSlot& w = sh.warps[slot];
    const uint32_t lp = S.ds.last_prefetched;
    const bool m = lp != kNone && w.ptr[lane] < w.end[lane] && lane_root(w, lane) == lp;
    return __popc(__ballot_sync(kFull, m));
  }

  // rt_unit::schedule_next_warp (shader.cc:4307-4392); kNone if no warp is ready
  __device__ uint32_t schedule() const {
    const uint32_t n_res = S.n_res;
    const bool rd = lane < n_res && !sh.warps[S.order[lane]].in_flight && sh.warps[S.order[lane]].live;
    const uint32_t ready = __ballot_sync(kFull, rd);
    if (!ready) return kNone;
    const bool treelet = cfg.prefetcher == RT_UNIT_PF_TREELET;
    if (treelet && cfg.scheduler == RT_UNIT_SCHED_OMR) {
      for (uint32_t m = ready; m; m &= m - 1) {
        const uint32_t o = __ffs(m) - 1;
        if (matching_lanes(S.order[o]) > 0) return S.order[o];
      }
    } else if (treelet && cfg.scheduler == RT_UNIT_SCHED_PMR) {
      uint32_t b = kNone, bc = 0;
      for (uint32_t m = ready; m; m &= m - 1) {
        const uint32_t o = __ffs(m) - 1;
        const uint32_t c = matching_lanes(S.order[o]);
        if (c > bc) {
          b = S.order[o];
          bc = c;
        }
      }
      if (b != kNone) return b;
    }
    return S.order[__ffs(ready) - 1];
  }

  // A round: each lane's next transaction, identical (address, size) pairs
  // once in lane order, split into 32-byte requests.
  __device__ void start_round(uint32_t slot) {
    WarpSlot& w = sh.warps[slot];
    const bool has = w.ptr[lane] < w.end[lane];
    const uint32_t v = has ? __ldg(a.visits + (unsigned long long)(w.gid * 32 + lane) * a.capacity + w.ptr[lane]) : 0u;
    const uint32_t size = tx_size(v & 7);
    const unsigned long long key = has ? (((unsigned long long)(v >> 3) << 8) | size) : ~0ull;
    const uint32_t peers = __match_any_sync(kFull, key);
    const bool leader = has && (uint32_t)(__ffs(peers) - 1) == lane;
    const uint32_t nch = leader ? (size + 31) / 32 : 0u;
    uint32_t incl = nch;
#pragma unroll
    for (int s = 1; s < 32; s <<= 1) {
      const uint32_t o = __shfl_up_sync(kFull, incl, s);
      if ((int)lane >= s) incl += o;
    }
    const uint32_t total = __shfl_sync(kFull, incl, 31);
    const unsigned long long addr = (unsigned long long)(v >> 3) * 64;
    for (uint32_t i = 0; i < nch; ++i) sh.chunk[incl - nch + i] = Request{addr + 32ull * i, addr, i == 0 ? 1u : 0u, 0u};
    uint32_t il = has ? intersection_latency(v & 7) : 0u;
    il = __reduce_max_sync(kFull, il);
    const uint32_t issued = __ballot_sync(kFull, has);
    __syncwarp();
    if (lane == 0) {
      w.issued = issued;
      w.in_flight = 1;
      w.all_sent = 0;
      w.ready = 0;
      w.ilat = il;
      S.ch_head = 0;
      S.ch_tail = total;
      S.serving = slot;
    }
    __syncwarp();
  }

  __device__ void send_demand(uint32_t t) {
    const Request r = sh.chunk[S.ch_head];
    if (cfg.prefetcher == RT_UNIT_PF_TREELET || cfg.prefetcher == RT_UNIT_PF_STRIDE) remove_queued(r.addr);
    WarpSlot& w = sh.warps[S.serving];
    if (lane == 0 && cfg.prefetcher == RT_UNIT_PF_STRIDE && r.first) stride_prefetch(w.wid, r.addr);
    __syncwarp();
    const uint32_t ret = demand(r.addr, t);
    if (lane == 0) {
      ++S.ch_head;
      w.ready = max(w.ready, ret);
      if (S.ch_head == S.ch_tail) {
        w.all_sent = 1;
        w.ready += w.ilat;
        S.serving = kNone;
      }
    }
    __syncwarp();
  }

  __device__ bool prefetch_issuable() const {  // lane 0
    const unsigned long long base = pq[2 * (S.pq_head % a.pq_cap) + 1];
    if (!cfg.wait_metadata || is_metadata(base)) return true;
    // shader.cc:4469-4476: the metadata of the treelet the request's base node belongs to
    const unsigned long long unit = base >> 6;
    const uint32_t root = (base % 64 == 0 && unit < a.n_units) ? __ldg(&a.meta[unit].x) : kNone;
    const uint32_t d = root == kNone ? kNone : dense_of(root);
    return S.most_recent_metadata == a.meta_base + (unsigned long long)(d == kNone ? 0u : d) * a.meta_size;
  }

  // Rounds whose data is back advance their lanes; warps with no lanes left
  // leave; new warps come in, in order.
  __device__ void retire_and_admit(uint32_t t, uint32_t n_warps) {
    const uint32_t n_res = S.n_res;
    const WarpSlot* wl = lane < n_res ? &sh.warps[S.order[lane]] : nullptr;
    const bool done_round = wl && wl->in_flight && wl->all_sent && wl->ready <= t;
    const uint32_t rounds = __ballot_sync(kFull, done_round);
    for (uint32_t m = rounds; m; m &= m - 1) {
      const uint32_t o = __ffs(m) - 1;
      WarpSlot& w = sh.warps[S.order[o]];
      const uint32_t issued = w.issued;
      if ((issued >> lane) & 1u) w.ptr[lane]++;
      const uint32_t live = __ballot_sync(kFull, w.ptr[lane] < w.end[lane]);
      __syncwarp();
      if (lane == 0) {
        S.st.transactions += __popc(issued);
        w.issued = 0;
        w.in_flight = 0;
        w.live = live;
        S.hist_dirty = 1;
      }
      __syncwarp();
    }
    const bool gone = lane < n_res && !sh.warps[S.order[lane]].in_flight && sh.warps[S.order[lane]].live == 0;
    const uint32_t leave = __ballot_sync(kFull, gone);
    if (leave) {
      const uint32_t slot = lane < n_res ? S.order[lane] : 0u;
      const uint32_t keep = __ballot_sync(kFull, lane < n_res && !gone);
      __syncwarp();
      if (lane < n_res && !gone) S.order[__popc(keep & lanemask_lt())] = slot;
      __syncwarp();
      if (lane == 0) {
        S.st.warps += __popc(leave);
        S.n_res = __popc(keep);
        S.hist_dirty = 1;
      }
      if (gone) atomicOr(&S.free_mask, 1u << slot);
      __syncwarp();
    }
    while (S.n_res < cfg.max_warps && S.next_gid < n_warps) {
      const uint32_t slot = __ffs(S.free_mask) - 1;
      WarpSlot& w = sh.warps[slot];
      const uint32_t gid = S.next_gid;
      const uint32_t r = gid * 32 + lane;
      w.ptr[lane] = 0;
      w.end[lane] = r < a.n ? min(a.hits[r].n_visits, a.capacity) : 0u;
      const uint32_t live = __ballot_sync(kFull, w.end[lane] != 0);
      __syncwarp();
      if (lane == 0) {
        w.gid = gid;
        w.wid = S.local++ % cfg.max_warps;
        w.in_flight = w.all_sent = 0;
        w.ready = w.ilat = w.issued = 0;
        w.live = live;
        S.free_mask &= ~(1u << slot);
        S.order[S.n_res++] = slot;
        S.next_gid = gid + cfg.n_rt_units;
        S.hist_dirty = 1;
      }
      __syncwarp();
    }
  }

  __device__ void run(uint32_t u) {
    const uint32_t n_warps = (a.n + 31) / 32;
    if (lane == 0) {
      S.st = rt_unit_stats{};
      S.most_recent_metadata = 0;
      S.ds = rt_prefetch_state{kNone, kNone, kNone, 0};
      S.pq_head = S.pq_tail = S.pq_live = 0;
      S.ch_head = S.ch_tail = 0;
      S.serving = kNone;
      S.n_res = 0;
      S.free_mask = (1u << cfg.max_warps) - 1u;
      S.mr_head = S.mr_tail = 0;
      S.n_keys = 0;
      S.best = kNone;
      S.best_cnt = S.total = S.distinct = S.best_nodes = 0;
      S.best_dense = S.second = kNone;
      S.hist_dirty = 1;
      S.full = 0;
      S.next_gid = u;
      S.local = 0;
    }
    if (lane < kMaxResident) sh.stride[lane].has = sh.stride[lane].n = 0;
    if (a.lines_shared)
      for (uint32_t i = lane; i < cfg.l1_sets * cfg.l1_ways; i += 32) lines[i].flags = 0;
    __syncwarp();
    const uint32_t tcap = a.cycle_cap;
    for (uint32_t t = 0;; ++t) {
      retire_and_admit(t, n_warps);
      if (S.n_res == 0) {
        if (lane == 0) S.st.cycles = t;
        break;
      }
      if (t >= tcap) {
        if (lane == 0) {
          S.st.cycles = t;
          S.st.status |= 2;
        }
        break;
      }
      if (lane == 0)
        while (S.mr_head != S.mr_tail && metaret[S.mr_head % kMetaRing].t <= t) {
          S.most_recent_metadata = metaret[S.mr_head % kMetaRing].base;
          ++S.mr_head;
        }
      __syncwarp();
      if (cfg.prefetcher == RT_UNIT_PF_TREELET && t % cfg.prefetch_delay == 0) decide();
      if (S.ch_head != S.ch_tail) {
        send_demand(t);
        continue;
      }
      const uint32_t s = schedule();
      if (s != kNone) {
        start_round(s);
        send_demand(t);
        continue;
      }
      if (cfg.prefetcher != RT_UNIT_PF_NONE && S.pq_live > 0) {
        uint32_t go = 0;
        unsigned long long addr = 0, base = 0;
        if (lane == 0 && prefetch_issuable()) {
          const uint32_t i = S.pq_head % a.pq_cap;
          addr = pq[2 * i];
          base = pq[2 * i + 1];
          dead[i] = 1;
          --S.pq_live;
          QueuedEntry* q = queued_entry(addr, false);
          if (q) q->count--;
          pq_drop_dead();
          go = 1;
        }
        __syncwarp();
        go = __shfl_sync(kFull, go, 0);
        if (go) {
          addr = __shfl_sync(kFull, addr, 0);
          base = __shfl_sync(kFull, base, 0);
          prefetch(addr, base, t);
        }
      }
    }
    __syncwarp();
    // final tally (gpu-sim.cc:1749-1790): lanes take sector-map slices
    const uint32_t n_sec = 1u << a.sec_log2;
    unsigned long long eff[5] = {0, 0, 0, 0, 0}, uba = 0;
    for (uint32_t i = lane; i < n_sec; i += 32) {
      const SectorEntry& e = sec[i];
      if (!e.key) continue;
      const uint32_t classified = e.count[0] + e.count[1] + e.count[2] + e.count[3];
      if (classified) {
        uba += e.n_unclassified;
        for (uint32_t c = 0; c < 4; ++c) eff[c] += e.count[c];
      } else {
        eff[RT_PF_NEVER_USED] += e.n_unclassified;
      }
    }
#pragma unroll
    for (int s = 16; s > 0; s >>= 1) {
      uba += __shfl_xor_sync(kFull, uba, s);
      for (int c = 0; c < 5; ++c) eff[c] += __shfl_xor_sync(kFull, eff[c], s);
    }
    if (lane == 0) {
      for (int c = 0; c < 5; ++c) S.st.effectiveness[c] = eff[c];
      S.st.unclassified_but_accessed = uba;
      if (S.full) S.st.status |= 1;
    }
    __syncwarp();
  }
};

__global__ void __launch_bounds__(32) unit_replay_kernel(ReplayArgs a) {
  extern __shared__ __align__(16) uint8_t replay_smem[];
  UnitShared& sh = *reinterpret_cast<UnitShared*>(replay_smem);
  Line* smem_lines = reinterpret_cast<Line*>(replay_smem + ((sizeof(UnitShared) + 15) & ~(size_t)15));
  const uint32_t u = blockIdx.x;
  WUnit unit(a, u, sh, smem_lines);
  unit.run(u);
  if ((threadIdx.x & 31u) == 0) a.stats[u] = sh.s.st;
}

}  // namespace rtr
