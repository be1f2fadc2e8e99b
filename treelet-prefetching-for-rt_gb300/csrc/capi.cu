// C ABI: contexts, device scenes, treelets, tracing, bounce rays and the
// prefetch decision.  Every entry point returns an rt_status and records a
// message for rt_last_error(); none aborts.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "capi_internal.h"
#include "trace_kernels.cuh"
#include "prefetch_kernels.cuh"
#include "replay_kernel.cuh"
#include "trace_queued.cuh"
#include "trace_treelet.cuh"
#include "treelets.h"

namespace rti {

namespace {
thread_local std::string g_error;
}

void set_error(const std::string& msg) { g_error = msg; }
rt_status fail(rt_status s, const std::string& msg) {
  g_error = msg;
  return s;
}

bool validate_blob(const uint8_t* b, uint64_t n, std::string* err) {
  auto bad = [&](const std::string& m) {
    if (err) *err = m;
    return false;
  };
  if (!b || n < 128 || n % 64) return bad("blob must be at least 128 bytes and a multiple of 64");
  const uint64_t units = n / 64;
  if (units >= (1ull << 29)) return bad("blob larger than 32 GiB");
  auto rd64 = [&](uint64_t off) {
    uint64_t v;
    std::memcpy(&v, b + off, 8);
    return v;
  };
  std::vector<uint8_t> seen(units, 0);
  struct Item {
    uint64_t unit;
    bool top;
  };
  std::vector<Item> work;
  const uint64_t root = rd64(rtf::HDR_ROOT_OFFSET);
  if (root % 64 || root / 64 >= units || root == 0) return bad("TLAS RootNodeOffset out of range");
  work.push_back({root / 64, true});
  while (!work.empty()) {
    const Item it = work.back();
    work.pop_back();
    if (seen[it.unit]) continue;
    seen[it.unit] = 1;
    const uint8_t* p = b + it.unit * 64;
    int32_t child_off;
    std::memcpy(&child_off, p + rtf::IN_CHILD_OFFSET, 4);
    bool any = false;
    for (int i = 0; i < 6; ++i) any |= (p[rtf::IN_CHILD_INFO + i] & 3u) != 0;
    if (!any) continue;
    if (child_off <= 0) return bad("internal node with a child block that does not follow it");
    uint64_t c = it.unit + (uint64_t)child_off;
    for (int i = 0; i < 6; ++i) {
      const uint8_t info = p[rtf::IN_CHILD_INFO + i];
      const uint32_t sz = rtf::child_size_units(info), ty = rtf::child_type(info);
      if (sz) {
        if (c + sz > units) return bad("child outside the blob");
        if (ty == rtf::CT_INTERNAL) {
          work.push_back({c, it.top});
        } else if (it.top) {
          if (ty != rtf::CT_INSTANCE || sz != 2) return bad("top-level leaf that is not a 128-byte instance leaf");
          if (!seen[c]) {
            seen[c] = 1;
            const uint64_t hdr = c * 64 + rd64(c * 64 + rtf::IL_BVH_ADDRESS);
            if (hdr % 64 || hdr / 64 >= units) return bad("instance BVHAddress out of range");
            const uint64_t broot = hdr + rd64(hdr + rtf::HDR_ROOT_OFFSET);
            if (broot % 64 || broot / 64 >= units || broot <= hdr) return bad("BLAS RootNodeOffset out of range");
            work.push_back({broot / 64, false});
          }
        } else {
          if (ty != rtf::CT_QUAD && ty != rtf::CT_PROCEDURAL) return bad("bottom-level leaf of unknown type");
        }
      }
      c += sz;
    }
  }
  return true;
}

// Device memory of the treelet queues (trace_queued.cuh), kept by a scene
// from its first queued launch on and grown as launches need.
struct QueueScratch {
  uint8_t* base = nullptr;
  size_t bytes = 0;
  uint4* state = nullptr;              // 64 B per ray
  unsigned long long* slab = nullptr;  // stack_depth entries per ray
  uint32_t *in_ray = nullptr, *in_key = nullptr, *out_ray = nullptr, *out_key = nullptr;
  uint32_t *hist = nullptr, *offset = nullptr, *block_sum = nullptr;
  uint32_t* ctr = nullptr;  // per round: hand-out counter, rays left
};

}  // namespace rti

struct rt_scene {
  rt_ctx* ctx = nullptr;
  std::vector<uint8_t> host_blob;
  uint8_t* d_blob = nullptr;
  uint64_t blob_bytes = 0;
  uint32_t n_units = 0;
  // treelets
  bool has_treelets = false;
  rtt::Partition part;
  uint2* d_meta = nullptr;
  uint8_t* d_images = nullptr;
  unsigned long long* d_image_off = nullptr;
  uint32_t* d_roots = nullptr;
  unsigned long long* d_member_first = nullptr;
  uint16_t* d_member_bytes = nullptr;
  uint32_t* d_members = nullptr;
  uint32_t* d_hint = nullptr;  // staged-mode predictions (8 per treelet) or null
  uint32_t slot_bytes = 0;
  std::vector<uint16_t> route;  // routing bits of the treelet-ordered walk
  bool offset_quirk = false;    // walk as the reference does with a nonzero device_offset
  uint16_t* d_route = nullptr;
  // pinned treelets of the staged walk (built when treelets, order or budget change)
  std::vector<uint32_t> pin_order;  // explicit order, empty = default
  std::vector<uint32_t> pin_default;
  uint8_t* d_pin = nullptr;
  rt_pinned_info pin_info{0, 0, 0, 0};
  uint32_t pin_root = 0;
  uint32_t pin_want = 0;  // the pinned_bytes the current image was built for
  // Images built for other pinned_bytes values under the current partition,
  // route bits and pin order, so that switching the tuning back and forth
  // (e.g. per ray batch) does not rebuild and re-upload them.
  struct PinImage {
    uint32_t want;
    uint8_t* d;
    rt_pinned_info info;
    uint32_t root;
  };
  std::vector<PinImage> pin_cache;
  // per-launch counters and status (library scratch)
  unsigned long long* d_stats = nullptr;
  uint32_t* d_status = nullptr;
  uint32_t* d_queue = nullptr;  // ray hand-out counter of the persistent kernels
  rt_tuning tuning{128, 256, 16, RT_TUNING_OFF, 8, 2048, 8, 96, 4096, rtk::kWaitTries, RT_TUNING_OFF, RT_TUNING_OFF};
  // host-buffer path: a copy-in stream, two trace streams (chunk c on
  // stream / stream2 by parity, so one chunk's launch fills the SMs that the
  // previous chunk's last rays leave idle), a copy-out stream, and events
  cudaStream_t stream = nullptr, stream2 = nullptr, xin = nullptr, xout = nullptr;
  cudaEvent_t ev_in[rti::kHostChunks] = {}, ev_done[rti::kHostChunks] = {};
  void* d_io = nullptr;
  size_t io_bytes = 0;
  void* d_pack = nullptr;  // packed access traces of rt_trace_host_packed
  size_t pack_bytes = 0;
  unsigned long long* h_tot = nullptr;  // page-locked chunk totals of rt_trace_host_packed
  rti::QueueScratch qs;  // treelet queues of RT_MODE_STAGED with queue_rounds
};

namespace {

rt_status cuda_fail(cudaError_t e, const char* what) {
  return rti::fail(RT_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

#define RT_CUDA(call)                                    \
  do {                                                   \
    cudaError_t e_ = (call);                             \
    if (e_ != cudaSuccess) return cuda_fail(e_, #call);  \
  } while (0)

template <class T>
rt_status dalloc(T** p, size_t bytes) {
  *p = nullptr;
  if (bytes == 0) bytes = 16;
  cudaError_t e = cudaMalloc((void**)p, bytes);
  if (e != cudaSuccess) return rti::fail(RT_ERR_OOM, std::string("cudaMalloc: ") + cudaGetErrorString(e));
  return RT_OK;
}

void free_treelets(rt_scene* s) {
  cudaFree(s->d_meta);
  cudaFree(s->d_images);
  cudaFree(s->d_image_off);
  cudaFree(s->d_roots);
  cudaFree(s->d_member_first);
  cudaFree(s->d_member_bytes);
  cudaFree(s->d_members);
  s->d_members = nullptr;
  cudaFree(s->d_hint);
  cudaFree(s->d_route);
  cudaFree(s->d_pin);
  for (auto& im : s->pin_cache) cudaFree(im.d);
  s->pin_cache.clear();
  s->d_route = nullptr;
  s->d_pin = nullptr;
  s->pin_info = rt_pinned_info{0, 0, 0, 0};
  s->pin_root = 0;
  s->pin_want = 0;
  s->route.clear();
  s->pin_default.clear();
  s->pin_order.clear();
  s->d_hint = nullptr;
  s->d_meta = nullptr;
  s->d_images = nullptr;
  s->d_image_off = nullptr;
  s->d_roots = nullptr;
  s->d_member_first = nullptr;
  s->d_member_bytes = nullptr;
  s->has_treelets = false;
}

// Blocks for a persistent launch: as many as fit on the device at once (no
// more than the rays need).
uint32_t persistent_grid(const void* kern, uint32_t threads, uint32_t n, size_t dyn_smem = 0) {
  // occupancy per (device, kernel, block, shared memory), computed once
  struct Key {
    int dev;
    const void* kern;
    uint32_t threads;
    size_t smem;
    bool operator==(const Key& o) const {
      return dev == o.dev && kern == o.kern && threads == o.threads && smem == o.smem;
    }
  };
  static std::mutex mu;
  static std::vector<std::pair<Key, uint64_t>> cache;
  int dev = 0;
  cudaGetDevice(&dev);
  const Key key{dev, kern, threads, dyn_smem};
  uint64_t full = 0;
  {
    std::lock_guard<std::mutex> lock(mu);
    for (const auto& kv : cache)
      if (kv.first == key) full = kv.second;
  }
  if (!full) {
    int sms = 0, per_sm = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, (int)threads, dyn_smem);
    full = (uint64_t)std::max(1, sms) * (uint64_t)std::max(1, per_sm);
    std::lock_guard<std::mutex> lock(mu);
    cache.emplace_back(key, full);
  }
  const uint64_t need = ((uint64_t)n + threads - 1) / threads;
  return (uint32_t)std::max<uint64_t>(1, std::min(full, need));
}

// Raises a kernel's dynamic shared-memory limit to at least `bytes`, once
// per (device, kernel, limit): a launch whose tuning switches between
// budgets (pinned images of different sizes per ray batch) then makes no
// attribute call at all once the largest has been set.
cudaError_t ensure_dyn_smem(const void* kern, size_t bytes) {
  static std::mutex mu;
  static std::vector<std::pair<std::pair<int, const void*>, size_t>> set;
  int dev = 0;
  cudaGetDevice(&dev);
  std::lock_guard<std::mutex> lock(mu);
  for (auto& kv : set) {
    if (kv.first.first != dev || kv.first.second != kern) continue;
    if (kv.second >= bytes) return cudaSuccess;
    const cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
    if (e == cudaSuccess) kv.second = bytes;
    return e;
  }
  const cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
  if (e == cudaSuccess) set.push_back({{dev, kern}, bytes});
  return e;
}

int max_smem_per_block() {
  int dev = 0, v = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&v, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  return v;
}

// Dynamic shared memory a staged CTA can use next to its static state.
uint32_t staged_smem_limit() {
  const int v = max_smem_per_block() - (int)(sizeof(rtk::WarpStage) * (rtk::kStagedMaxThreads / 32)) - 1024;
  return v > 0 ? (uint32_t)v : 0u;
}

rt_status rebuild_pinned(rt_scene* s, bool keep_current = false);

// Frees the images kept for other pinned_bytes values (their partition,
// route bits or order changed).
void drop_pin_cache(rt_scene* s) {
  for (auto& im : s->pin_cache) cudaFree(im.d);
  s->pin_cache.clear();
}

// Computes the route bits of the walk (treelets.h) into s->route, uploads
// them and rebuilds the pinned image that embeds them.  With a nonzero
// device_offset the reference's comparisons stop matching at the first pop
// from the other-treelet stack (vulkan_ray_tracing.cc:1752); the current
// stack is empty then and nothing is pushed to it again, so every later node
// is popped from the other stack.  Clearing the bits a node popped from the
// other stack reads (6-11 and 13) therefore gives that walk, while a node
// popped from the current stack, which happens only before the first such
// pop, keeps its comparisons.
rt_status upload_route(rt_scene* s) {
  rtt::route_masks(s->host_blob.data(), s->blob_bytes, s->part, s->route);
  if (s->offset_quirk)
    for (uint16_t& r : s->route) r &= (uint16_t)~((0x3Fu << rtt::kRouteOtherShift) | (2u << rtt::kRouteInstShift));
  RT_CUDA(cudaMemcpy(s->d_route, s->route.data(), sizeof(uint16_t) * s->route.size(), cudaMemcpyHostToDevice));
  drop_pin_cache(s);
  return rebuild_pinned(s);
}

// Rebuilds the pinned image for the scene's order and budget (the budget is
// clamped to what a CTA can hold).  keep_current (a tuning change) keeps the
// image being replaced for a later switch back, and takes a kept image for
// the new budget instead of building it again.
rt_status rebuild_pinned(rt_scene* s, bool keep_current) {
  constexpr size_t kPinCache = 4;
  if (keep_current && s->d_pin) {
    if (s->pin_cache.size() == kPinCache) {
      cudaFree(s->pin_cache.front().d);
      s->pin_cache.erase(s->pin_cache.begin());
    }
    s->pin_cache.push_back({s->pin_want, s->d_pin, s->pin_info, s->pin_root});
  } else {
    cudaFree(s->d_pin);
  }
  s->d_pin = nullptr;
  s->pin_info = rt_pinned_info{0, 0, 0, 0};
  s->pin_root = 0;
  s->pin_want = 0;
  const uint32_t want = s->tuning.pinned_bytes;
  if (!s->has_treelets || want == RT_TUNING_OFF || want == 0) return RT_OK;
  for (size_t i = 0; i < s->pin_cache.size(); ++i) {
    if (s->pin_cache[i].want != want) continue;
    s->d_pin = s->pin_cache[i].d;
    s->pin_info = s->pin_cache[i].info;
    s->pin_root = s->pin_cache[i].root;
    s->pin_want = want;
    s->pin_cache.erase(s->pin_cache.begin() + (ptrdiff_t)i);
    return RT_OK;
  }
  const uint32_t budget = std::min(want, staged_smem_limit() > 128 ? staged_smem_limit() - 128 : 0u);
  if (s->pin_default.empty() && s->pin_order.empty())
    rtt::default_pin_order(s->host_blob.data(), s->blob_bytes, s->pin_default, s->part);
  rtt::Pinned pin;
  rtt::build_pinned(s->host_blob.data(), s->blob_bytes, s->part, s->route,
                    s->pin_order.empty() ? s->pin_default : s->pin_order, budget, pin);
  if (pin.bytes.empty()) return RT_OK;
  rt_status st = dalloc(&s->d_pin, pin.bytes.size());
  if (st != RT_OK) return st;
  RT_CUDA(cudaMemcpy(s->d_pin, pin.bytes.data(), pin.bytes.size(), cudaMemcpyHostToDevice));
  s->pin_info = rt_pinned_info{(uint32_t)pin.bytes.size(), pin.n_treelets, pin.n_records, pin.root_soff ? 1u : 0u};
  s->pin_root = pin.root_soff;
  s->pin_want = want;
  return RT_OK;
}

// Merges the nonzero fields of `t` into `cur` after checking them.
rt_status merge_tuning(const rt_tuning& cur, const rt_tuning* t, rt_tuning& n) {
  n = cur;
  auto ok_threads = [](uint32_t v, uint32_t hi) { return v >= 32 && v <= hi && v % 32 == 0; };
  if (t->block_threads) {
    if (!ok_threads(t->block_threads, 256))
      return rti::fail(RT_ERR_INVALID, "block_threads must be 32..256, multiple of 32");
    n.block_threads = t->block_threads;
  }
  if (t->staged_threads) {
    if (!ok_threads(t->staged_threads, rtk::kStagedMaxThreads))
      return rti::fail(RT_ERR_INVALID, "staged_threads must be 32.." + std::to_string(rtk::kStagedMaxThreads) +
                                           ", multiple of 32");
    n.staged_threads = t->staged_threads;
  }
  if (t->staged_epoch) n.staged_epoch = t->staged_epoch;
  if (t->refill_lanes) {
    if (t->refill_lanes > 32) return rti::fail(RT_ERR_INVALID, "refill_lanes must be 1..32");
    n.refill_lanes = t->refill_lanes;
  }
  if (t->staged_slots) {
    if (t->staged_slots != RT_TUNING_OFF && t->staged_slots > (uint32_t)rtk::kMaxSlots)
      return rti::fail(RT_ERR_INVALID, "staged_slots must be 1..8 or RT_TUNING_OFF");
    n.staged_slots = t->staged_slots;
  }
  if (t->staged_slot_bytes) {
    if (t->staged_slot_bytes < 64 || t->staged_slot_bytes > 65536)
      return rti::fail(RT_ERR_INVALID, "staged_slot_bytes must be 64..65536");
    n.staged_slot_bytes = t->staged_slot_bytes;
  }
  if (t->staged_min_votes) {
    if (t->staged_min_votes > 32) return rti::fail(RT_ERR_INVALID, "staged_min_votes must be 1..32");
    n.staged_min_votes = t->staged_min_votes;
  }
  if (t->stack_depth) {
    if (t->stack_depth != 48 && t->stack_depth != 96 && t->stack_depth != 160)
      return rti::fail(RT_ERR_INVALID, "stack_depth must be 48, 96 or 160");
    n.stack_depth = t->stack_depth;
  }
  if (t->pinned_bytes) {
    if (t->pinned_bytes != RT_TUNING_OFF && (t->pinned_bytes < 256 || t->pinned_bytes > 229376))
      return rti::fail(RT_ERR_INVALID, "pinned_bytes must be 256..229376 or RT_TUNING_OFF");
    n.pinned_bytes = t->pinned_bytes;
  }
  if (t->wait_tries) {
    if (t->wait_tries > (1u << 24)) return rti::fail(RT_ERR_INVALID, "wait_tries must be 1..2^24");
    n.wait_tries = t->wait_tries;
  }
  if (t->queue_rounds) {
    if (t->queue_rounds != RT_TUNING_OFF && t->queue_rounds > rti::kMaxQueueRounds)
      return rti::fail(RT_ERR_INVALID, "queue_rounds must be 1..64 or RT_TUNING_OFF");
    n.queue_rounds = t->queue_rounds;
  }
  if (t->short_stack) {
    if (t->short_stack != 1 && t->short_stack != RT_TUNING_OFF)
      return rti::fail(RT_ERR_INVALID, "short_stack must be 1 or RT_TUNING_OFF");
    n.short_stack = t->short_stack;
  }
  return RT_OK;
}

// The treelet-queued staged walk (trace_queued.cuh): round 0 over every ray,
// then per round the counting sort of the rays left by the treelet they need
// next (scan, top-level scan, scatter) and a binned round, then the last
// round without queues.  Every kernel is stream-ordered on `st`; the scratch
// must hold a.n rays, CAP stack entries per ray and n_bins bins.
template <int CAP>
rt_status launch_queued(rtk::TraceArgs& a, const rt_tuning& t, uint32_t largest_image, const rti::QueueScratch& qs,
                        cudaStream_t st) {
  const uint32_t rounds = t.queue_rounds;
  const uint32_t n_bins = a.n_treelets + 1;
  const uint32_t n_blocks = (n_bins + rtk::kBinScanItems - 1) / rtk::kBinScanItems;
  if (n_blocks > rtk::kBinScanItems)
    return rti::fail(RT_ERR_TOO_LARGE, "treelet queues: more than 2^24 treelets");
  a.tbuf_off = rtk::kNone;  // rays move between lanes: trace entries go straight to the rows
  RT_CUDA(cudaMemsetAsync(qs.ctr, 0, sizeof(uint32_t) * 2 * (rti::kMaxQueueRounds + 1), st));
  RT_CUDA(cudaMemsetAsync(qs.hist, 0, sizeof(uint32_t) * n_bins, st));
  const uint32_t bt = rtk::kStagedMaxThreads;
  // a warp's slot holds a whole treelet of the 8 KiB budgets, the first
  // 8 KiB of larger ones (three CTAs of eight warps per SM); the rest of a
  // larger treelet is read from global memory
  const uint32_t slot = std::min((largest_image + 127u) & ~127u, rtk::kQueueSlotMax);
  const size_t dyn = (size_t)(bt / 32) * slot + 128;
  auto kern = rtk::trace_queued_kernel<CAP, false>;
  auto fin = rtk::trace_queued_kernel<CAP, true>;
  RT_CUDA(ensure_dyn_smem((const void*)kern, dyn));
  RT_CUDA(ensure_dyn_smem((const void*)fin, 128));
  const uint32_t grid = persistent_grid((const void*)kern, bt, a.n, dyn);
  const uint32_t grid_fin = persistent_grid((const void*)fin, bt, a.n, 128);
  a.min_votes = t.staged_min_votes;
  rtk::QueueArgs q{};
  q.state = qs.state;
  q.slab = qs.slab;
  q.hist = qs.hist;
  q.n_bins = n_bins;
  q.slot_bytes = slot;
  for (uint32_t k = 0; k < rounds; ++k) {
    if (k > 0) {
      // the rays left after round k-1, grouped by the treelet they need
      rtk::bin_scan_kernel<<<n_blocks, 1024, 0, st>>>(qs.hist, qs.offset, qs.block_sum, n_bins);
      rtk::bin_scan_top_kernel<<<1, 1024, 0, st>>>(qs.block_sum, n_blocks);
      rtk::bin_scatter_kernel<<<std::min<uint32_t>((a.n + 255) / 256, 4096), 256, 0, st>>>(
          qs.out_ray, qs.out_key, qs.ctr + 2 * (k - 1) + 1, qs.offset, qs.block_sum, qs.in_ray, qs.in_key);
    }
    q.in_ray = k ? qs.in_ray : nullptr;
    q.in_key = k ? qs.in_key : nullptr;
    q.n_in = k ? qs.ctr + 2 * (k - 1) + 1 : nullptr;
    q.take = qs.ctr + 2 * k;
    q.out_ray = qs.out_ray;
    q.out_key = qs.out_key;
    q.n_out = qs.ctr + 2 * k + 1;
    kern<<<grid, bt, dyn, st>>>(a, q);
  }
  // the rays left walk to their ends; the queue lists of the last round are
  // its input as they are (no sort)
  q.in_ray = qs.out_ray;
  q.in_key = qs.out_key;
  q.n_in = qs.ctr + 2 * (rounds - 1) + 1;
  q.take = qs.ctr + 2 * rounds;
  q.out_ray = q.out_key = q.n_out = nullptr;
  q.slot_bytes = 0;
  fin<<<grid_fin, bt, 128, st>>>(a, q);
  RT_CUDA(cudaGetLastError());
  return RT_OK;
}

// Zeroes the launch's queue (and its counters unless `keep` is set: chunks of
// one call add up), then launches the kernel of `mode` with stack depth CAP.
template <int CAP>
rt_status launch_cap(rtk::TraceArgs& a, uint32_t mode, const rt_tuning& t, uint32_t largest_image, cudaStream_t st,
                     bool keep, const rti::QueueScratch* qs) {
  a.epoch = t.staged_epoch;
  a.refill = t.refill_lanes;
  a.wait_tries = t.wait_tries;
  if (!keep) {
    RT_CUDA(cudaMemsetAsync(a.stats, 0, sizeof(unsigned long long) * rtk::ST_COUNT, st));
    RT_CUDA(cudaMemsetAsync(a.status, 0, sizeof(uint32_t), st));
  }
  RT_CUDA(cudaMemsetAsync(a.queue, 0, sizeof(uint32_t), st));
  // A launch that writes traces runs the walks compiled with the trace code
  // (TRACED).  The plain walk writes its rows a whole 32-byte sector at a
  // time through shared memory (rtk::trace_put) when every row starts on a
  // 32-byte boundary, else entry by entry; the treelet walks write entry by
  // entry (staging their rows through shared memory, inline at each
  // recording site or through a per-lane ring written once per node visit,
  // measured 5-31% slower on their traced launches).
  const bool traced = a.cap != 0;
  const bool stage_rows = traced && mode == RT_MODE_PLAIN && (a.cap % 8u) == 0 &&
                          ((uintptr_t)a.visits & 31u) == 0 && ((uintptr_t)a.tl_trace & 31u) == 0;
  const uint32_t stage_warp_bytes = rtk::kTraceBufWarpBytes;
  a.tbuf_off = rtk::kNone;
  a.ss_off = rtk::kNone;
  if (mode == RT_MODE_PLAIN || mode == RT_MODE_TREELET) {
    const uint32_t bt = t.block_threads;
    size_t dyn = stage_rows ? (size_t)(bt / 32) * stage_warp_bytes + 128 : 0;
    if (stage_rows) a.tbuf_off = 0;
    // the warp-synchronous short stack, after the trace staging area
    const bool short_stack = mode == RT_MODE_PLAIN && !a.n_items && t.short_stack == 1;
    if (short_stack) {
      a.ss_off = stage_rows ? (uint32_t)(bt / 32) * stage_warp_bytes : 0u;
      dyn = a.ss_off + (size_t)(bt / 32) * rtk::kShortStackWarpBytes + 128;
    }
    void (*kern)(rtk::TraceArgs);
    if (short_stack)
      kern = traced ? rtk::trace_plain_kernel<CAP, false, true, true> : rtk::trace_plain_kernel<CAP, false, false, true>;
    else if (mode == RT_MODE_PLAIN)
      kern = a.n_items ? (traced ? rtk::trace_plain_kernel<CAP, true, true> : rtk::trace_plain_kernel<CAP, true, false>)
                       : (traced ? rtk::trace_plain_kernel<CAP, false, true> : rtk::trace_plain_kernel<CAP, false, false>);
    else
      kern = a.n_items
                 ? (traced ? rtk::trace_treelet_kernel<CAP, true, true> : rtk::trace_treelet_kernel<CAP, true, false>)
                 : (traced ? rtk::trace_treelet_kernel<CAP, false, true> : rtk::trace_treelet_kernel<CAP, false, false>);
    kern<<<persistent_grid((const void*)kern, bt, a.n, dyn), bt, dyn, st>>>(a);
  } else if (qs) {
    if (a.n_items) return rti::fail(RT_ERR_INVALID, "staged traces run over one scene");
    return launch_queued<CAP>(a, t, largest_image, *qs, st);
  } else {
    // the staged kernel is compiled for launches over one scene
    if (a.n_items) return rti::fail(RT_ERR_INVALID, "staged traces run over one scene");
    const uint32_t bt = t.staged_threads;
    const uint32_t warps = bt / 32;
    // per-warp slots: the whole largest image, or the first staged_slot_bytes of each
    uint32_t slot_bytes = largest_image;
    if (t.staged_slot_bytes) slot_bytes = std::min(slot_bytes, (t.staged_slot_bytes + 127u) & ~127u);
    uint32_t slots = t.staged_slots == RT_TUNING_OFF ? 0u : t.staged_slots;
    if (slot_bytes == 0) slots = 0;
    const uint64_t limit = staged_smem_limit();
    if ((uint64_t)a.pin_bytes + 128 > limit) {  // cannot happen for images built by rebuild_pinned
      a.pin_bytes = 0;
      a.pin_root = 0;
    }
    while (slots > 0 && (uint64_t)a.pin_bytes + (uint64_t)warps * slots * slot_bytes + 128 > limit) --slots;
    a.slots = slots;
    a.slot_bytes = slot_bytes;
    a.min_votes = t.staged_min_votes;
    const size_t dyn = (size_t)a.pin_bytes + (size_t)warps * slots * slot_bytes + 128;
    auto kern = slots ? (traced ? rtk::trace_staged_kernel<CAP, true, true> : rtk::trace_staged_kernel<CAP, true, false>)
                      : (traced ? rtk::trace_staged_kernel<CAP, false, true> : rtk::trace_staged_kernel<CAP, false, false>);
    RT_CUDA(ensure_dyn_smem((const void*)kern, dyn));
    kern<<<persistent_grid((const void*)kern, bt, a.n, dyn), bt, dyn, st>>>(a);
  }
  RT_CUDA(cudaGetLastError());
  return RT_OK;
}

// Stack depths compiled in (entries per stack per ray); a ray that needs more
// is flagged RT_RAY_STACK_OVERFLOW.
rt_status launch_trace(rtk::TraceArgs& a, uint32_t mode, const rt_tuning& t, uint32_t largest_image,
                       cudaStream_t st, bool keep = false, const rti::QueueScratch* qs = nullptr) {
  switch (t.stack_depth) {
    case 48:
      return launch_cap<48>(a, mode, t, largest_image, st, keep, qs);
    case 160:
      return launch_cap<160>(a, mode, t, largest_image, st, keep, qs);
    default:
      return launch_cap<96>(a, mode, t, largest_image, st, keep, qs);
  }
}

// True when a staged launch of the scene runs with treelet queues.
bool queued(const rt_scene* s, uint32_t mode) {
  return mode == RT_MODE_STAGED && s->tuning.queue_rounds != RT_TUNING_OFF && s->tuning.queue_rounds > 0;
}

// Grows the scene's queue memory to n rays (stack_depth entries per ray).
rt_status ensure_queue_scratch(rt_scene* s, uint32_t n) {
  rti::QueueScratch& q = s->qs;
  const uint64_t cap = s->tuning.stack_depth;
  const uint64_t n_bins = (uint64_t)s->part.roots.size() + 1;
  const uint64_t n_blocks = (n_bins + rtk::kBinScanItems - 1) / rtk::kBinScanItems;
  auto al = [](uint64_t b) { return (b + 255) & ~255ull; };
  const uint64_t b_state = al(64ull * n), b_slab = al(8ull * cap * n), b_list = al(4ull * n);
  const uint64_t b_bins = al(4ull * n_bins), b_blocks = al(4ull * n_blocks);
  const uint64_t b_ctr = al(sizeof(uint32_t) * 2 * (rti::kMaxQueueRounds + 1));
  const uint64_t need = b_state + b_slab + 4 * b_list + 2 * b_bins + b_blocks + b_ctr;
  if (need > q.bytes) {
    cudaFree(q.base);
    q = rti::QueueScratch{};
    rt_status st = dalloc(&q.base, need);
    if (st != RT_OK) return st;
    q.bytes = need;
  }
  uint8_t* p = q.base;
  auto take = [&](uint64_t b) {
    uint8_t* r = p;
    p += b;
    return r;
  };
  q.state = reinterpret_cast<uint4*>(take(b_state));
  q.slab = reinterpret_cast<unsigned long long*>(take(b_slab));
  q.in_ray = reinterpret_cast<uint32_t*>(take(b_list));
  q.in_key = reinterpret_cast<uint32_t*>(take(b_list));
  q.out_ray = reinterpret_cast<uint32_t*>(take(b_list));
  q.out_key = reinterpret_cast<uint32_t*>(take(b_list));
  q.hist = reinterpret_cast<uint32_t*>(take(b_bins));
  q.offset = reinterpret_cast<uint32_t*>(take(b_bins));
  q.block_sum = reinterpret_cast<uint32_t*>(take(b_blocks));
  q.ctr = reinterpret_cast<uint32_t*>(take(b_ctr));
  return RT_OK;
}

}  // namespace

extern "C" {

const char* rt_last_error(void) { return rti::g_error.c_str(); }
const char* rt_version(void) { return "treelet_rt 0.1 (sm_103a)"; }

rt_status rt_blob_validate(const rt_blob* blob) {
  if (!blob) return rti::fail(RT_ERR_INVALID, "rt_blob_validate: NULL");
  std::string err;
  if (!rti::validate_blob(blob->bytes.data(), blob->bytes.size(), &err)) return rti::fail(RT_ERR_BLOB, err);
  return RT_OK;
}

rt_status rt_ctx_create(int device, rt_ctx** out) {
  if (!out) return rti::fail(RT_ERR_INVALID, "rt_ctx_create: out is NULL");
  *out = nullptr;
  int n = 0;
  cudaError_t e = cudaGetDeviceCount(&n);
  if (e != cudaSuccess || n == 0) return rti::fail(RT_ERR_NO_DEVICE, "rt_ctx_create: no CUDA device");
  if (device < 0 || device >= n) return rti::fail(RT_ERR_INVALID, "rt_ctx_create: bad device ordinal");
  RT_CUDA(cudaSetDevice(device));
  auto* c = new rt_ctx();
  c->device = device;
  *out = c;
  return RT_OK;
}

rt_status rt_ctx_destroy(rt_ctx* ctx) {
  delete ctx;
  return RT_OK;
}

rt_status rt_scene_create(rt_ctx* ctx, const rt_blob* blob, rt_scene** out) {
  if (!ctx || !blob || !out) return rti::fail(RT_ERR_INVALID, "rt_scene_create: NULL argument");
  *out = nullptr;
  std::string err;
  if (!rti::validate_blob(blob->bytes.data(), blob->bytes.size(), &err)) return rti::fail(RT_ERR_BLOB, err);
  if (blob->bytes.size() / 64 >= (1ull << 29))
    return rti::fail(RT_ERR_TOO_LARGE, "rt_scene_create: blobs are limited to 2^29 units of 64 bytes");
  RT_CUDA(cudaSetDevice(ctx->device));
  auto* s = new rt_scene();
  s->ctx = ctx;
  s->host_blob = blob->bytes;
  s->blob_bytes = blob->bytes.size();
  s->n_units = (uint32_t)(s->blob_bytes / 64);
  rt_status st = dalloc(&s->d_blob, s->blob_bytes);
  if (st == RT_OK) st = dalloc(&s->d_stats, sizeof(unsigned long long) * rtk::ST_COUNT);
  if (st == RT_OK) st = dalloc(&s->d_status, sizeof(uint32_t));
  if (st == RT_OK) st = dalloc(&s->d_queue, sizeof(uint32_t) * rti::kHostChunks);
  if (st != RT_OK) {
    rt_scene_destroy(s);
    return st;
  }
  cudaError_t e = cudaMemcpy(s->d_blob, blob->bytes.data(), s->blob_bytes, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemset(s->d_stats, 0, sizeof(unsigned long long) * rtk::ST_COUNT);
  if (e == cudaSuccess) e = cudaMemset(s->d_status, 0, sizeof(uint32_t));
  for (cudaStream_t* x : {&s->stream, &s->stream2, &s->xin, &s->xout})
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(x, cudaStreamNonBlocking);
  for (uint32_t c = 0; c < rti::kHostChunks; ++c) {
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&s->ev_in[c], cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&s->ev_done[c], cudaEventDisableTiming);
  }
  if (e != cudaSuccess) {
    rt_scene_destroy(s);
    return cuda_fail(e, "rt_scene_create");
  }
  *out = s;
  return RT_OK;
}

rt_status rt_scene_destroy(rt_scene* s) {
  if (!s) return RT_OK;
  cudaSetDevice(s->ctx->device);
  free_treelets(s);
  cudaFree(s->d_blob);
  cudaFree(s->d_stats);
  cudaFree(s->d_status);
  cudaFree(s->d_queue);
  cudaFree(s->d_io);
  cudaFree(s->d_pack);
  if (s->h_tot) cudaFreeHost(s->h_tot);
  cudaFree(s->qs.base);
  for (uint32_t c = 0; c < rti::kHostChunks; ++c) {
    if (s->ev_in[c]) cudaEventDestroy(s->ev_in[c]);
    if (s->ev_done[c]) cudaEventDestroy(s->ev_done[c]);
  }
  for (cudaStream_t x : {s->stream, s->stream2, s->xin, s->xout})
    if (x) cudaStreamDestroy(x);
  delete s;
  return RT_OK;
}

rt_status rt_scene_device_blob(const rt_scene* s, const void** dptr, uint64_t* n_bytes) {
  if (!s || !dptr || !n_bytes) return rti::fail(RT_ERR_INVALID, "rt_scene_device_blob: NULL");
  *dptr = s->d_blob;
  *n_bytes = s->blob_bytes;
  return RT_OK;
}

rt_status rt_treelets_form(rt_scene* s, uint32_t max_treelet_bytes, rt_treelet_info* info) {
  if (!s) return rti::fail(RT_ERR_INVALID, "rt_treelets_form: NULL scene");
  std::string err;
  rtt::Partition p;
  if (!rtt::form_treelets(s->host_blob.data(), s->blob_bytes, max_treelet_bytes, p, &err))
    return rti::fail(RT_ERR_INVALID, "rt_treelets_form: " + err);
  std::vector<uint8_t> store;
  rtt::build_images(s->host_blob.data(), p, store);
  RT_CUDA(cudaSetDevice(s->ctx->device));
  free_treelets(s);
  const uint32_t n = (uint32_t)p.roots.size();
  std::vector<uint2> meta(s->n_units);
  for (uint32_t u = 0; u < s->n_units; ++u) meta[u] = make_uint2(p.node_root[u], p.node_loc[u]);
  rt_status st = dalloc(&s->d_meta, sizeof(uint2) * meta.size());
  if (st == RT_OK) st = dalloc(&s->d_images, store.size());
  if (st == RT_OK) st = dalloc(&s->d_image_off, sizeof(unsigned long long) * (n + 1));
  if (st == RT_OK) st = dalloc(&s->d_roots, sizeof(uint32_t) * n);
  if (st == RT_OK) st = dalloc(&s->d_member_first, sizeof(unsigned long long) * (n + 1));
  if (st == RT_OK) st = dalloc(&s->d_member_bytes, sizeof(uint16_t) * p.member_bytes.size());
  if (st != RT_OK) {
    free_treelets(s);
    return st;
  }
  std::vector<unsigned long long> off(p.image_off.begin(), p.image_off.end());
  std::vector<unsigned long long> mf(p.member_first.begin(), p.member_first.end());
  RT_CUDA(cudaMemcpy(s->d_meta, meta.data(), sizeof(uint2) * meta.size(), cudaMemcpyHostToDevice));
  if (!store.empty()) RT_CUDA(cudaMemcpy(s->d_images, store.data(), store.size(), cudaMemcpyHostToDevice));
  RT_CUDA(cudaMemcpy(s->d_image_off, off.data(), sizeof(unsigned long long) * off.size(), cudaMemcpyHostToDevice));
  if (n) RT_CUDA(cudaMemcpy(s->d_roots, p.roots.data(), sizeof(uint32_t) * n, cudaMemcpyHostToDevice));
  RT_CUDA(cudaMemcpy(s->d_member_first, mf.data(), sizeof(unsigned long long) * mf.size(), cudaMemcpyHostToDevice));
  if (!p.member_bytes.empty())
    RT_CUDA(cudaMemcpy(s->d_member_bytes, p.member_bytes.data(), sizeof(uint16_t) * p.member_bytes.size(),
                       cudaMemcpyHostToDevice));
  st = dalloc(&s->d_members, sizeof(uint32_t) * p.members.size());
  if (st != RT_OK) {
    free_treelets(s);
    return st;
  }
  if (!p.members.empty())
    RT_CUDA(cudaMemcpy(s->d_members, p.members.data(), sizeof(uint32_t) * p.members.size(), cudaMemcpyHostToDevice));
  s->slot_bytes = (p.largest_image + 127u) & ~127u;
  s->part = std::move(p);
  st = dalloc(&s->d_route, sizeof(uint16_t) * (s->blob_bytes / 64));
  if (st != RT_OK) {
    free_treelets(s);
    return st;
  }
  s->has_treelets = true;
  st = upload_route(s);
  if (st != RT_OK) {
    free_treelets(s);
    return st;
  }
  if (info) {
    info->n_treelets = n;
    info->max_treelet_bytes = max_treelet_bytes;
    info->member_entries = s->part.members.size();
    info->image_bytes = s->part.image_bytes;
    info->largest_image = s->part.largest_image;
    info->reserved = 0;
  }
  return RT_OK;
}

rt_status rt_treelets_get(const rt_scene* s, uint32_t* roots, uint64_t* member_first, uint32_t* members,
                          uint16_t* member_bytes, uint32_t* node_root) {
  if (!s) return rti::fail(RT_ERR_INVALID, "rt_treelets_get: NULL scene");
  if (!s->has_treelets) return rti::fail(RT_ERR_STATE, "rt_treelets_get: treelets not formed");
  const rtt::Partition& p = s->part;
  if (roots) std::copy(p.roots.begin(), p.roots.end(), roots);
  if (member_first) std::copy(p.member_first.begin(), p.member_first.end(), member_first);
  if (members) std::copy(p.members.begin(), p.members.end(), members);
  if (member_bytes) std::copy(p.member_bytes.begin(), p.member_bytes.end(), member_bytes);
  if (node_root) std::copy(p.node_root.begin(), p.node_root.end(), node_root);
  return RT_OK;
}

rt_status rt_treelets_remap(const rt_scene* s, uint32_t stride, uint64_t* new_addr) {
  if (!s || !new_addr) return rti::fail(RT_ERR_INVALID, "rt_treelets_remap: NULL argument");
  if (!s->has_treelets) return rti::fail(RT_ERR_STATE, "rt_treelets_remap: treelets not formed");
  std::vector<uint64_t> m;
  std::string err;
  if (!rtt::remap_layout(s->part, s->n_units, stride, m, &err)) return rti::fail(RT_ERR_STATE, err);
  std::copy(m.begin(), m.end(), new_addr);
  return RT_OK;
}

rt_status rt_scene_set_tuning(rt_scene* s, const rt_tuning* t) {
  if (!s || !t) return rti::fail(RT_ERR_INVALID, "rt_scene_set_tuning: NULL");
  rt_tuning n;
  rt_status st = merge_tuning(s->tuning, t, n);
  if (st != RT_OK) return st;
  const bool repin = n.pinned_bytes != s->tuning.pinned_bytes;
  s->tuning = n;
  if (repin && s->has_treelets) {
    RT_CUDA(cudaSetDevice(s->ctx->device));
    return rebuild_pinned(s, true);
  }
  return RT_OK;
}

rt_status rt_scene_set_pin_order(rt_scene* s, const uint32_t* order, uint32_t n) {
  if (!s) return rti::fail(RT_ERR_INVALID, "rt_scene_set_pin_order: NULL scene");
  if (!s->has_treelets) return rti::fail(RT_ERR_STATE, "rt_scene_set_pin_order: call rt_treelets_form first");
  if (order && n == 0) return rti::fail(RT_ERR_INVALID, "rt_scene_set_pin_order: empty order");
  if (order) s->pin_order.assign(order, order + n);
  else s->pin_order.clear();
  RT_CUDA(cudaSetDevice(s->ctx->device));
  drop_pin_cache(s);
  return rebuild_pinned(s);
}

rt_status rt_scene_set_device_offset(rt_scene* s, uint64_t device_offset) {
  if (!s) return rti::fail(RT_ERR_INVALID, "rt_scene_set_device_offset: NULL scene");
  if (s->offset_quirk == (device_offset != 0)) return RT_OK;
  s->offset_quirk = device_offset != 0;
  if (!s->has_treelets) return RT_OK;
  RT_CUDA(cudaSetDevice(s->ctx->device));
  return upload_route(s);
}

rt_status rt_scene_pinned_info(rt_scene* s, rt_pinned_info* info) {
  if (!s || !info) return rti::fail(RT_ERR_INVALID, "rt_scene_pinned_info: NULL");
  *info = s->pin_info;
  return RT_OK;
}

rt_status rt_scene_get_tuning(const rt_scene* s, rt_tuning* t) {
  if (!s || !t) return rti::fail(RT_ERR_INVALID, "rt_scene_get_tuning: NULL");
  *t = s->tuning;
  return RT_OK;
}

}  // extern "C"

namespace {

// Argument checks shared by rt_trace and rt_trace_host.
rt_status check_trace(const rt_scene* s, uint32_t mode, const rt_trace_buf* trace, const char* who) {
  if (mode > RT_MODE_STAGED) return rti::fail(RT_ERR_INVALID, std::string(who) + ": unknown mode");
  const bool want_tl = trace && trace->treelets;
  if ((mode != RT_MODE_PLAIN || want_tl) && !s->has_treelets)
    return rti::fail(RT_ERR_STATE, std::string(who) + ": call rt_treelets_form first");
  if (trace && (trace->visits || trace->treelets) && trace->capacity == 0)
    return rti::fail(RT_ERR_INVALID, std::string(who) + ": trace capacity is 0");
  if (mode == RT_MODE_STAGED && s->part.roots.size() >= rtt::kMaxDense)
    return rti::fail(RT_ERR_TOO_LARGE, std::string(who) + ": too many treelets for staged mode (max 4194304)");
  return RT_OK;
}

// Launches one trace over device arrays.  `queue` is the ray hand-out
// counter of this launch; `keep` adds the counters to the previous launch's.
rt_status trace_launch(rt_scene* s, const rt_ray* rays, const uint32_t* flags, uint32_t default_flags, uint32_t n,
                       uint32_t mode, rt_hit* hits, const rt_trace_buf* trace, cudaStream_t st, uint32_t* queue,
                       bool keep, bool allow_queues = true) {
  rtk::TraceArgs a{};
  a.blob = reinterpret_cast<const uint4*>(s->d_blob);
  a.n_units = s->n_units;
  a.rays = rays;
  a.flags = flags;
  a.default_flags = default_flags;
  a.n = n;
  a.hits = hits;
  a.visits = trace ? trace->visits : nullptr;
  a.tl_trace = trace ? trace->treelets : nullptr;
  a.cap = (trace && (trace->visits || trace->treelets)) ? trace->capacity : 0;
  a.meta = s->d_meta;
  a.route = s->d_route;
  if (mode == RT_MODE_STAGED && s->d_pin) {
    a.pin_image = reinterpret_cast<const uint4*>(s->d_pin);
    a.pin_bytes = s->pin_info.bytes;
    a.pin_root = s->pin_root;
  }
  a.images = reinterpret_cast<const uint4*>(s->d_images);
  a.image_off = s->d_image_off;
  a.n_treelets = s->has_treelets ? (uint32_t)s->part.roots.size() : 0;
  a.stats = s->d_stats;
  a.status = s->d_status;
  a.queue = queue;
  a.hint = s->d_hint;
  if (allow_queues && queued(s, mode)) {
    rt_status qst = ensure_queue_scratch(s, n);
    if (qst != RT_OK) return qst;
    return launch_trace(a, mode, s->tuning, s->slot_bytes, st, keep, &s->qs);
  }
  return launch_trace(a, mode, s->tuning, s->slot_bytes, st, keep);
}

// The device address of a page-locked, mapped host array (cudaHostAlloc or
// cudaHostRegister with mapping, which unified addressing gives by default),
// or nullptr for pageable memory.
void* mapped_host(const void* p) {
  cudaPointerAttributes at{};
  if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
    cudaGetLastError();  // pageable memory on older drivers: not an error here
    return nullptr;
  }
  return at.type == cudaMemoryTypeHost ? at.devicePointer : nullptr;
}

// Waits for every stream of the host path; returns `st` (or the first CUDA
// error if `st` is RT_OK).
rt_status host_finish(rt_scene* s, rt_status st) {
  cudaError_t e = cudaSuccess;
  for (cudaStream_t x : {s->xin, s->stream, s->stream2, s->xout}) {
    if (!x) continue;
    const cudaError_t ex = cudaStreamSynchronize(x);
    if (e == cudaSuccess) e = ex;
  }
  if (st == RT_OK && e != cudaSuccess) return cuda_fail(e, "rt_trace_host");
  if (st == RT_OK) return rti::check_device_status(s, "rt_trace_host");
  return st;
}

}  // namespace

namespace rti {

// Reads the scene's device status word after its traces have finished and
// turns a bounded wait that gave up into RT_ERR_TIMEOUT.  Hit records stay
// valid then: the kernel stops staging and reads nodes from global memory.
rt_status check_device_status(rt_scene* s, const char* who) {
  uint32_t status = 0;
  const cudaError_t e = cudaMemcpy(&status, s->d_status, sizeof(status), cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return cuda_fail(e, who);
  if (status & rtk::kStatusTimeout)
    return fail(RT_ERR_TIMEOUT, std::string(who) +
                                    ": a bounded staging wait gave up (hit records are valid; staging was switched "
                                    "off for the rest of the launch)");
  return RT_OK;
}

}  // namespace rti

extern "C" {

rt_status rt_trace(rt_scene* s, const rt_ray* rays, const uint32_t* flags, uint32_t default_flags, uint32_t n,
                   uint32_t mode, rt_hit* hits, const rt_trace_buf* trace, void* stream) {
  if (!s) return rti::fail(RT_ERR_INVALID, "rt_trace: NULL scene");
  if (n == 0) return RT_OK;
  if (!rays || !hits) return rti::fail(RT_ERR_INVALID, "rt_trace: NULL rays or hits");
  rt_status st = check_trace(s, mode, trace, "rt_trace");
  if (st != RT_OK) return st;
  RT_CUDA(cudaSetDevice(s->ctx->device));
  return trace_launch(s, rays, flags, default_flags, n, mode, hits, trace, (cudaStream_t)stream, s->d_queue, false);
}

rt_status rt_scene_set_stage_hints(rt_scene* s, const uint32_t* hints) {
  if (!s) return rti::fail(RT_ERR_INVALID, "rt_scene_set_stage_hints: NULL scene");
  if (!s->has_treelets) return rti::fail(RT_ERR_STATE, "rt_scene_set_stage_hints: call rt_treelets_form first");
  RT_CUDA(cudaSetDevice(s->ctx->device));
  cudaFree(s->d_hint);
  s->d_hint = nullptr;
  if (!hints) return RT_OK;
  const size_t n = (size_t)s->part.roots.size() * 8;
  rt_status st = dalloc(&s->d_hint, sizeof(uint32_t) * n);
  if (st != RT_OK) return st;
  RT_CUDA(cudaMemcpy(s->d_hint, hints, sizeof(uint32_t) * n, cudaMemcpyHostToDevice));
  return RT_OK;
}

rt_status rt_trace_stats_get(rt_scene* s, rt_trace_stats* out) {
  if (!s || !out) return rti::fail(RT_ERR_INVALID, "rt_trace_stats_get: NULL");
  unsigned long long v[rtk::ST_COUNT];
  uint32_t status = 0;
  RT_CUDA(cudaMemcpy(v, s->d_stats, sizeof(v), cudaMemcpyDeviceToHost));
  RT_CUDA(cudaMemcpy(&status, s->d_status, sizeof(status), cudaMemcpyDeviceToHost));
  out->node_bytes = v[rtk::ST_NODE_BYTES];
  out->staged_bytes = v[rtk::ST_STAGED_BYTES];
  out->smem_reads = v[rtk::ST_SMEM_READS];
  out->gmem_reads = v[rtk::ST_GMEM_READS];
  out->stagings = v[rtk::ST_STAGINGS];
  out->device_status = status;
  return RT_OK;
}

rt_status rt_trace_host(rt_scene* s, const rt_ray* rays, const uint32_t* flags, uint32_t default_flags, uint32_t n,
                        uint32_t mode, rt_hit* hits, const rt_trace_buf* trace) {
  if (!s) return rti::fail(RT_ERR_INVALID, "rt_trace_host: NULL scene");
  if (n == 0) return RT_OK;
  if (!rays || !hits) return rti::fail(RT_ERR_INVALID, "rt_trace_host: NULL rays or hits");
  rt_status st = check_trace(s, mode, trace, "rt_trace_host");
  if (st != RT_OK) return st;
  RT_CUDA(cudaSetDevice(s->ctx->device));
  const uint32_t cap = (trace && (trace->visits || trace->treelets)) ? trace->capacity : 0;
  auto al = [](size_t b) { return (b + 255) & ~(size_t)255; };
  // Page-locked hit records: the kernel writes them straight into host memory
  // as rays finish, so no copy-out follows the trace and one launch over all
  // rays needs no chunks (chunked launches each pay a tail of long rays).
  // Page-locked rays (and flags) are read by the kernel where they are, each
  // once, when a lane takes its ray; pageable ones are copied in first, in one
  // copy each.
  if (!cap) {
    rt_hit* mapped_hits = static_cast<rt_hit*>(mapped_host(hits));
    const rt_ray* mapped_rays = mapped_hits ? static_cast<const rt_ray*>(mapped_host(rays)) : nullptr;
    const uint32_t* mapped_flags = (mapped_rays && flags) ? static_cast<const uint32_t*>(mapped_host(flags)) : nullptr;
    if (mapped_rays && (!flags || mapped_flags)) {
      st = trace_launch(s, mapped_rays, mapped_flags, default_flags, n, mode, mapped_hits, nullptr, s->stream,
                        s->d_queue, false);
      return host_finish(s, st);
    }
    if (mapped_hits) {
      const size_t b_rays = al(sizeof(rt_ray) * (size_t)n), b_flags = flags ? sizeof(uint32_t) * (size_t)n : 0;
      if (b_rays + b_flags > s->io_bytes) {
        cudaFree(s->d_io);
        s->d_io = nullptr;
        s->io_bytes = 0;
        st = dalloc((uint8_t**)&s->d_io, b_rays + b_flags);
        if (st != RT_OK) return st;
        s->io_bytes = b_rays + b_flags;
      }
      rt_ray* d_rays = (rt_ray*)s->d_io;
      uint32_t* d_flags = flags ? (uint32_t*)((uint8_t*)s->d_io + b_rays) : nullptr;
      cudaError_t e = cudaMemcpyAsync(d_rays, rays, sizeof(rt_ray) * (size_t)n, cudaMemcpyHostToDevice, s->stream);
      if (e == cudaSuccess && flags)
        e = cudaMemcpyAsync(d_flags, flags, sizeof(uint32_t) * (size_t)n, cudaMemcpyHostToDevice, s->stream);
      if (e != cudaSuccess) return host_finish(s, cuda_fail(e, "rt_trace_host"));
      st = trace_launch(s, d_rays, d_flags, default_flags, n, mode, mapped_hits, nullptr, s->stream, s->d_queue,
                        false);
      return host_finish(s, st);
    }
  }
  const size_t b_rays = al(sizeof(rt_ray) * (size_t)n), b_flags = flags ? al(sizeof(uint32_t) * (size_t)n) : 0;
  const size_t b_hits = al(sizeof(rt_hit) * (size_t)n);
  const size_t b_vis = (trace && trace->visits) ? al(sizeof(uint32_t) * (size_t)n * cap) : 0;
  const size_t b_tl = (trace && trace->treelets) ? al(sizeof(uint32_t) * (size_t)n * cap) : 0;
  const size_t need = b_rays + b_flags + b_hits + b_vis + b_tl;
  if (need > s->io_bytes) {
    cudaFree(s->d_io);
    s->d_io = nullptr;
    s->io_bytes = 0;
    st = dalloc((uint8_t**)&s->d_io, need);
    if (st != RT_OK) return st;
    s->io_bytes = need;
  }
  uint8_t* base = (uint8_t*)s->d_io;
  rt_ray* d_rays = (rt_ray*)base;
  uint32_t* d_flags = flags ? (uint32_t*)(base + b_rays) : nullptr;
  rt_hit* d_hits = (rt_hit*)(base + b_rays + b_flags);
  uint32_t* d_vis = b_vis ? (uint32_t*)(base + b_rays + b_flags + b_hits) : nullptr;
  uint32_t* d_tl = b_tl ? (uint32_t*)(base + b_rays + b_flags + b_hits + b_vis) : nullptr;

  // Chunks pipeline the copies with the traces: rays of chunk c+1 go in and
  // hits of chunk c-1 come out while chunk c is traced.
  uint64_t bound[rti::kHostChunks + 1];
  // a queued staged launch runs whole: its queues are the scene's, one set
  uint32_t chunks = 1;
  bound[0] = 0;
  bound[1] = n;
  if (!queued(s, mode)) chunks = rti::host_chunk_bounds(n, bound);
  // counters of the whole call start at zero, ahead of every chunk's copy-in
  RT_CUDA(cudaMemsetAsync(s->d_stats, 0, sizeof(unsigned long long) * rtk::ST_COUNT, s->xin));
  RT_CUDA(cudaMemsetAsync(s->d_status, 0, sizeof(uint32_t), s->xin));
  cudaError_t e = cudaSuccess;
  for (uint32_t c = 0; c < chunks && e == cudaSuccess && st == RT_OK; ++c) {
    const size_t lo = bound[c], m = bound[c + 1] - bound[c];
    e = cudaMemcpyAsync(d_rays + lo, rays + lo, sizeof(rt_ray) * m, cudaMemcpyHostToDevice, s->xin);
    if (e == cudaSuccess && flags)
      e = cudaMemcpyAsync(d_flags + lo, flags + lo, sizeof(uint32_t) * m, cudaMemcpyHostToDevice, s->xin);
    if (e == cudaSuccess) e = cudaEventRecord(s->ev_in[c], s->xin);
    cudaStream_t cs = (c & 1) ? s->stream2 : s->stream;
    if (e == cudaSuccess) e = cudaStreamWaitEvent(cs, s->ev_in[c], 0);
    if (e != cudaSuccess) break;
    rt_trace_buf tb{d_vis ? d_vis + lo * cap : nullptr, d_tl ? d_tl + lo * cap : nullptr, cap};
    st = trace_launch(s, d_rays + lo, d_flags ? d_flags + lo : nullptr, default_flags, (uint32_t)m, mode, d_hits + lo,
                      cap ? &tb : nullptr, cs, s->d_queue + c, true);
    if (st == RT_OK) e = cudaEventRecord(s->ev_done[c], cs);
  }
  for (uint32_t c = 0; c < chunks && e == cudaSuccess && st == RT_OK; ++c) {
    const size_t lo = bound[c], m = bound[c + 1] - bound[c];
    e = cudaStreamWaitEvent(s->xout, s->ev_done[c], 0);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(hits + lo, d_hits + lo, sizeof(rt_hit) * m, cudaMemcpyDeviceToHost, s->xout);
    if (e == cudaSuccess && d_vis)
      e = cudaMemcpyAsync(trace->visits + lo * cap, d_vis + lo * cap, sizeof(uint32_t) * m * cap,
                          cudaMemcpyDeviceToHost, s->xout);
    if (e == cudaSuccess && d_tl)
      e = cudaMemcpyAsync(trace->treelets + lo * cap, d_tl + lo * cap, sizeof(uint32_t) * m * cap,
                          cudaMemcpyDeviceToHost, s->xout);
  }
  if (st == RT_OK && e != cudaSuccess) st = cuda_fail(e, "rt_trace_host");
  return host_finish(s, st);
}

}  // extern "C"

// ------------------------------------------------------------ bounce rays
namespace {

__global__ void bounce_kernel(const uint4* blob, uint32_t n_units, const rt_ray* rays, const rt_hit* hits, uint32_t n,
                              uint64_t seed, float tmin, float tmax, rt_ray* out) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const rt_hit h = hits[i];
  const rt_ray ray = rays[i];
  rt_ray o;
  if (!h.hit_geometry || h.closest_leaf >= n_units || h.closest_instance + 1 >= n_units) {
    o = ray;
    o.tmin = 1.0f;
    o.tmax = 0.0f;
    out[i] = o;
    return;
  }
  rti::BounceInput in;
  uint4* lp = reinterpret_cast<uint4*>(in.leaf);
  uint4* ip = reinterpret_cast<uint4*>(in.inst);
  for (int q = 0; q < 4; ++q) lp[q] = blob[(uint64_t)h.closest_leaf * 4 + q];
  for (int q = 0; q < 8; ++q) ip[q] = blob[(uint64_t)h.closest_instance * 4 + q];
  rti::make_bounce(in, ray, h, seed, i, tmin, tmax, o);
  out[i] = o;
}

}  // namespace

extern "C" rt_status rt_gen_bounce_rays(rt_scene* s, const rt_ray* rays, const rt_hit* hits, uint32_t n, uint64_t seed,
                                        float tmin, float tmax, rt_ray* out, void* stream) {
  if (!s || !rays || !hits || !out) return rti::fail(RT_ERR_INVALID, "rt_gen_bounce_rays: NULL argument");
  if (n == 0) return RT_OK;
  RT_CUDA(cudaSetDevice(s->ctx->device));
  bounce_kernel<<<(n + 255) / 256, 256, 0, (cudaStream_t)stream>>>(reinterpret_cast<const uint4*>(s->d_blob),
                                                                     s->n_units, rays, hits, n, seed, tmin, tmax, out);
  RT_CUDA(cudaGetLastError());
  return RT_OK;
}

extern "C" rt_status rt_prefetch_decide(rt_scene* s, const uint32_t* next_unit, uint32_t n_units, uint32_t lanes,
                                        const rt_prefetch_params* params, rt_prefetch_state* state,
                                        rt_prefetch_decision* out, void* stream) {
  if (!s || !next_unit || !params || !state || !out) return rti::fail(RT_ERR_INVALID, "rt_prefetch_decide: NULL");
  if (!s->has_treelets) return rti::fail(RT_ERR_STATE, "rt_prefetch_decide: call rt_treelets_form first");
  if (lanes == 0 || lanes > (uint32_t)rtk::kMaxLanes)
    return rti::fail(RT_ERR_TOO_LARGE, "rt_prefetch_decide: lanes must be 1..1024");
  if (params->heuristic > RT_PREFETCH_LATTER) return rti::fail(RT_ERR_INVALID, "rt_prefetch_decide: unknown heuristic");
  if ((params->variant & 3u) > RT_PREFETCH_TREELET_QUEUE || (params->variant & ~(3u | RT_PREFETCH_FLUSH_ON_NEW_TREELET)))
    return rti::fail(RT_ERR_INVALID, "rt_prefetch_decide: unknown variant");
  if (n_units == 0) return RT_OK;
  RT_CUDA(cudaSetDevice(s->ctx->device));
  rtk::PrefetchArgs a{};
  a.next_unit = next_unit;
  a.n_groups = n_units;
  a.lanes = lanes;
  a.p = *params;
  a.state = state;
  a.out = out;
  a.meta = s->d_meta;
  a.n_units = s->n_units;
  a.roots = s->d_roots;
  a.member_first = s->d_member_first;
  a.member_bytes = s->d_member_bytes;
  a.n_treelets = (uint32_t)s->part.roots.size();
  rtk::prefetch_decide_kernel<<<n_units, 512, 0, (cudaStream_t)stream>>>(a);
  RT_CUDA(cudaGetLastError());
  return RT_OK;
}

extern "C" rt_status rt_unit_replay(rt_scene* s, const rt_hit* hits, const uint32_t* visits, uint32_t n,
                                    uint32_t capacity, const rt_unit_config* cfg, rt_unit_stats* stats,
                                    void* stream) {
  if (!s || !cfg || !stats) return rti::fail(RT_ERR_INVALID, "rt_unit_replay: NULL argument");
  if (!s->has_treelets) return rti::fail(RT_ERR_STATE, "rt_unit_replay: call rt_treelets_form first");
  const rt_unit_config& c = *cfg;
  auto bad = [](const char* m) { return rti::fail(RT_ERR_INVALID, std::string("rt_unit_replay: ") + m); };
  if (c.n_rt_units == 0) return bad("n_rt_units must be >= 1");
  if (c.max_warps == 0 || c.max_warps > rtr::kMaxResident) return bad("max_warps must be 1..16");
  if (c.l1_sets == 0 || (c.l1_sets & (c.l1_sets - 1)) || c.l1_sets > 65536) return bad("l1_sets must be a power of two <= 65536");
  if (c.l1_ways == 0 || c.l1_ways > 32) return bad("l1_ways must be 1..32");
  if (c.hit_latency == 0 || c.miss_latency == 0 || c.miss_latency >= rtr::kMetaRing || c.hit_latency > c.miss_latency)
    return bad("latencies must satisfy 1 <= hit <= miss < 4096");
  if (c.prefetcher > RT_UNIT_PF_STRIDE || c.scheduler > RT_UNIT_SCHED_PMR) return bad("unknown prefetcher or scheduler");
  if (c.prefetch_delay == 0) return bad("prefetch_delay must be >= 1");
  if (c.decision.heuristic > RT_PREFETCH_LATTER) return bad("unknown heuristic");
  if (c.decision.variant != 0) return bad("the replay models the main decision block: decision.variant must be 0");
  if (n == 0) {
    RT_CUDA(cudaMemsetAsync(stats, 0, sizeof(rt_unit_stats) * c.n_rt_units, (cudaStream_t)stream));
    return RT_OK;
  }
  if (!hits || !visits || capacity == 0) return bad("hits and visits are required");
  RT_CUDA(cudaSetDevice(s->ctx->device));
  const uint64_t n_treelets = s->part.roots.size();
  const uint64_t meta_size = (uint64_t)(s->part.max_bytes / 64) * 4;
  const uint64_t meta_base = (s->blob_bytes + 4095) & ~4095ull;
  // per-unit tables, sized to the sectors the unit can prefetch (blob and metadata), at most 2^20 entries
  auto log2_ceil = [](uint64_t v) {
    uint32_t l = 0;
    while ((1ull << l) < v) ++l;
    return l;
  };
  const uint64_t sectors = s->blob_bytes / 32 + n_treelets * meta_size / 32 + 4096;
  const uint32_t tab_log2 = std::max<uint32_t>(12, std::min<uint32_t>(20, log2_ceil(2 * sectors)));
  const uint32_t pq_cap = 1u << 18;
  auto align = [](uint64_t v) { return (v + 255) & ~255ull; };
  rtr::ReplayArgs a{};
  uint64_t off = 0;
  // the L1 lines live in shared memory when they fit, else in the scratch slice
  const uint64_t n_lines = (uint64_t)c.l1_sets * c.l1_ways;
  a.lines_shared = n_lines <= rtr::kSmemLinesMax ? 1u : 0u;
  a.off_lines = off;
  if (!a.lines_shared) off = align(off + sizeof(rtr::Line) * n_lines);
  a.off_sec = off;
  off = align(off + sizeof(rtr::SectorEntry) * (1ull << tab_log2));
  a.off_queued = off;
  off = align(off + sizeof(rtr::QueuedEntry) * (1ull << tab_log2));
  a.off_pq = off;
  off = align(off + 16ull * pq_cap);
  a.off_dead = off;
  off = align(off + pq_cap);
  a.off_meta = off;
  off = align(off + sizeof(rtr::MetaReturn) * rtr::kMetaRing);
  a.unit_bytes = off;
  const uint64_t total = off * c.n_rt_units;
  uint8_t* scratch = nullptr;
  rt_status st = dalloc(&scratch, total);
  if (st != RT_OK) return st;
  // the model's own bound on a unit's cycles: every round sends at most 128
  // requests, then waits at most a miss latency plus an intersection latency
  const uint64_t warps_per_unit = ((uint64_t)(n + 31) / 32 + c.n_rt_units - 1) / c.n_rt_units;
  uint64_t cap = warps_per_unit * capacity * (rtr::kChunkCap + c.miss_latency + 8) + 1024;
  if (c.max_cycles) cap = std::min<uint64_t>(cap, c.max_cycles);
  a.cycle_cap = (uint32_t)std::min<uint64_t>(cap, rtr::kTimeCap);
  a.hits = hits;
  a.visits = visits;
  a.n = n;
  a.capacity = capacity;
  a.cfg = c;
  a.stats = stats;
  a.meta = s->d_meta;
  a.n_units = s->n_units;
  a.roots = s->d_roots;
  a.member_first = s->d_member_first;
  a.members = s->d_members;
  a.member_bytes = s->d_member_bytes;
  a.n_treelets = (uint32_t)n_treelets;
  a.meta_base = meta_base;
  a.meta_size = meta_size;
  a.scratch = scratch;
  a.sec_log2 = a.queued_log2 = tab_log2;
  a.pq_cap = pq_cap;
  cudaStream_t sm = (cudaStream_t)stream;
  cudaError_t e = cudaMemsetAsync(scratch, 0, total, sm);
  if (e == cudaSuccess) {
    // one warp (CTA) per RT unit, its state in shared memory
    const size_t smem = ((sizeof(rtr::UnitShared) + 15) & ~(size_t)15) + (a.lines_shared ? sizeof(rtr::Line) * n_lines : 0);
    e = cudaFuncSetAttribute(rtr::unit_replay_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e == cudaSuccess) {
      rtr::unit_replay_kernel<<<c.n_rt_units, 32, smem, sm>>>(a);
      e = cudaGetLastError();
    }
  }
  // the scratch is released once the replay has finished on the stream
  if (e == cudaSuccess) e = cudaStreamSynchronize(sm);
  cudaFree(scratch);
  if (e != cudaSuccess) return cuda_fail(e, "rt_unit_replay");
  return RT_OK;
}

// ------------------------------------------------------------ batches
struct rt_batch {
  rt_ctx* ctx = nullptr;
  std::vector<rt_scene*> scenes;
  rtk::SceneView* d_views = nullptr;
  std::vector<rtk::SceneView> views;  // host copy of d_views
  uint32_t* d_item_begin = nullptr;
  uint32_t* d_item_scene = nullptr;
  uint32_t n_items = 0, n_rays = 0;
  std::vector<uint32_t> item_begin, item_scene;  // host copies (staged batches launch per item)
  unsigned long long* d_stats = nullptr;
  uint32_t* d_status = nullptr;
  uint32_t* d_queue = nullptr;
  rt_tuning tuning{128, 128, 16, 1, 8, 2048, 2, 96, RT_TUNING_OFF, rtk::kWaitTries, RT_TUNING_OFF,
                   RT_TUNING_OFF};  // batches pin nothing
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  // staged batches: item launches spread over side streams (one per scene
  // index modulo kBatchLanes), forked from and joined to the caller's stream
  static constexpr uint32_t kBatchLanes = 8;
  cudaStream_t lane[kBatchLanes] = {};
  cudaEvent_t ev_fork = nullptr, ev_join[kBatchLanes] = {};
};

namespace {

void free_graph(rt_batch* b) {
  if (b->exec) cudaGraphExecDestroy(b->exec);
  if (b->graph) cudaGraphDestroy(b->graph);
  b->exec = nullptr;
  b->graph = nullptr;
}

rt_status batch_args(rt_batch* b, const rt_ray* rays, const uint32_t* flags, uint32_t default_flags, uint32_t mode,
                     rt_hit* hits, rtk::TraceArgs& a) {
  if (!rays || !hits) return rti::fail(RT_ERR_INVALID, "rt_trace_batch: NULL rays or hits");
  if (mode > RT_MODE_STAGED) return rti::fail(RT_ERR_INVALID, "rt_trace_batch: unknown mode");
  if (b->n_items == 0) return rti::fail(RT_ERR_STATE, "rt_trace_batch: call rt_batch_set_items first");
  if (mode != RT_MODE_PLAIN)
    for (rt_scene* s : b->scenes)
      if (!s->has_treelets) return rti::fail(RT_ERR_STATE, "rt_trace_batch: a scene has no treelets");
  // scenes may have (re)formed their treelets since the views were uploaded
  bool stale = false;
  for (size_t i = 0; i < b->scenes.size(); ++i) {
    const rt_scene* s = b->scenes[i];
    const rtk::SceneView nv{reinterpret_cast<const uint4*>(s->d_blob), s->d_meta, s->d_route, s->n_units};
    const rtk::SceneView& ov = b->views[i];
    if (nv.blob != ov.blob || nv.meta != ov.meta || nv.route != ov.route || nv.n_units != ov.n_units) {
      b->views[i] = nv;
      stale = true;
    }
  }
  if (stale) {
    RT_CUDA(cudaSetDevice(b->ctx->device));
    RT_CUDA(cudaMemcpy(b->d_views, b->views.data(), sizeof(rtk::SceneView) * b->views.size(), cudaMemcpyHostToDevice));
  }
  a = rtk::TraceArgs{};
  a.scenes = b->d_views;
  a.item_begin = b->d_item_begin;
  a.item_scene = b->d_item_scene;
  a.n_items = b->n_items;
  a.rays = rays;
  a.flags = flags;
  a.default_flags = default_flags;
  a.n = b->n_rays;
  a.hits = hits;
  a.stats = b->d_stats;
  a.status = b->d_status;
  a.queue = b->d_queue;
  return RT_OK;
}

// A staged batch: each item runs its scene's own staged walk (the scene's
// pinned treelets in shared memory and its own tuning, without treelet
// queues, whose memory a scene grows on demand), one launch per item in
// order on `st`.  A CTA's shared memory holds one scene's treelets, so the
// items are not merged into one persistent launch as the other modes are.
// A staged batch runs each item as its scene's own staged launch (a CTA's
// shared memory holds one scene's pinned treelets).  The launches go to
// kBatchLanes side streams forked from `st` (and joined back), so that the
// launches of small items, whose persistent grids leave SMs free, run side by
// side: a scene's items all go to one lane, in item order, since they share
// the scene's ray counter and statistics.  The fork and join are recorded
// into a graph when `st` is being captured.
rt_status batch_staged(rt_batch* b, const rt_ray* rays, const uint32_t* flags, uint32_t default_flags, rt_hit* hits,
                       cudaStream_t st) {
  if (!b->ev_fork) {
    for (uint32_t j = 0; j < rt_batch::kBatchLanes; ++j) {
      RT_CUDA(cudaStreamCreateWithFlags(&b->lane[j], cudaStreamNonBlocking));
      RT_CUDA(cudaEventCreateWithFlags(&b->ev_join[j], cudaEventDisableTiming));
    }
    RT_CUDA(cudaEventCreateWithFlags(&b->ev_fork, cudaEventDisableTiming));
  }
  RT_CUDA(cudaEventRecord(b->ev_fork, st));
  for (uint32_t j = 0; j < rt_batch::kBatchLanes; ++j) RT_CUDA(cudaStreamWaitEvent(b->lane[j], b->ev_fork, 0));
  rt_status r = RT_OK;
  for (uint32_t k = 0; k < b->n_items && r == RT_OK; ++k) {
    const uint32_t lo = b->item_begin[k], m = b->item_begin[k + 1] - lo;
    if (m == 0) continue;
    rt_scene* s = b->scenes[b->item_scene[k]];
    r = check_trace(s, RT_MODE_STAGED, nullptr, "rt_trace_batch");
    if (r == RT_OK)
      r = trace_launch(s, rays + lo, flags ? flags + lo : nullptr, default_flags, m, RT_MODE_STAGED, hits + lo,
                       nullptr, b->lane[b->item_scene[k] % rt_batch::kBatchLanes], s->d_queue, false, false);
  }
  // join every lane back, also after a failure (a capture must end joined)
  for (uint32_t j = 0; j < rt_batch::kBatchLanes; ++j) {
    RT_CUDA(cudaEventRecord(b->ev_join[j], b->lane[j]));
    RT_CUDA(cudaStreamWaitEvent(st, b->ev_join[j], 0));
  }
  return r;
}

}  // namespace

extern "C" {

rt_status rt_batch_create(rt_ctx* ctx, rt_scene* const* scenes, uint32_t n_scenes, rt_batch** out) {
  if (!ctx || !scenes || !out || n_scenes == 0) return rti::fail(RT_ERR_INVALID, "rt_batch_create: bad argument");
  *out = nullptr;
  RT_CUDA(cudaSetDevice(ctx->device));
  auto* b = new rt_batch();
  b->ctx = ctx;
  b->scenes.assign(scenes, scenes + n_scenes);
  rt_status st = dalloc(&b->d_views, sizeof(rtk::SceneView) * n_scenes);
  if (st == RT_OK) st = dalloc(&b->d_stats, sizeof(unsigned long long) * rtk::ST_COUNT);
  if (st == RT_OK) st = dalloc(&b->d_status, sizeof(uint32_t));
  if (st == RT_OK) st = dalloc(&b->d_queue, sizeof(uint32_t));
  if (st != RT_OK) {
    rt_batch_destroy(b);
    return st;
  }
  std::vector<rtk::SceneView> v(n_scenes);
  for (uint32_t i = 0; i < n_scenes; ++i) {
    if (!scenes[i] || scenes[i]->ctx->device != ctx->device) {
      rt_batch_destroy(b);
      return rti::fail(RT_ERR_INVALID, "rt_batch_create: NULL scene or scene on another device");
    }
    v[i] = rtk::SceneView{reinterpret_cast<const uint4*>(scenes[i]->d_blob), scenes[i]->d_meta, scenes[i]->d_route,
                          scenes[i]->n_units};
  }
  cudaError_t e = cudaMemcpy(b->d_views, v.data(), sizeof(rtk::SceneView) * n_scenes, cudaMemcpyHostToDevice);
  b->views = v;
  if (e != cudaSuccess) {
    rt_batch_destroy(b);
    return cuda_fail(e, "rt_batch_create");
  }
  *out = b;
  return RT_OK;
}

rt_status rt_batch_destroy(rt_batch* b) {
  if (!b) return RT_OK;
  free_graph(b);
  for (uint32_t j = 0; j < rt_batch::kBatchLanes; ++j) {
    if (b->lane[j]) cudaStreamDestroy(b->lane[j]);
    if (b->ev_join[j]) cudaEventDestroy(b->ev_join[j]);
  }
  if (b->ev_fork) cudaEventDestroy(b->ev_fork);
  cudaFree(b->d_views);
  cudaFree(b->d_item_begin);
  cudaFree(b->d_item_scene);
  cudaFree(b->d_stats);
  cudaFree(b->d_status);
  cudaFree(b->d_queue);
  delete b;
  return RT_OK;
}

rt_status rt_batch_set_items(rt_batch* b, const uint32_t* ray_begin, const uint32_t* item_scene, uint32_t n_items) {
  if (!b || !ray_begin || !item_scene || n_items == 0) return rti::fail(RT_ERR_INVALID, "rt_batch_set_items: bad argument");
  for (uint32_t k = 0; k < n_items; ++k) {
    if (ray_begin[k + 1] < ray_begin[k]) return rti::fail(RT_ERR_INVALID, "rt_batch_set_items: ray_begin not ascending");
    if (item_scene[k] >= b->scenes.size()) return rti::fail(RT_ERR_INVALID, "rt_batch_set_items: scene index");
  }
  if (ray_begin[0] != 0) return rti::fail(RT_ERR_INVALID, "rt_batch_set_items: ray_begin[0] must be 0");
  RT_CUDA(cudaSetDevice(b->ctx->device));
  free_graph(b);
  cudaFree(b->d_item_begin);
  cudaFree(b->d_item_scene);
  b->d_item_begin = nullptr;
  b->d_item_scene = nullptr;
  rt_status st = dalloc(&b->d_item_begin, sizeof(uint32_t) * (n_items + 1));
  if (st == RT_OK) st = dalloc(&b->d_item_scene, sizeof(uint32_t) * n_items);
  if (st != RT_OK) return st;
  RT_CUDA(cudaMemcpy(b->d_item_begin, ray_begin, sizeof(uint32_t) * (n_items + 1), cudaMemcpyHostToDevice));
  RT_CUDA(cudaMemcpy(b->d_item_scene, item_scene, sizeof(uint32_t) * n_items, cudaMemcpyHostToDevice));
  b->n_items = n_items;
  b->n_rays = ray_begin[n_items];
  b->item_begin.assign(ray_begin, ray_begin + n_items + 1);
  b->item_scene.assign(item_scene, item_scene + n_items);
  return RT_OK;
}

rt_status rt_batch_set_tuning(rt_batch* b, const rt_tuning* t) {
  if (!b || !t || b->scenes.empty()) return rti::fail(RT_ERR_INVALID, "rt_batch_set_tuning: NULL");
  rt_tuning n;
  rt_status st = merge_tuning(b->tuning, t, n);
  if (st != RT_OK) return st;
  b->tuning = n;
  return RT_OK;
}

rt_status rt_trace_batch(rt_batch* b, const rt_ray* rays, const uint32_t* flags, uint32_t default_flags, uint32_t mode,
                         rt_hit* hits, void* stream) {
  if (!b) return rti::fail(RT_ERR_INVALID, "rt_trace_batch: NULL batch");
  rtk::TraceArgs a;
  rt_status st = batch_args(b, rays, flags, default_flags, mode, hits, a);
  if (st != RT_OK) return st;
  if (b->n_rays == 0) return RT_OK;
  RT_CUDA(cudaSetDevice(b->ctx->device));
  if (mode == RT_MODE_STAGED) return batch_staged(b, rays, flags, default_flags, hits, (cudaStream_t)stream);
  return launch_trace(a, mode, b->tuning, 0, (cudaStream_t)stream);
}

rt_status rt_batch_graph_capture(rt_batch* b, const rt_ray* rays, const uint32_t* flags, uint32_t default_flags,
                                 uint32_t mode, rt_hit* hits, void* stream) {
  if (!b) return rti::fail(RT_ERR_INVALID, "rt_batch_graph_capture: NULL batch");
  if (!stream) return rti::fail(RT_ERR_INVALID, "rt_batch_graph_capture: capture needs a non-default stream");
  rtk::TraceArgs a;
  rt_status st = batch_args(b, rays, flags, default_flags, mode, hits, a);
  if (st != RT_OK) return st;
  RT_CUDA(cudaSetDevice(b->ctx->device));
  free_graph(b);
  cudaStream_t s = (cudaStream_t)stream;
  if (mode == RT_MODE_STAGED) {
    // the staged kernels' shared-memory attributes and launch shapes are set
    // by one launch of the batch outside the capture
    st = batch_staged(b, rays, flags, default_flags, hits, s);
    if (st != RT_OK) return st;
    RT_CUDA(cudaStreamSynchronize(s));
  }
  RT_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
  st = mode == RT_MODE_STAGED ? batch_staged(b, rays, flags, default_flags, hits, s) : launch_trace(a, mode, b->tuning, 0, s);
  cudaGraph_t g = nullptr;
  const cudaError_t e = cudaStreamEndCapture(s, &g);
  if (st != RT_OK) {
    if (g) cudaGraphDestroy(g);
    return st;
  }
  if (e != cudaSuccess) return cuda_fail(e, "rt_batch_graph_capture: cudaStreamEndCapture");
  b->graph = g;
  RT_CUDA(cudaGraphInstantiate(&b->exec, b->graph, 0));
  return RT_OK;
}

rt_status rt_batch_graph_launch(rt_batch* b, void* stream) {
  if (!b || !b->exec) return rti::fail(RT_ERR_STATE, "rt_batch_graph_launch: no captured graph");
  RT_CUDA(cudaSetDevice(b->ctx->device));
  RT_CUDA(cudaGraphLaunch(b->exec, (cudaStream_t)stream));
  return RT_OK;
}

}  // extern "C"

// ------------------------------------------------------------ packed traces
namespace {

// Transactions each ray keeps in its trace row: min(n_visits, row capacity).
__global__ void trace_counts_kernel(const rt_hit* __restrict__ hits, uint32_t n, uint32_t cap,
                                    uint32_t* __restrict__ counts) {
  const uint32_t r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r < n) counts[r] = min(hits[r].n_visits, cap);
}

// Turns the block-local exclusive offsets of bin_scan_kernel into offsets
// within the chunk (in place) and writes the chunk's total.
__global__ void trace_offsets_kernel(uint32_t* __restrict__ off, const uint32_t* __restrict__ block_sum,
                                     const rt_hit* __restrict__ hits, uint32_t n, uint32_t cap,
                                     unsigned long long* __restrict__ total) {
  const uint32_t r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= n) return;
  const uint32_t o = block_sum[r / rtk::kBinScanItems] + off[r];
  off[r] = o;
  if (r == n - 1) *total = (unsigned long long)o + min(hits[r].n_visits, cap);
}

// One warp per ray: the ray's global offset (base + chunk offset) into
// `goff`, and the used prefix of its trace rows to its place in the packed
// staging arrays (NULL: not written).
__global__ void trace_pack_kernel(const uint32_t* __restrict__ vis_rows, const uint32_t* __restrict__ tl_rows,
                                  const uint32_t* __restrict__ off, uint32_t n, uint32_t cap, uint32_t chunk_total,
                                  unsigned long long base, unsigned long long* __restrict__ goff,
                                  uint32_t* __restrict__ vis, uint32_t* __restrict__ tl) {
  const uint32_t warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31u;
  const uint32_t warps = (gridDim.x * blockDim.x) >> 5;
  for (uint32_t r = warp; r < n; r += warps) {
    const uint32_t o = off[r];
    const uint32_t m = (r + 1 < n ? off[r + 1] : chunk_total) - o;
    if (lane == 0) goff[r] = base + o;
    const uint64_t row = (uint64_t)r * cap;
    for (uint32_t j = lane; j < m; j += 32) {
      if (vis) vis[o + j] = vis_rows[row + j];
      if (tl) tl[o + j] = tl_rows[row + j];
    }
  }
}

}  // namespace

// Chunks pipeline the call: the rays of every chunk go in on one stream;
// each chunk is traced, counted and scanned on one of two streams; the host
// waits for chunk c's total, queues its packing (into a device staging area)
// and copies on a third stream, and then queues chunk c + 1's trace, so that
// the copies of chunk c overlap the trace of chunk c + 1.
extern "C" rt_status rt_trace_host_packed(rt_scene* s, const rt_ray* rays, const uint32_t* flags,
                                          uint32_t default_flags, uint32_t n, uint32_t mode, uint32_t row_capacity,
                                          rt_hit* hits, uint64_t* offsets, uint32_t* visits, uint32_t* treelets,
                                          uint64_t capacity, uint64_t* total) {
  if (!s) return rti::fail(RT_ERR_INVALID, "rt_trace_host_packed: NULL scene");
  if (total) *total = 0;
  if (n == 0) {
    if (offsets) offsets[0] = 0;
    return RT_OK;
  }
  if (!rays || !hits || !offsets || !total) return rti::fail(RT_ERR_INVALID, "rt_trace_host_packed: NULL argument");
  if (row_capacity == 0 || (!visits && !treelets))
    return rti::fail(RT_ERR_INVALID, "rt_trace_host_packed: no trace asked for (row_capacity 0 or no arrays)");
  if ((uint64_t)n * row_capacity >= (1ull << 32))
    return rti::fail(RT_ERR_TOO_LARGE, "rt_trace_host_packed: rays x row_capacity must stay below 2^32");
  if ((uint64_t)n > (uint64_t)rtk::kBinScanItems * rtk::kBinScanItems)
    return rti::fail(RT_ERR_TOO_LARGE, "rt_trace_host_packed: at most 2^24 rays per call");
  // only the pointers' presence matters to the argument check
  uint32_t mark = 0;
  const rt_trace_buf probe{visits ? &mark : nullptr, treelets ? &mark : nullptr, row_capacity};
  rt_status st = check_trace(s, mode, &probe, "rt_trace_host_packed");
  if (st != RT_OK) return st;
  RT_CUDA(cudaSetDevice(s->ctx->device));
  const uint32_t cap = row_capacity;
  auto al = [](size_t b) { return (b + 255) & ~(size_t)255; };
  // four equal chunks from 2^19 rays on (a queued staged launch runs whole:
  // its queues are the scene's, one set)
  uint64_t bound[rti::kHostChunks + 1];
  uint32_t chunks = 1;
  bound[0] = 0;
  bound[1] = n;
  if (!queued(s, mode) && n >= (1u << 19)) {
    chunks = rti::kHostChunks;
    for (uint32_t c = 0; c <= chunks; ++c) bound[c] = (uint64_t)n * c / chunks;
  }
  const size_t b_rays = al(sizeof(rt_ray) * (size_t)n), b_flags = flags ? al(sizeof(uint32_t) * (size_t)n) : 0;
  const size_t b_hits = al(sizeof(rt_hit) * (size_t)n), b_row = al(sizeof(uint32_t) * (size_t)n * cap);
  const size_t b_cnt = al(sizeof(uint32_t) * (size_t)n);
  const size_t b_blk = al(sizeof(uint32_t) * rtk::kBinScanItems) * rti::kHostChunks;
  const size_t b_goff = al(sizeof(unsigned long long) * (size_t)n);
  const size_t b_tot = al(sizeof(unsigned long long) * rti::kHostChunks);
  const size_t need = b_rays + b_flags + b_hits + (visits ? b_row : 0) + (treelets ? b_row : 0) + 2 * b_cnt + b_blk +
                      b_goff + b_tot;
  if (need > s->io_bytes) {
    cudaFree(s->d_io);
    s->d_io = nullptr;
    s->io_bytes = 0;
    st = dalloc((uint8_t**)&s->d_io, need);
    if (st != RT_OK) return st;
    s->io_bytes = need;
  }
  if (!s->h_tot) {
    cudaError_t e = cudaHostAlloc(&s->h_tot, sizeof(unsigned long long) * rti::kHostChunks, cudaHostAllocDefault);
    if (e != cudaSuccess) {
      s->h_tot = nullptr;
      return cuda_fail(e, "rt_trace_host_packed: cudaHostAlloc");
    }
  }
  uint8_t* p = (uint8_t*)s->d_io;
  auto take = [&](size_t b) {
    uint8_t* r = p;
    p += b;
    return r;
  };
  rt_ray* d_rays = (rt_ray*)take(b_rays);
  uint32_t* d_flags = flags ? (uint32_t*)take(b_flags) : nullptr;
  rt_hit* d_hits = (rt_hit*)take(b_hits);
  uint32_t* d_vis = visits ? (uint32_t*)take(b_row) : nullptr;
  uint32_t* d_tl = treelets ? (uint32_t*)take(b_row) : nullptr;
  uint32_t* d_cnt = (uint32_t*)take(b_cnt);
  uint32_t* d_off = (uint32_t*)take(b_cnt);
  uint32_t* d_blk = (uint32_t*)take(b_blk);
  unsigned long long* d_goff = (unsigned long long*)take(b_goff);
  unsigned long long* d_tot = (unsigned long long*)take(b_tot);
  const size_t blk_stride = al(sizeof(uint32_t) * rtk::kBinScanItems) / sizeof(uint32_t);

  RT_CUDA(cudaMemsetAsync(s->d_stats, 0, sizeof(unsigned long long) * rtk::ST_COUNT, s->xin));
  RT_CUDA(cudaMemsetAsync(s->d_status, 0, sizeof(uint32_t), s->xin));
  cudaError_t e = cudaSuccess;
  // every chunk's rays in
  for (uint32_t c = 0; c < chunks && e == cudaSuccess; ++c) {
    const size_t lo = bound[c];
    const uint32_t m = (uint32_t)(bound[c + 1] - bound[c]);
    e = cudaMemcpyAsync(d_rays + lo, rays + lo, sizeof(rt_ray) * m, cudaMemcpyHostToDevice, s->xin);
    if (e == cudaSuccess && flags)
      e = cudaMemcpyAsync(d_flags + lo, flags + lo, sizeof(uint32_t) * m, cudaMemcpyHostToDevice, s->xin);
    if (e == cudaSuccess) e = cudaEventRecord(s->ev_in[c], s->xin);
  }
  // chunk c's trace, counts, offsets and total (copied to the page-locked
  // h_tot[c]), ending in ev_done[c]
  auto trace_chunk = [&](uint32_t c) -> bool {
    const size_t lo = bound[c];
    const uint32_t m = (uint32_t)(bound[c + 1] - bound[c]);
    cudaStream_t cs = (c & 1) ? s->stream2 : s->stream;
    e = cudaStreamWaitEvent(cs, s->ev_in[c], 0);
    if (e != cudaSuccess) return false;
    rt_trace_buf rows{d_vis ? d_vis + lo * cap : nullptr, d_tl ? d_tl + lo * cap : nullptr, cap};
    st = trace_launch(s, d_rays + lo, d_flags ? d_flags + lo : nullptr, default_flags, m, mode, d_hits + lo, &rows, cs,
                      s->d_queue + c, true);
    if (st != RT_OK) return false;
    const uint32_t nb = (m + rtk::kBinScanItems - 1) / rtk::kBinScanItems;
    uint32_t* blk = d_blk + c * blk_stride;
    trace_counts_kernel<<<(m + 255) / 256, 256, 0, cs>>>(d_hits + lo, m, cap, d_cnt + lo);
    rtk::bin_scan_kernel<<<nb, 1024, 0, cs>>>(d_cnt + lo, d_off + lo, blk, m);
    rtk::bin_scan_top_kernel<<<1, 1024, 0, cs>>>(blk, nb);
    trace_offsets_kernel<<<(m + 255) / 256, 256, 0, cs>>>(d_off + lo, blk, d_hits + lo, m, cap, d_tot + c);
    e = cudaGetLastError();
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(s->h_tot + c, d_tot + c, sizeof(unsigned long long), cudaMemcpyDeviceToHost, cs);
    if (e == cudaSuccess) e = cudaEventRecord(s->ev_done[c], cs);
    return e == cudaSuccess;
  };
  // In chunk order: wait for chunk c's total, queue its packing and copies,
  // then queue chunk c + 1's trace, so that the GPU runs the short pack
  // kernel before the next persistent trace fills the SMs and the copies
  // overlap that trace.
  unsigned long long base = 0;
  bool fits = true;
  if (e == cudaSuccess) trace_chunk(0);
  for (uint32_t c = 0; c < chunks && e == cudaSuccess && st == RT_OK; ++c) {
    const size_t lo = bound[c];
    const uint32_t m = (uint32_t)(bound[c + 1] - bound[c]);
    e = cudaEventSynchronize(s->ev_done[c]);
    if (e != cudaSuccess) break;
    const unsigned long long tot_c = reinterpret_cast<volatile unsigned long long*>(s->h_tot)[c];
    fits = fits && base + tot_c <= capacity;
    uint32_t *dst_vis = nullptr, *dst_tl = nullptr;
    if (fits && tot_c > 0) {
      // one staging area for the packed entries of one chunk: the pack and
      // copy of chunk c follow chunk c-1's on the same stream
      const size_t b_pack = al(sizeof(uint32_t) * (size_t)tot_c);
      const size_t pack_need = (visits ? b_pack : 0) + (treelets ? b_pack : 0);
      if (pack_need > s->pack_bytes) {
        e = cudaStreamSynchronize(s->xout);
        if (e != cudaSuccess) break;
        cudaFree(s->d_pack);
        s->d_pack = nullptr;
        s->pack_bytes = 0;
        st = dalloc((uint8_t**)&s->d_pack, pack_need + pack_need / 4);
        if (st != RT_OK) break;
        s->pack_bytes = pack_need + pack_need / 4;
      }
      dst_vis = visits ? (uint32_t*)s->d_pack : nullptr;
      dst_tl = treelets ? (uint32_t*)((uint8_t*)s->d_pack + (visits ? b_pack : 0)) : nullptr;
    }
    e = cudaStreamWaitEvent(s->xout, s->ev_done[c], 0);
    if (e != cudaSuccess) break;
    unsigned long long* goff = d_goff + lo;
    trace_pack_kernel<<<std::min<uint32_t>((m + 3) / 4, 152 * 8), 128, 0, s->xout>>>(
        d_vis ? d_vis + lo * cap : nullptr, d_tl ? d_tl + lo * cap : nullptr, d_off + lo, m, cap, (uint32_t)tot_c, base,
        goff, dst_vis, dst_tl);
    e = cudaGetLastError();
    if (e == cudaSuccess && c + 1 < chunks && !trace_chunk(c + 1)) break;
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(hits + lo, d_hits + lo, sizeof(rt_hit) * m, cudaMemcpyDeviceToHost, s->xout);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(offsets + lo, d_goff + lo, sizeof(unsigned long long) * m, cudaMemcpyDeviceToHost, s->xout);
    if (dst_vis && e == cudaSuccess)
      e = cudaMemcpyAsync(visits + base, dst_vis, sizeof(uint32_t) * tot_c, cudaMemcpyDeviceToHost, s->xout);
    if (dst_tl && e == cudaSuccess)
      e = cudaMemcpyAsync(treelets + base, dst_tl, sizeof(uint32_t) * tot_c, cudaMemcpyDeviceToHost, s->xout);
    base += tot_c;
  }
  if (st == RT_OK && e != cudaSuccess) st = cuda_fail(e, "rt_trace_host_packed");
  st = host_finish(s, st);
  if (st != RT_OK) return st;
  offsets[n] = base;
  *total = base;
  if (base > capacity)
    return rti::fail(RT_ERR_TOO_LARGE, "rt_trace_host_packed: " + std::to_string(base) +
                                           " trace entries exceed the arrays' capacity (hits and offsets are filled)");
  return RT_OK;
}
