// Runs three more pieces of the REFERENCE's RT-unit model on batches of cases
// and writes what they did: the golden data the replay's warp selection,
// stride prefetcher and prefetch tally are pinned against.
//
//  - rt_unit::schedule_next_warp (src/gpgpu-sim/shader.cc:4307-4392): which
//    resident warp the RT unit serves next, under the OMR (1), PMR (2) or
//    oldest-first (0) rule, over treelets formed by the reference's own
//    createTreelets.
//  - the Lee MICRO'10 stride prefetcher of rt_unit::memory_cycle
//    (shader.cc:4779-4828): the removal of queued prefetches of a demand
//    address, then the per-warp stride training and the two queued prefetches.
//  - the end-of-run tally of each RT unit's prefetch records into the
//    effectiveness classes (src/gpgpu-sim/gpu-sim.cc:1749-1795), with the
//    record struct prefetch_block_info (gpu-cache.h:99-131) and its class enum
//    (abstract_hardware_model.h:247-254).
//
// The reference code is not copied here.  The Makefile in this folder extracts
// the ranges, unmodified, into oracle/_ref/extract/ (rt_schedule.inc: the
// definition of rt_unit::schedule_next_warp; rt_lee.inc: the two blocks;
// rt_effect.inc, rt_blockinfo.inc, rt_tally.inc) and this file compiles them
// against its own stand-in classes `rt_unit` and TallyGpu, whose members
// carry the names the code uses.
//
// Usage:
//   pin_rtunit schedule <blob file> <max bytes per treelet> <cases file> <out file>
//     cases (uint32 words), per case: scheduler, treelet_prefetch,
//     last_prefetched (root unit or 0xFFFFFFFF), n_warps, then per warp (in
//     increasing uid order): uid, stalled, 32 next-access units (0xFFFFFFFF =
//     no pending access).
//     out (uint64 words), per case: the chosen warp's uid (~0 for none), the
//     number of warps left resident.
//   pin_rtunit stride <events file> <max_queue> <prefill> <out file>
//     The queue starts with `prefill` entries (request = base = 32 (i + 1)).
//     events (uint32 words), per event: warp id, pops, next_addr low, high.
//     `pops` entries leave the queue front first (issued prefetches).
//     out (uint64 words), per event: removed, appended, per appended entry
//     (request, base), queue length.
//   pin_rtunit tally <records file> <out file>
//     records (uint32 words): n_clusters, then per cluster: n_records, then
//     per record: block address low, high, class (0-5).
//     out (uint64 words): unclassified_but_accessed, the five class totals,
//     then the per-cluster counts, class-major (cluster i, class c at
//     i + c n_clusters).
#include "treelet_env.h"

#define RT_SCHEDULER_DPRINTF(...)

#include "rt_effect.inc"
#include "rt_blockinfo.inc"

// ---- the warp instruction, as far as the scheduler and the prefetcher see it
struct RTMemoryTransactionRecordStandIn {
  new_addr_type address;
};
struct ThreadInfoStandIn {
  std::deque<RTMemoryTransactionRecordStandIn> RT_mem_accesses;
};
class warp_inst_t {
 public:
  bool m_empty = true;
  unsigned m_uid = 0;
  unsigned m_warp_id = 0;
  bool m_stalled = false;
  ThreadInfoStandIn m_threads[32];

  bool empty() const { return m_empty; }
  unsigned get_uid() const { return m_uid; }
  unsigned get_warp_id() const { return m_warp_id; }
  bool is_stalled() const { return m_stalled; }
  const ThreadInfoStandIn& get_thread_info(int i) const { return m_threads[i]; }
};

class rt_unit {
 public:
  const pin::ShaderConfig* m_config = &pin::g_core.cfg;
  pin::Core* m_core = &pin::g_core;
  unsigned m_sid = 0;
  std::map<unsigned, warp_inst_t> m_current_warps;
  uint8_t* last_prefetched_treelet = NULL;
  std::deque<std::pair<new_addr_type, new_addr_type>> prefetch_mem_access_q;
  std::deque<std::pair<unsigned long long, new_addr_type>> prefetch_generation_cycles;
  std::map<unsigned, std::map<int, unsigned>> pws_table;
  std::map<unsigned, new_addr_type> pws_last_accessed_addr;
  unsigned prefetches_removed_from_queue = 0;
  unsigned prefetches_added_to_queue = 0;
  std::map<new_addr_type, std::vector<prefetch_block_info>> prefetch_request_tracker;

  void schedule_next_warp(warp_inst_t& inst);

  void stride_demand(warp_inst_t& inst, new_addr_type next_addr) {
#include "rt_lee.inc"
  }
};

#include "rt_schedule.inc"

// ---- the GPU, as far as the end-of-run tally sees it
struct TallyCore {
  rt_unit unit;
  rt_unit* get_m_rt_unit() { return &unit; }
};
struct TallyCluster {
  TallyCore core;
  TallyCore* cores[1] = {&core};
  TallyCore** get_m_core() { return cores; }
};
struct TallyConfig {
  unsigned n_clusters = 0;
  unsigned num_cluster() const { return n_clusters; }
};
class TallyGpu {
 public:
  TallyConfig m_config;
  std::vector<TallyCluster*> m_cluster;
  unsigned out_unclassified_but_accessed = 0;
  std::vector<unsigned> out_total, out_per_cluster;

  void tally() {
#include "rt_tally.inc"
    out_unclassified_but_accessed = unclassified_but_accessed;
    out_total = total_prefetch_effectiveness;
    out_per_cluster = prefetch_effectiveness_per_cluster;
  }
};

namespace {

int run_schedule(int argc, char** argv) {
  if (argc != 6) return 2;
  const std::vector<uint8_t> raw = read_file(argv[4]);
  if (!load_scene(argv[2], atoi(argv[3])) || raw.size() % 4) return 2;
  std::vector<uint32_t> w(raw.size() / 4);
  memcpy(w.data(), raw.data(), raw.size());
  std::vector<uint64_t> out;
  size_t i = 0;
  while (i < w.size()) {
    if (i + 4 > w.size()) return 2;
    pin::ShaderConfig& cfg = pin::g_core.cfg;
    cfg.m_treelet_scheduler = w[i];
    cfg.m_treelet_prefetch = w[i + 1] != 0;
    rt_unit unit;
    unit.last_prefetched_treelet = addr_of(w[i + 2]);
    const uint32_t n_warps = w[i + 3];
    i += 4;
    if (i + (size_t)n_warps * 34 > w.size()) return 2;
    for (uint32_t k = 0; k < n_warps; ++k, i += 34) {
      warp_inst_t& warp = unit.m_current_warps[w[i]];
      warp.m_empty = false;
      warp.m_uid = w[i];
      warp.m_warp_id = k;
      warp.m_stalled = w[i + 1] != 0;
      for (int l = 0; l < 32; ++l)
        if (w[i + 2 + l] != 0xFFFFFFFFu)
          warp.m_threads[l].RT_mem_accesses.push_back({(new_addr_type)(uintptr_t)addr_of(w[i + 2 + l])});
    }
    warp_inst_t chosen;
    unit.schedule_next_warp(chosen);
    out.push_back(chosen.empty() ? ~0ull : (uint64_t)chosen.get_uid());
    out.push_back(unit.m_current_warps.size());
  }
  FILE* f = fopen(argv[5], "wb");
  if (!f) return 2;
  fwrite(out.data(), sizeof(uint64_t), out.size(), f);
  fclose(f);
  return 0;
}

int run_stride(int argc, char** argv) {
  if (argc != 6) return 2;
  const std::vector<uint8_t> raw = read_file(argv[2]);
  if (raw.size() % 16) return 2;
  std::vector<uint32_t> w(raw.size() / 4);
  memcpy(w.data(), raw.data(), raw.size());
  pin::g_core.cfg.m_lee_micro_prefetcher = true;
  pin::g_core.cfg.m_max_prefetch_queue_size = (unsigned)atoi(argv[3]);
  rt_unit unit;
  for (int k = 0, prefill = atoi(argv[4]); k < prefill; ++k) {
    const new_addr_type a = 32ull * (k + 1);
    unit.prefetch_mem_access_q.push_back({a, a});
    unit.prefetch_generation_cycles.push_back({0, a});
  }
  std::vector<uint64_t> out;
  for (size_t i = 0; i < w.size(); i += 4) {
    for (uint32_t p = 0; p < w[i + 1] && !unit.prefetch_mem_access_q.empty(); ++p) {
      unit.prefetch_mem_access_q.pop_front();
      unit.prefetch_generation_cycles.pop_front();
    }
    warp_inst_t inst;
    inst.m_empty = false;
    inst.m_warp_id = w[i];
    const new_addr_type next_addr = (new_addr_type)w[i + 2] | ((new_addr_type)w[i + 3] << 32);
    const unsigned removed0 = unit.prefetches_removed_from_queue;
    const size_t len0 = unit.prefetch_mem_access_q.size();
    unit.stride_demand(inst, next_addr);
    const uint64_t removed = unit.prefetches_removed_from_queue - removed0;
    const size_t first_new = len0 - removed;
    out.push_back(removed);
    out.push_back(unit.prefetch_mem_access_q.size() - first_new);
    for (size_t q = first_new; q < unit.prefetch_mem_access_q.size(); ++q) {
      out.push_back(unit.prefetch_mem_access_q[q].first);
      out.push_back(unit.prefetch_mem_access_q[q].second);
    }
    out.push_back(unit.prefetch_mem_access_q.size());
  }
  FILE* f = fopen(argv[5], "wb");
  if (!f) return 2;
  fwrite(out.data(), sizeof(uint64_t), out.size(), f);
  fclose(f);
  return 0;
}

int run_tally(int argc, char** argv) {
  if (argc != 4) return 2;
  const std::vector<uint8_t> raw = read_file(argv[2]);
  if (raw.size() % 4 || raw.empty()) return 2;
  std::vector<uint32_t> w(raw.size() / 4);
  memcpy(w.data(), raw.data(), raw.size());
  TallyGpu gpu;
  gpu.m_config.n_clusters = w[0];
  std::vector<TallyCluster> clusters(w[0]);
  size_t i = 1;
  for (auto& c : clusters) {
    gpu.m_cluster.push_back(&c);
    if (i >= w.size()) return 2;
    const uint32_t n = w[i++];
    if (i + (size_t)n * 3 > w.size()) return 2;
    for (uint32_t k = 0; k < n; ++k, i += 3) {
      prefetch_block_info info;
      info.m_block_addr = (new_addr_type)w[i] | ((new_addr_type)w[i + 1] << 32);
      info.effectiveness = (prefetch_request_effectiveness)w[i + 2];
      c.core.unit.prefetch_request_tracker[info.m_block_addr].push_back(info);
    }
  }
  gpu.tally();
  std::vector<uint64_t> out;
  out.push_back(gpu.out_unclassified_but_accessed);
  for (unsigned v : gpu.out_total) out.push_back(v);
  for (unsigned v : gpu.out_per_cluster) out.push_back(v);
  FILE* f = fopen(argv[3], "wb");
  if (!f) return 2;
  fwrite(out.data(), sizeof(uint64_t), out.size(), f);
  fclose(f);
  return 0;
}

}  // namespace

int main(int argc, char** argv) {
  if (argc >= 2 && strcmp(argv[1], "schedule") == 0) return run_schedule(argc, argv);
  if (argc >= 2 && strcmp(argv[1], "stride") == 0) return run_stride(argc, argv);
  if (argc >= 2 && strcmp(argv[1], "tally") == 0) return run_tally(argc, argv);
  fprintf(stderr,
          "usage: pin_rtunit schedule <blob> <max bytes per treelet> <cases> <out>\n"
          "       pin_rtunit stride <events> <max_queue> <prefill> <out>\n"
          "       pin_rtunit tally <records> <out>\n");
  return 2;
}
