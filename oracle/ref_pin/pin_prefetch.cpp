// Runs the REFERENCE's own treelet-prefetch decision of the RT unit
// (src/gpgpu-sim/shader.cc:3419-3685, the decision block of rt_unit::cycle)
// on a batch of cases and writes what it queued: the golden data the
// oracle's prefetch decision is pinned against.
//
// The reference code is not copied here.  The Makefile in this folder
// extracts the block, unmodified, into oracle/_ref/extract/pf_decide.inc and
// this file compiles it as the body of a member function of its own stand-in
// for the RT unit, whose members carry the names the block uses (the
// configuration, the resident warps with each thread's pending accesses, the
// prefetch queue and the last-prefetched / last-rejected treelets).  The
// treelet maps come from the reference's own createTreelets
// (tl_maps.inc, tl_create.inc, as for pin_treelets).
//
// Usage: pin_prefetch <blob file> <max bytes per treelet> <cases file> <out file>
//                     [<queue variant> <flush>]
// queue variant 1 runs the pipelined treelet queue's copy of the decision
// (shader.cc:3780-3932, extracted into pf_decide_queue.inc) instead, variant 2
// the treelet queue's copy (shader.cc:4020-4060, pf_decide_tq.inc); flush 1
// sets -flush_prefetch_queue_on_new_treelet.
// cases file (uint32 words), per case: heuristic, max_queue, threshold as a
// float's bits, second_prefetch, last_prefetched, last_prefetched_second,
// last_rejected (root units or 0xFFFFFFFF), queue_len, lanes, then `lanes`
// next-access units (0xFFFFFFFF = idle lane).  Lane k is thread k % 32 of
// resident warp k / 32.
// out file (uint64 words), per case: the number of queue entries the decision
// appended, then per entry (chunk address - blob, base node unit); then the
// last_prefetched, last_prefetched_second and last_rejected root units
// (0xFFFFFFFF for none) and the queue length after the decision.
#include "treelet_env.h"

// ---- the RT unit, as far as the decision block sees it
struct PendingAccess {
  new_addr_type address;
};
struct ThreadAccesses {
  std::deque<PendingAccess> RT_mem_accesses;
};
struct ResidentWarp {
  ThreadAccesses threads[32];
  const ThreadAccesses& get_thread_info(int i) const { return threads[i]; }
};

class RtUnitStandIn {
 public:
  const pin::ShaderConfig* m_config = &pin::g_core.cfg;
  pin::Core* m_core = &pin::g_core;
  unsigned m_sid = 0;
  std::map<unsigned, ResidentWarp> m_current_warps;
  std::deque<std::pair<new_addr_type, new_addr_type>> prefetch_mem_access_q;
  std::deque<std::pair<unsigned, new_addr_type>> prefetch_generation_cycles;
  uint8_t* last_prefetched_treelet = NULL;
  uint8_t* last_prefetched_second_treelet = NULL;
  uint8_t* last_rejected_treelet = NULL;
  unsigned prefetch_treelet_switches = 0;
  unsigned timestamp_of_last_treelet = 0;
  unsigned total_cycles_between_prefetch_treelet_switch = 0;
  unsigned prefetches_added_to_queue = 0;
  unsigned prefetch_metadata_added = 0;
  unsigned matches = 0;
  unsigned comparisons = 0;

  bool executing = true;  // the pipelined treelet queue is dispatching its warps

  void decide() {
#include "pf_decide.inc"
  }
  void decide_queue() {
#include "pf_decide_queue.inc"
  }
  void decide_treelet_queue() {
#include "pf_decide_tq.inc"
  }
};

int main(int argc, char** argv) {
  if (argc != 5 && argc != 7) {
    fprintf(stderr, "usage: pin_prefetch <blob> <max bytes per treelet> <cases> <out> [<queue variant> <flush>]\n");
    return 2;
  }
  const int queue_variant = argc == 7 ? atoi(argv[5]) : 0;
  pin::g_core.cfg.m_flush_prefetch_queue_on_new_treelet = argc == 7 && atoi(argv[6]) != 0;
  const std::vector<uint8_t> raw = read_file(argv[3]);
  if (!load_scene(argv[1], atoi(argv[2])) || raw.size() % 4) return 2;
  std::vector<uint32_t> w(raw.size() / 4);
  memcpy(w.data(), raw.data(), raw.size());

  std::vector<uint64_t> out;
  size_t i = 0;
  while (i < w.size()) {
    if (i + 9 > w.size()) return 2;
    pin::ShaderConfig& cfg = pin::g_core.cfg;
    cfg.m_treelet_prefetch_heuristic = (int)w[i];
    cfg.m_max_prefetch_queue_size = w[i + 1];
    float thr;
    memcpy(&thr, &w[i + 2], 4);
    cfg.m_treelet_prefetch_threshold = thr;
    cfg.prefetch_next_treelet_when_queue_empty = w[i + 3] != 0;
    RtUnitStandIn unit;
    unit.last_prefetched_treelet = addr_of(w[i + 4]);
    unit.last_prefetched_second_treelet = addr_of(w[i + 5]);
    unit.last_rejected_treelet = addr_of(w[i + 6]);
    const uint32_t queue_len = w[i + 7], lanes = w[i + 8];
    i += 9;
    if (i + lanes > w.size()) return 2;
    for (uint32_t q = 0; q < queue_len; ++q) unit.prefetch_mem_access_q.push_back({0, 0});
    for (uint32_t k = 0; k < lanes; ++k) {
      ResidentWarp& warp = unit.m_current_warps[k / 32];
      if (w[i + k] != 0xFFFFFFFFu)
        warp.threads[k % 32].RT_mem_accesses.push_back({(new_addr_type)(uintptr_t)addr_of(w[i + k])});
    }
    i += lanes;
    if (queue_variant == 2)
      unit.decide_treelet_queue();
    else if (queue_variant == 1)
      unit.decide_queue();
    else
      unit.decide();
    // the carried entries are (0, 0) and stay at the front unless a flush cleared them
    size_t keep = 0;
    while (keep < unit.prefetch_mem_access_q.size() && unit.prefetch_mem_access_q[keep].first == 0 &&
           unit.prefetch_mem_access_q[keep].second == 0)
      ++keep;
    out.push_back(unit.prefetch_mem_access_q.size() - keep);
    for (size_t q = keep; q < unit.prefetch_mem_access_q.size(); ++q) {
      out.push_back(unit.prefetch_mem_access_q[q].first - (new_addr_type)(uintptr_t)g_blob.data());
      out.push_back((unit.prefetch_mem_access_q[q].second - (new_addr_type)(uintptr_t)g_blob.data()) / 64);
    }
    out.push_back(unit_of(unit.last_prefetched_treelet));
    out.push_back(unit_of(unit.last_prefetched_second_treelet));
    out.push_back(unit_of(unit.last_rejected_treelet));
    out.push_back(unit.prefetch_mem_access_q.size());
  }
  FILE* f = fopen(argv[4], "wb");
  if (!f) return 2;
  fwrite(out.data(), sizeof(uint64_t), out.size(), f);
  fclose(f);
  return 0;
}
