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
// cases file (uint32 words), per case: heuristic, max_queue, threshold as a
// float's bits, second_prefetch, last_prefetched, last_prefetched_second,
// last_rejected (root units or 0xFFFFFFFF), queue_len, lanes, then `lanes`
// next-access units (0xFFFFFFFF = idle lane).  Lane k is thread k % 32 of
// resident warp k / 32.
// out file (uint64 words), per case: the number of queue entries the decision
// appended, then per entry (chunk address - blob, base node unit); then the
// last_prefetched, last_prefetched_second and last_rejected root units
// (0xFFFFFFFF for none) and the queue length after the decision.
#include <cassert>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <deque>
#include <iostream>
#include <map>
#include <string>
#include <utility>
#include <vector>
#include <vector_types.h>

#include "vulkan_acceleration_structure_util.h"

typedef void* VkAccelerationStructureKHR;
typedef unsigned long long new_addr_type;
#define TOMMY_DPRINTF(...)
#define SECOND_PREFETCH_DPRINTF(...)

#include "geom_ray.inc"
#include "tl_stackentry.inc"

namespace pin {
struct ShaderConfig {
  // read by createTreelets
  bool remap_to_treelet_layout = false;
  uint64_t treelet_remap_stride = 0;
  // read by the decision block
  bool m_treelet_prefetch = true;
  unsigned prefetch_delay = 1;
  int m_treelet_prefetch_heuristic = 0;
  double m_treelet_prefetch_threshold = 0.5;
  unsigned m_max_prefetch_queue_size = 0;
  bool m_flush_prefetch_queue_on_new_treelet = false;
  bool load_treelet_metadata = false;
  bool prefetch_next_treelet_when_queue_empty = false;
};
struct Core;
struct Cluster {
  Core* core;
  Core* cores[1];
  Core** get_m_core() { return cores; }
};
struct GpuConfig {
  uint64_t max_treelet_size = 0;
};
struct Gpu {
  Cluster cluster;
  Cluster* clusters[1] = {&cluster};
  GpuConfig cfg;
  unsigned long long gpu_sim_cycle = 0, gpu_tot_sim_cycle = 0;
  Cluster** get_m_cluster() { return clusters; }
  const GpuConfig& get_config() const { return cfg; }
};
struct Core {
  ShaderConfig cfg;
  Gpu* gpu;
  const ShaderConfig* get_config() const { return &cfg; }
  Gpu* get_gpu() { return gpu; }
};
struct Sim {
  Gpu* g_the_gpu;
};
struct Context {
  Sim* the_gpgpusim;
};
Gpu g_gpu;
Core g_core{{}, &g_gpu};
Sim g_sim{&g_gpu};
Context g_ctx{&g_sim};
uint8_t* g_layout_base = reinterpret_cast<uint8_t*>(uintptr_t(1) << 40);
}  // namespace pin

pin::Context* GPGPU_Context() { return &pin::g_ctx; }
void* gpgpusim_malloc(size_t) { return pin::g_layout_base; }

struct VulkanRayTracing {
  static std::map<void*, void*> blas_addr_map;
  static std::map<StackEntry, std::vector<StackEntry>> treelet_roots;
  static std::map<uint8_t*, std::vector<StackEntry>> treelet_roots_addr_only;
  static std::map<StackEntry, std::vector<StackEntry>> treelet_child_map;
  static std::map<uint8_t*, std::vector<StackEntry>> treelet_addr_only_child_map;
  static std::map<uint8_t*, uint8_t*> node_map_addr_only;
  static std::map<uint8_t*, uint8_t*> original_bvh_to_treelet_bvh_mapping;
  static std::map<uint8_t*, unsigned> treelet_addr_to_metadata_idx;
  static uint8_t* treelet_layout_bvh;
  static void* treelet_metadata;
  static unsigned per_treelet_metadata_size;

  static bool isTreeletRoot(StackEntry node);
  static bool isTreeletRoot(uint8_t* addr);
  static uint8_t* addrToTreeletID(uint8_t* addr);
  static void buildNodeToRootMap();
  static std::vector<StackEntry> treeletIDToChildren(StackEntry treelet_root);
  static std::vector<StackEntry> treeletIDToChildren(uint8_t* treelet_root);
  static float calculateSAH(float3 lo, float3 hi);
  static void createTreelets(VkAccelerationStructureKHR _topLevelAS, int64_t device_offset, int maxBytesPerTreelet);
  static void remapBVHToTreeletLayout();
};

std::map<void*, void*> VulkanRayTracing::blas_addr_map;
std::map<StackEntry, std::vector<StackEntry>> VulkanRayTracing::treelet_roots;
std::map<uint8_t*, std::vector<StackEntry>> VulkanRayTracing::treelet_roots_addr_only;
std::map<StackEntry, std::vector<StackEntry>> VulkanRayTracing::treelet_child_map;
std::map<uint8_t*, std::vector<StackEntry>> VulkanRayTracing::treelet_addr_only_child_map;
std::map<uint8_t*, uint8_t*> VulkanRayTracing::node_map_addr_only;
std::map<uint8_t*, uint8_t*> VulkanRayTracing::original_bvh_to_treelet_bvh_mapping;
std::map<uint8_t*, unsigned> VulkanRayTracing::treelet_addr_to_metadata_idx;
uint8_t* VulkanRayTracing::treelet_layout_bvh = nullptr;
void* VulkanRayTracing::treelet_metadata = nullptr;
unsigned VulkanRayTracing::per_treelet_metadata_size = 0;

#include "tl_maps.inc"
#include "tl_create.inc"

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

  void decide() {
#include "pf_decide.inc"
  }
};

namespace {

std::vector<uint8_t> g_blob;

void find_blases(uint64_t off) {
  GEN_RT_BVH_INTERNAL_NODE n;
  GEN_RT_BVH_INTERNAL_NODE_unpack(&n, g_blob.data() + off);
  uint64_t child = off + (int64_t)n.ChildOffset * 64;
  for (int i = 0; i < 6; ++i) {
    if (n.ChildSize[i] > 0) {
      if (n.ChildType[i] == NODE_TYPE_INTERNAL) {
        find_blases(child);
      } else {
        GEN_RT_BVH_INSTANCE_LEAF leaf;
        GEN_RT_BVH_INSTANCE_LEAF_unpack(&leaf, g_blob.data() + child);
        void* blas = g_blob.data() + child + leaf.BVHAddress;
        VulkanRayTracing::blas_addr_map[blas] = blas;
      }
    }
    child += (uint64_t)n.ChildSize[i] * 64;
  }
}

std::vector<uint8_t> read_file(const char* path) {
  std::vector<uint8_t> v;
  FILE* f = fopen(path, "rb");
  if (!f) return v;
  fseek(f, 0, SEEK_END);
  v.resize((size_t)ftell(f));
  fseek(f, 0, SEEK_SET);
  if (fread(v.data(), 1, v.size(), f) != v.size()) v.clear();
  fclose(f);
  return v;
}

uint8_t* addr_of(uint32_t unit) { return unit == 0xFFFFFFFFu ? nullptr : g_blob.data() + (uint64_t)unit * 64; }
uint64_t unit_of(const uint8_t* a) { return a ? (uint64_t)(a - g_blob.data()) / 64 : 0xFFFFFFFFull; }

}  // namespace

int main(int argc, char** argv) {
  if (argc != 5) {
    fprintf(stderr, "usage: pin_prefetch <blob> <max bytes per treelet> <cases> <out>\n");
    return 2;
  }
  g_blob = read_file(argv[1]);
  const int budget = atoi(argv[2]);
  const std::vector<uint8_t> raw = read_file(argv[3]);
  if (g_blob.empty() || raw.size() % 4) return 2;
  std::vector<uint32_t> w(raw.size() / 4);
  memcpy(w.data(), raw.data(), raw.size());
  pin::g_gpu.cluster.core = &pin::g_core;
  pin::g_gpu.cluster.cores[0] = &pin::g_core;
  pin::g_gpu.cfg.max_treelet_size = (uint64_t)budget;
  GEN_RT_BVH top;
  GEN_RT_BVH_unpack(&top, g_blob.data());
  find_blases(top.RootNodeOffset);
  std::cout.setstate(std::ios::failbit);
  VulkanRayTracing::createTreelets((VkAccelerationStructureKHR)g_blob.data(), 0, budget);

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
    unit.decide();
    out.push_back(unit.prefetch_mem_access_q.size() - queue_len);
    for (size_t q = queue_len; q < unit.prefetch_mem_access_q.size(); ++q) {
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
