// Forms treelets with the REFERENCE's own createTreelets / buildNodeToRootMap
// / remapBVHToTreeletLayout and writes the partition, the node->root map and
// the remapped addresses: the golden data the oracle's partition is pinned
// against.
//
// The reference functions are not copied here.  The Makefile in this folder
// extracts them, unmodified, into oracle/_ref/extract/ (git-ignored):
//   geom_ray.inc         struct Ray               src/abstract_hardware_model.h:333-370
//   tl_stackentry.inc    struct StackEntry        src/cuda-sim/vulkan_ray_tracing.h:180-208
//   tl_maps.inc          isTreeletRoot .. calculateSAH      src/cuda-sim/vulkan_ray_tracing.cc:456-510
//   tl_create.inc        createTreelets, remapBVHToTreeletLayout
//                                                 src/cuda-sim/vulkan_ray_tracing.cc:823-1509
// What they use of the rest of the simulator is declared below in this
// file's own code: the VulkanRayTracing class with the static members the
// functions read and write, and a configuration stand-in for the
// GPGPU_Context() chain (remap_to_treelet_layout off, so createTreelets leaves
// the maps in original addresses; remapBVHToTreeletLayout is called
// separately, with the given stride).
//
// One address space, as the oracle models it: device_offset = 0 and every
// BLAS is its own device address (blas_addr_map[a] = a).
//
// Usage: pin_treelets <blob file> <max bytes per treelet> <remap stride> <out file>
// Output (uint64 words) in <out file>: n_roots, then per root (ascending
// address): root unit, member count, member units in member-list order; then
// n_map and (node unit, root unit) pairs of node_map_addr_only; then n_meta and
// (root unit, metadata index) pairs of treelet_addr_to_metadata_idx.  In
// <out file>.remap: n_remap and (node unit, remapped offset from the layout
// base) pairs.
#include <cassert>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <deque>
#include <iostream>
#include <map>
#include <string>
#include <vector>
#include <vector_types.h>

#include "vulkan_acceleration_structure_util.h"

typedef void* VkAccelerationStructureKHR;

#include "geom_ray.inc"
#include "tl_stackentry.inc"

// ---- configuration stand-in for GPGPU_Context()->the_gpgpusim->g_the_gpu
namespace pin {
struct ShaderConfig {
  bool remap_to_treelet_layout = false;
  uint64_t treelet_remap_stride = 0;
};
struct Core {
  ShaderConfig cfg;
  const ShaderConfig* get_config() const { return &cfg; }
};
struct Cluster {
  Core core;
  Core* cores[1] = {&core};
  Core** get_m_core() { return cores; }
};
struct GpuConfig {
  uint64_t max_treelet_size = 0;
};
struct Gpu {
  Cluster cluster;
  Cluster* clusters[1] = {&cluster};
  GpuConfig cfg;
  Cluster** get_m_cluster() { return clusters; }
  const GpuConfig& get_config() const { return cfg; }
};
struct Sim {
  Gpu* g_the_gpu;
};
struct Context {
  Sim* the_gpgpusim;
};
Gpu g_gpu;
Sim g_sim{&g_gpu};
Context g_ctx{&g_sim};
// the remapped layout's base: an address of its own, never dereferenced
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

#include "tl_maps.inc"
#include "tl_create.inc"

namespace {

std::vector<uint8_t> g_blob;

// Every BLAS header an instance leaf of the TLAS names (one address space).
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

uint64_t unit_of(const uint8_t* p) { return (uint64_t)(p - g_blob.data()) / 64; }

bool write_words(const std::string& path, const std::vector<uint64_t>& w) {
  FILE* o = fopen(path.c_str(), "wb");
  if (!o) return false;
  const bool ok = fwrite(w.data(), sizeof(uint64_t), w.size(), o) == w.size();
  return fclose(o) == 0 && ok;
}

}  // namespace

int main(int argc, char** argv) {
  if (argc != 5) {
    fprintf(stderr, "usage: pin_treelets <blob file> <max bytes per treelet> <remap stride> <out file>\n");
    return 2;
  }
  FILE* f = fopen(argv[1], "rb");
  if (!f) return 2;
  fseek(f, 0, SEEK_END);
  g_blob.resize((size_t)ftell(f));
  fseek(f, 0, SEEK_SET);
  if (fread(g_blob.data(), 1, g_blob.size(), f) != g_blob.size()) return 2;
  fclose(f);
  const int budget = atoi(argv[2]);
  pin::g_gpu.cfg.max_treelet_size = (uint64_t)budget;
  pin::g_gpu.cluster.core.cfg.treelet_remap_stride = strtoull(argv[3], nullptr, 10);

  GEN_RT_BVH top;
  GEN_RT_BVH_unpack(&top, g_blob.data());
  find_blases(top.RootNodeOffset);
  std::cout.setstate(std::ios::failbit);  // the reference's progress lines are not output
  VulkanRayTracing::createTreelets((VkAccelerationStructureKHR)g_blob.data(), 0, budget);

  std::vector<uint64_t> out;
  out.push_back(VulkanRayTracing::treelet_roots_addr_only.size());
  for (const auto& root : VulkanRayTracing::treelet_roots_addr_only) {
    out.push_back(unit_of(root.first));
    out.push_back(root.second.size());
    for (const StackEntry& m : root.second) out.push_back(unit_of(m.addr));
  }
  out.push_back(VulkanRayTracing::node_map_addr_only.size());
  for (const auto& kv : VulkanRayTracing::node_map_addr_only) {
    out.push_back(unit_of(kv.first));
    out.push_back(unit_of(kv.second));
  }
  out.push_back(VulkanRayTracing::treelet_addr_to_metadata_idx.size());
  for (const auto& kv : VulkanRayTracing::treelet_addr_to_metadata_idx) {
    out.push_back(unit_of(kv.first));
    out.push_back(kv.second);
  }
  if (!write_words(argv[4], out)) return 2;

  // The remap runs last: where the reference asserts in it (a treelet root
  // that is already a member of an earlier treelet) the process aborts and
  // the .remap file is not written.
  VulkanRayTracing::remapBVHToTreeletLayout();
  std::vector<uint64_t> rm;
  rm.push_back(VulkanRayTracing::original_bvh_to_treelet_bvh_mapping.size());
  for (const auto& kv : VulkanRayTracing::original_bvh_to_treelet_bvh_mapping) {
    rm.push_back(unit_of(kv.first));
    rm.push_back((uint64_t)(kv.second - pin::g_layout_base));
  }
  if (!write_words(std::string(argv[4]) + ".remap", rm)) return 2;
  return 0;
}
