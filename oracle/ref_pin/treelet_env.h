// The setting the RT-unit harnesses (pin_prefetch.cpp, pin_rtunit.cpp) share:
// stand-ins for the simulator objects that the reference's createTreelets and
// the RT unit's code reach (the shader and GPU configuration, the cycle
// counters, GPGPU_Context), VulkanRayTracing with the treelet maps, and the
// reference's own treelet formation, extracted unmodified by the Makefile
// into tl_maps.inc and tl_create.inc.  load_scene() reads a blob and forms
// its treelets with it.
#pragma once
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
  // read by rt_unit::schedule_next_warp and the stride prefetcher
  unsigned m_treelet_scheduler = 0;
  bool m_lee_micro_prefetcher = false;
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

bool load_scene(const char* blob_path, int budget) {
  g_blob = read_file(blob_path);
  if (g_blob.empty()) return false;
  pin::g_gpu.cluster.core = &pin::g_core;
  pin::g_gpu.cluster.cores[0] = &pin::g_core;
  pin::g_gpu.cfg.max_treelet_size = (uint64_t)budget;
  GEN_RT_BVH top;
  GEN_RT_BVH_unpack(&top, g_blob.data());
  find_blases(top.RootNodeOffset);
  std::cout.setstate(std::ios::failbit);
  VulkanRayTracing::createTreelets((VkAccelerationStructureKHR)g_blob.data(), 0, budget);
  return true;
}

}  // namespace

