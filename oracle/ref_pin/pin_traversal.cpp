// Traces rays with the REFERENCE's own VulkanRayTracing::traceRay and
// traceRayWithTreelets and writes each ray's hit record, its memory
// transactions (the visit trace) and, for the treelet walk, the treelet of
// every transaction: the golden data the oracle's traversal is pinned against.
//
// The reference functions are not copied here.  The Makefile in this folder
// extracts them, unmodified, into oracle/_ref/extract/ (git-ignored):
//   geom_*.inc, tl_*.inc   as for pin_geometry and pin_treelets
//   tr_records.inc   TransactionType .. StoreTransactionType  src/abstract_hardware_model.h:201-216
//   tr_memrec.inc    MemoryTransactionRecord, MemoryStoreTransactionRecord
//                                                            src/abstract_hardware_model.h:315-329
//   tr_hitdata.inc   Hit_data, Traversal_data               src/cuda-sim/vulkan_rt_thread_data.h:29-58
//   tr_walks.inc     traceRayWithTreelets, traceRay         src/cuda-sim/vulkan_ray_tracing.cc:1522-3076
// What they use of the rest of the simulator is declared below in this
// file's own code: a thread object that keeps the transactions and the
// traversal record the walk hands it, a memory space that copies the record,
// statistics counters, and the configuration chain (no remap, no metadata).
//
// Usage: pin_traversal <blob file> <rays file> <mode 0 traceRay | 1 traceRayWithTreelets>
//                      <ray flags> <max bytes per treelet> <device offset> <out file>
// rays file: records of 8 floats (origin, tmin, direction, tmax).
// out file, per ray (uint32 words): hit_geometry, geometry_index,
// primitive_index, instance_index, world_min_thit, barycentric x y z,
// intersection_point x y z (floats as bits), n transactions, then per
// transaction: (address - blob - device offset) / 64, type, size, treelet
// (root unit of addrToTreeletID(address), or 0xFFFFFFFF in traceRay).
//
// Timing: pin_traversal --time <blob> <rays> <mode> <ray flags> <treelet bytes>
//                              <threads> <reps> [<hits out>]   (see time_walk)
#include <algorithm>
#include <atomic>
#include <cassert>
#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <deque>
#include <fstream>
#include <iostream>
#include <list>
#include <map>
#include <string>
#include <thread>
#include <utility>
#include <vector>
#include <vector_types.h>

#include "vulkan_acceleration_structure_util.h"

typedef void* VkAccelerationStructureKHR;
typedef unsigned int uint;

// SPIR-V ray flags (the SPIR-V specification's RayFlags values)
enum {
  SpvRayFlagsOpaqueKHRMask = 0x1,
  SpvRayFlagsNoOpaqueKHRMask = 0x2,
  SpvRayFlagsTerminateOnFirstHitKHRMask = 0x4,
  SpvRayFlagsSkipClosestHitShaderKHRMask = 0x8,
};
// VkGeometryTypeKHR (the Vulkan specification's values)
typedef enum VkGeometryTypeKHR {
  VK_GEOMETRY_TYPE_TRIANGLES_KHR = 0,
  VK_GEOMETRY_TYPE_AABBS_KHR = 1,
  VK_GEOMETRY_TYPE_INSTANCES_KHR = 2,
} VkGeometryTypeKHR;

#define MAX_DESCRIPTOR_SETS 1
#define MAX_DESCRIPTOR_SET_BINDINGS 32
#define VSIM_DPRINTF(...)
#define RT_DPRINTF(...)

#include "geom_minmax.inc"
#include "geom_ray.inc"
#include "geom_vecmath.inc"
#include "tl_stackentry.inc"
#include "tr_records.inc"
#include "tr_memrec.inc"
#include "tr_hitdata.inc"

// ---- the simulator objects the walks touch
class ptx_instruction;
class ptx_thread_info;

class memory_space {
 public:
  // the walk writes its Traversal_data record here; it is kept for output
  void write(void* addr, size_t size, const void* data, ptx_thread_info*, const ptx_instruction*) {
    (void)addr;
    last.assign((const uint8_t*)data, (const uint8_t*)data + size);
  }
  std::vector<uint8_t> last;
};

struct Vulkan_RT_thread_data {
  std::vector<Traversal_data*> traversal_data;
  std::vector<Hit_data*> all_hit_data;
  void set_hitAttribute(float3, const ptx_instruction*, ptx_thread_info*) {}
};

class ptx_thread_info {
 public:
  dim3 get_ctaid() const { return dim3(0, 0, 0); }
  dim3 get_tid() const { return dim3(0, 0, 0); }
  unsigned get_uid() const { return 0; }
  unsigned get_hw_tid() const { return 0; }
  memory_space* get_global_memory() { return &mem; }
  void add_ray_properties(Ray) {}
  void add_ray_intersect() {}
  void set_rt_transactions(std::vector<MemoryTransactionRecord> t) { tx = t; }
  void set_rt_store_transactions(std::vector<MemoryStoreTransactionRecord>) {}
  Vulkan_RT_thread_data* RT_thread_data = &rt;
  Vulkan_RT_thread_data rt;
  memory_space mem;
  std::vector<MemoryTransactionRecord> tx;
};

// The any-hit / intersection shader tables of non-opaque and procedural
// geometry are not part of the pinned path: a table here records nothing and
// adds no transactions, so the walk's own visits are what is compared.
struct warp_intersection_table {
  std::pair<std::vector<MemoryTransactionRecord>, std::vector<MemoryStoreTransactionRecord>> add_intersection(
      uint32_t, uint32_t, uint32_t, uint32_t, const ptx_instruction*, ptx_thread_info*) {
    return {};
  }
};
warp_intersection_table g_table;
warp_intersection_table* g_table_row[1] = {&g_table};
warp_intersection_table** g_table_grid[1] = {g_table_row};

namespace pin {
// Statistics the walks update.  Atomic so that the timing mode can run the
// walks on several threads; the world bounds are set by the first ray, which
// the timing mode traces alone before any thread starts.
struct FuncSim {
  std::atomic<unsigned long long> g_n_anyhit_rays{0}, g_n_closesthit_rays{0};
  std::atomic<unsigned long long> g_rt_mem_access_type[16] = {};
  std::atomic<bool> g_rt_world_set{false};
  float3 g_rt_world_min{}, g_rt_world_max{};
  std::atomic<unsigned long long> g_max_nodes_per_ray{0}, g_tot_nodes_per_ray{0}, g_max_tree_depth{0};
  std::atomic<unsigned long long> g_rt_num_hits{0}, g_rt_num_any_hits{0};
};
struct ShaderConfig {
  bool remap_to_treelet_layout = false;
  bool load_treelet_metadata = false;
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
  unsigned long long gpu_sim_cycle = 0;
  Cluster** get_m_cluster() { return clusters; }
  const GpuConfig& get_config() const { return cfg; }
};
struct Sim {
  Gpu* g_the_gpu;
};
struct Context {
  Sim* the_gpgpusim;
  FuncSim* func_sim;
};
Gpu g_gpu;
Sim g_sim{&g_gpu};
FuncSim g_func;
Context g_ctx{&g_sim, &g_func};
uint8_t* g_layout_base = reinterpret_cast<uint8_t*>(uintptr_t(1) << 40);
}  // namespace pin

typedef pin::Context gpgpu_context;
gpgpu_context* GPGPU_Context() { return &pin::g_ctx; }
void* gpgpusim_malloc(size_t) { return pin::g_layout_base; }

struct DESCRIPTOR_SET_STRUCT;

struct VulkanRayTracing {
  static std::map<void*, void*> blas_addr_map;
  static void* tlas_addr;
  static bool dumped;
  static DESCRIPTOR_SET_STRUCT* descriptorSet;
  static void* launcher_descriptorSets[MAX_DESCRIPTOR_SETS][MAX_DESCRIPTOR_SET_BINDINGS];
  static void* launcher_deviceDescriptorSets[MAX_DESCRIPTOR_SETS][MAX_DESCRIPTOR_SET_BINDINGS];
  static warp_intersection_table*** intersection_table;
  static warp_intersection_table*** anyhit_table;
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
  static std::atomic<unsigned> accessedDataSize;

  static bool isTreeletRoot(StackEntry node);
  static bool isTreeletRoot(uint8_t* addr);
  static uint8_t* addrToTreeletID(uint8_t* addr);
  static void buildNodeToRootMap();
  static std::vector<StackEntry> treeletIDToChildren(StackEntry treelet_root);
  static std::vector<StackEntry> treeletIDToChildren(uint8_t* treelet_root);
  static float calculateSAH(float3 lo, float3 hi);
  static void createTreelets(VkAccelerationStructureKHR _topLevelAS, int64_t device_offset, int maxBytesPerTreelet);
  static void remapBVHToTreeletLayout();
  static bool mt_ray_triangle_test(float3 p0, float3 p1, float3 p2, Ray ray_properties, float* thit);
  static float3 Barycentric(float3 p, float3 a, float3 b, float3 c);
  // simulated device memory for the records the walk writes; the memory
  // space above keeps the bytes, so no address is needed
  static void* gpgpusim_alloc(size_t) { return nullptr; }
  static void dump_AS(DESCRIPTOR_SET_STRUCT*, VkAccelerationStructureKHR) { abort(); }
  static void traceRayWithTreelets(VkAccelerationStructureKHR _topLevelAS, uint rayFlags, uint cullMask,
                                   uint sbtRecordOffset, uint sbtRecordStride, uint missIndex, float3 origin,
                                   float Tmin, float3 direction, float Tmax, int payload, const ptx_instruction* pI,
                                   ptx_thread_info* thread);
  static void traceRay(VkAccelerationStructureKHR _topLevelAS, uint rayFlags, uint cullMask, uint sbtRecordOffset,
                       uint sbtRecordStride, uint missIndex, float3 origin, float Tmin, float3 direction, float Tmax,
                       int payload, const ptx_instruction* pI, ptx_thread_info* thread);
};

std::map<void*, void*> VulkanRayTracing::blas_addr_map;
void* VulkanRayTracing::tlas_addr = nullptr;
bool VulkanRayTracing::dumped = false;
DESCRIPTOR_SET_STRUCT* VulkanRayTracing::descriptorSet = nullptr;
void* VulkanRayTracing::launcher_descriptorSets[MAX_DESCRIPTOR_SETS][MAX_DESCRIPTOR_SET_BINDINGS] = {};
void* VulkanRayTracing::launcher_deviceDescriptorSets[MAX_DESCRIPTOR_SETS][MAX_DESCRIPTOR_SET_BINDINGS] = {};
warp_intersection_table*** VulkanRayTracing::intersection_table = g_table_grid;
warp_intersection_table*** VulkanRayTracing::anyhit_table = g_table_grid;
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
std::atomic<unsigned> VulkanRayTracing::accessedDataSize{0};

// the file-scope state of vulkan_ray_tracing.cc the walks read and write (the
// ray counter per thread: it only numbers rays)
thread_local unsigned rayCount = 0;
bool use_external_launcher = false;
const bool dump_trace = false;
bool treeletsFormed = false;
bool debugTraversal = false;

#include "geom_vrt_a.inc"
#include "geom_vrt_b.inc"
#include "tl_maps.inc"
#include "tl_create.inc"
#include "tr_walks.inc"

namespace {

std::vector<uint8_t> g_blob;

void find_blases(uint64_t off, int64_t device_offset) {
  GEN_RT_BVH_INTERNAL_NODE n;
  GEN_RT_BVH_INTERNAL_NODE_unpack(&n, g_blob.data() + off);
  uint64_t child = off + (int64_t)n.ChildOffset * 64;
  for (int i = 0; i < 6; ++i) {
    if (n.ChildSize[i] > 0) {
      if (n.ChildType[i] == NODE_TYPE_INTERNAL) {
        find_blases(child, device_offset);
      } else {
        GEN_RT_BVH_INSTANCE_LEAF leaf;
        GEN_RT_BVH_INSTANCE_LEAF_unpack(&leaf, g_blob.data() + child);
        uint8_t* blas = g_blob.data() + child + leaf.BVHAddress;
        VulkanRayTracing::blas_addr_map[blas] = blas + device_offset;
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

uint32_t bits(float f) {
  uint32_t u;
  memcpy(&u, &f, 4);
  return u;
}

}  // namespace

// Timing mode: the reference's own walk over the rays on `threads` host
// threads (contiguous ray ranges), `reps` times after one untimed pass; prints
// "rep <i> <seconds>" per pass on stderr.  The first ray is traced alone
// first, so that the walk's lazy one-time set-up (createTreelets, the world
// bounds) is done before the threads start.
// With `hits_out`, one more untimed pass writes each ray's 11 hit words (the
// layout of the result file below, without the transactions) there.
int time_walk(int mode, uint32_t flags, const std::vector<uint8_t>& rays, int threads, int reps,
              const char* hits_out) {
  uint8_t* tlas = g_blob.data();
  const size_t n = rays.size() / 32;
  std::vector<uint32_t> words;
  auto trace_range = [&](size_t lo, size_t hi) {
    for (size_t r = lo; r < hi; ++r) {
      float v[8];
      memcpy(v, rays.data() + 32 * r, 32);
      ptx_thread_info thread;
      const float3 o = {v[0], v[1], v[2]}, d = {v[4], v[5], v[6]};
      if (mode == 0)
        VulkanRayTracing::traceRay(tlas, flags, 0xFF, 0, 0, 0, o, v[3], d, v[7], 0, nullptr, &thread);
      else
        VulkanRayTracing::traceRayWithTreelets(tlas, flags, 0xFF, 0, 0, 0, o, v[3], d, v[7], 0, nullptr, &thread);
      if (!words.empty()) {
        Traversal_data td;
        memcpy(&td, thread.mem.last.data(), sizeof td);
        const Hit_data& h = td.closest_hit;
        uint32_t* w = words.data() + 11 * r;
        if (td.hit_geometry) {
          const uint32_t x[11] = {1u, h.geometry_index, h.primitive_index, h.instance_index, bits(h.world_min_thit),
                                  bits(h.barycentric_coordinates.x), bits(h.barycentric_coordinates.y),
                                  bits(h.barycentric_coordinates.z), bits(h.intersection_point.x),
                                  bits(h.intersection_point.y), bits(h.intersection_point.z)};
          memcpy(w, x, sizeof x);
        }
      }
    }
  };
  trace_range(0, std::min<size_t>(1, n));
  for (int rep = -1; rep < reps; ++rep) {
    const auto t0 = std::chrono::steady_clock::now();
    std::vector<std::thread> pool;
    for (int t = 0; t < threads; ++t)
      pool.emplace_back(trace_range, n * t / threads, n * (t + 1) / threads);
    for (auto& th : pool) th.join();
    const double s = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    if (rep >= 0) fprintf(stderr, "rep %d %.6f\n", rep, s);
  }
  if (hits_out) {
    words.assign(11 * n, 0u);
    std::vector<std::thread> pool;
    for (int t = 0; t < threads; ++t)
      pool.emplace_back(trace_range, n * t / threads, n * (t + 1) / threads);
    for (auto& th : pool) th.join();
    FILE* f = fopen(hits_out, "wb");
    if (!f) return 2;
    fwrite(words.data(), sizeof(uint32_t), words.size(), f);
    fclose(f);
  }
  return 0;
}

int main(int argc, char** argv) {
  if ((argc == 9 || argc == 10) && std::string(argv[1]) == "--time") {
    // pin_traversal --time <blob> <rays> <mode> <ray flags> <treelet bytes> <threads> <reps> [<hits out>]
    g_blob = read_file(argv[2]);
    const std::vector<uint8_t> rays = read_file(argv[3]);
    const int mode = atoi(argv[4]);
    pin::g_gpu.cfg.max_treelet_size = strtoull(argv[6], nullptr, 10);
    const int threads = atoi(argv[7]), reps = atoi(argv[8]);
    if (g_blob.empty() || rays.empty() || rays.size() % 32 || (mode != 0 && mode != 1) || threads < 1 || reps < 1)
      return 2;
    VulkanRayTracing::tlas_addr = g_blob.data();
    GEN_RT_BVH top;
    GEN_RT_BVH_unpack(&top, g_blob.data());
    find_blases(top.RootNodeOffset, 0);
    if (!freopen("/dev/null", "w", stdout)) return 2;
    std::cout.setstate(std::ios::failbit);
    return time_walk(mode, (uint32_t)strtoul(argv[5], nullptr, 10), rays, threads, reps, argc == 10 ? argv[9] : nullptr);
  }
  if (argc != 8) {
    fprintf(stderr, "usage: pin_traversal <blob> <rays> <mode 0|1> <ray flags> <treelet bytes> <device offset> <out>\n");
    return 2;
  }
  g_blob = read_file(argv[1]);
  const std::vector<uint8_t> rays = read_file(argv[2]);
  const int mode = atoi(argv[3]);
  const uint32_t flags = (uint32_t)strtoul(argv[4], nullptr, 10);
  pin::g_gpu.cfg.max_treelet_size = strtoull(argv[5], nullptr, 10);
  const int64_t device_offset = strtoll(argv[6], nullptr, 10);
  if (g_blob.empty() || rays.size() % 32 || (mode != 0 && mode != 1)) return 2;

  uint8_t* tlas = g_blob.data();
  // the simulated device address of the TLAS; every BLAS is offset alike
  VulkanRayTracing::tlas_addr = tlas + device_offset;
  GEN_RT_BVH top;
  GEN_RT_BVH_unpack(&top, tlas);
  find_blases(top.RootNodeOffset, device_offset);
  // the reference prints a treelet line per ray and progress to stdout
  if (!freopen("/dev/null", "w", stdout)) return 2;
  std::cout.setstate(std::ios::failbit);

  std::vector<uint32_t> out;
  const size_t n = rays.size() / 32;
  for (size_t r = 0; r < n; ++r) {
    float v[8];
    memcpy(v, rays.data() + 32 * r, 32);
    ptx_thread_info thread;
    const float3 o = {v[0], v[1], v[2]}, d = {v[4], v[5], v[6]};
    if (mode == 0)
      VulkanRayTracing::traceRay(tlas, flags, 0xFF, 0, 0, 0, o, v[3], d, v[7], 0, nullptr, &thread);
    else
      VulkanRayTracing::traceRayWithTreelets(tlas, flags, 0xFF, 0, 0, 0, o, v[3], d, v[7], 0, nullptr, &thread);
    Traversal_data td;
    assert(thread.mem.last.size() == sizeof(Traversal_data));
    memcpy(&td, thread.mem.last.data(), sizeof td);
    const Hit_data& h = td.closest_hit;
    if (td.hit_geometry) {
      out.insert(out.end(), {1u, h.geometry_index, h.primitive_index, h.instance_index, bits(h.world_min_thit),
                             bits(h.barycentric_coordinates.x), bits(h.barycentric_coordinates.y),
                             bits(h.barycentric_coordinates.z), bits(h.intersection_point.x),
                             bits(h.intersection_point.y), bits(h.intersection_point.z)});
    } else {
      out.insert(out.end(), 11, 0u);
    }
    out.push_back((uint32_t)thread.tx.size());
    for (const MemoryTransactionRecord& t : thread.tx) {
      uint8_t* dev = (uint8_t*)t.address;
      out.push_back((uint32_t)((dev - device_offset - tlas) / 64));
      out.push_back((uint32_t)t.type);
      out.push_back(t.size);
      uint32_t tl = 0xFFFFFFFFu;
      if (mode == 1) tl = (uint32_t)((VulkanRayTracing::addrToTreeletID(dev) - device_offset - tlas) / 64);
      out.push_back(tl);
    }
  }
  FILE* f = fopen(argv[7], "wb");
  if (!f) return 2;
  fwrite(out.data(), sizeof(uint32_t), out.size(), f);
  fclose(f);
  return 0;
}
