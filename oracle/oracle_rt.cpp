// oracle_rt.cpp - CPU restatement of the reference's functional RT path.
//
// TEST INFRASTRUCTURE ONLY (the checker; see oracle_rt.h for the parity
// status).  Each function follows the cited lines of the reference, keeping
// its containers (std::list used as a stack, std::map keyed by address,
// std::deque queues) and its operation order.  Built with
// -ffp-contract=off so that no multiply-add is fused.
//
// Address model: one address space.  A node address is a pointer into the
// blob; device_offset and every BLAS offset are 0, so the "host" and
// "device" addresses of the reference coincide.
#include "oracle_rt.h"

#include <cmath>
#include <cstring>
#include <deque>
#include <list>
#include <map>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

namespace {

thread_local std::string g_err;

// ---------------------------------------------------------------- math types
struct float3 {
  float x, y, z;
};
struct float4 {
  float x, y, z, w;
};

// float4x4 (vulkan_acceleration_structure_util.h:44-56)
struct float4x4 {
  float m[4][4];
  float4 operator*(const float4& v_) const {
    float vec[] = {v_.x, v_.y, v_.z, v_.w};
    float res[] = {0, 0, 0, 0};
    for (int i = 0; i < 4; i++)
      for (int j = 0; j < 4; j++) res[i] += this->m[j][i] * vec[j];
    return {res[0], res[1], res[2], res[3]};
  }
};

// vector-math.cc:1-82
float3 make_float3(float a, float b, float c) { return {a, b, c}; }
float3 operator-(float3 a, float3 b) { return make_float3(a.x - b.x, a.y - b.y, a.z - b.z); }
float3 operator+(float3 a, float3 b) { return make_float3(a.x + b.x, a.y + b.y, a.z + b.z); }
float3 cross(float3 a, float3 b) { return make_float3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x); }
float dot(float3 a, float3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }

// vulkan_ray_tracing.h:53-56
inline float MAXf(float a, float b) { return ((a) > (b)) ? (a) : (b); }
inline float MINf(float a, float b) { return ((a) < (b)) ? (a) : (b); }
inline float MIN_MAX(float a, float b, float c) { return MAXf(MINf(a, b), c); }
inline float MAX_MIN(float a, float b, float c) { return MINf(MAXf(a, b), c); }

// Ray (abstract_hardware_model.h:333-370)
struct Ray {
  float4 origin_tmin;
  float4 dir_tmax;
  float3 get_origin() const { return {origin_tmin.x, origin_tmin.y, origin_tmin.z}; }
  float get_tmin() const { return origin_tmin.w; }
  float get_tmax() const { return dir_tmax.w; }
  float3 get_direction() const { return {dir_tmax.x, dir_tmax.y, dir_tmax.z}; }
  void make_ray(float3 o, float3 d, float t_min, float t_max) {
    origin_tmin = {o.x, o.y, o.z, t_min};
    dir_tmax = {d.x, d.y, d.z, t_max};
  }
};

// ------------------------------------------------------------- node decoders
// vulkan_acceleration_structure_util.h:73-497
template <class T>
T rd(const uint8_t* p) {
  T v;
  std::memcpy(&v, p, sizeof(T));
  return v;
}

struct GEN_RT_BVH {
  uint64_t RootNodeOffset;
  float3 BoundsMin, BoundsMax;
};
void unpack_bvh(GEN_RT_BVH* d, const uint8_t* p) {
  d->RootNodeOffset = rd<uint64_t>(p);
  d->BoundsMin = {rd<float>(p + 8), rd<float>(p + 12), rd<float>(p + 16)};
  d->BoundsMax = {rd<float>(p + 20), rd<float>(p + 24), rd<float>(p + 28)};
}

struct GEN_RT_BVH_INTERNAL_NODE {
  float3 Origin;
  int32_t ChildOffset;
  uint32_t NodeType;
  int32_t ChildBoundsExponentX, ChildBoundsExponentY, ChildBoundsExponentZ;
  uint32_t NodeRayMask;
  uint32_t ChildSize[6], ChildType[6];
  uint32_t ChildLowerXBound[6], ChildUpperXBound[6];
  uint32_t ChildLowerYBound[6], ChildUpperYBound[6];
  uint32_t ChildLowerZBound[6], ChildUpperZBound[6];
};
void unpack_internal(GEN_RT_BVH_INTERNAL_NODE* d, const uint8_t* p) {
  d->Origin = {rd<float>(p), rd<float>(p + 4), rd<float>(p + 8)};
  d->ChildOffset = rd<int32_t>(p + 12);
  d->NodeType = p[16];
  d->ChildBoundsExponentX = (int32_t)(int8_t)p[18];
  d->ChildBoundsExponentY = (int32_t)(int8_t)p[19];
  d->ChildBoundsExponentZ = (int32_t)(int8_t)p[20];
  d->NodeRayMask = p[21];
  for (int i = 0; i < 6; i++) {
    const uint8_t t = p[22 + i] & 0x3f;
    d->ChildSize[i] = t & 0x03;
    d->ChildType[i] = t >> 2;
  }
  for (int i = 0; i < 6; i++) d->ChildLowerXBound[i] = p[28 + i];
  for (int i = 0; i < 6; i++) d->ChildUpperXBound[i] = p[34 + i];
  for (int i = 0; i < 6; i++) d->ChildLowerYBound[i] = p[40 + i];
  for (int i = 0; i < 6; i++) d->ChildUpperYBound[i] = p[46 + i];
  for (int i = 0; i < 6; i++) d->ChildLowerZBound[i] = p[52 + i];
  for (int i = 0; i < 6; i++) d->ChildUpperZBound[i] = p[58 + i];
}
constexpr uint32_t NODE_TYPE_INTERNAL = 0;
constexpr uint32_t NODE_TYPE_INSTANCE = 1;

// The decoded instance leaf keeps the reference struct's field order for the
// two 12-float runs that instance_leaf_matrix_to_float4x4 reads
// (asu.h:210-224, struct :226-262):
//   w2o_run = WorldToObjectm00..m22, ObjectToWorldm30..m32
//   o2w_run = ObjectToWorldm00..m22, WorldToObjectm30..m32
struct GEN_RT_BVH_INSTANCE_LEAF {
  uint32_t ShaderIndex, GeometryRayMask, InstanceContributionToHitGroupIndex, LeafType, GeometryFlags;
  uint32_t InstanceFlags;
  float w2o_run[12];
  uint64_t BVHAddress;
  uint32_t InstanceID, InstanceIndex;
  float o2w_run[12];
};
void unpack_instance(GEN_RT_BVH_INSTANCE_LEAF* d, const uint8_t* p) {
  d->ShaderIndex = rd<uint32_t>(p) & 0x00ffffff;
  d->GeometryRayMask = p[3];
  d->InstanceContributionToHitGroupIndex = rd<uint32_t>(p + 4) & 0x00ffffff;
  const uint8_t t = p[7] >> 5;
  d->LeafType = t & 1;
  d->GeometryFlags = t >> 1;
  d->InstanceFlags = p[14];
  for (int k = 0; k < 9; ++k) d->w2o_run[k] = rd<float>(p + 16 + 4 * k);   // WorldToObjectm00..m22
  for (int k = 0; k < 3; ++k) d->o2w_run[9 + k] = rd<float>(p + 52 + 4 * k);  // WorldToObjectm30..m32
  d->BVHAddress = rd<uint64_t>(p + 64);
  d->InstanceID = rd<uint32_t>(p + 72);
  d->InstanceIndex = rd<uint32_t>(p + 76);
  for (int k = 0; k < 9; ++k) d->o2w_run[k] = rd<float>(p + 80 + 4 * k);   // ObjectToWorldm00..m22
  for (int k = 0; k < 3; ++k) d->w2o_run[9 + k] = rd<float>(p + 116 + 4 * k);  // ObjectToWorldm30..m32
}

float4x4 instance_leaf_matrix_to_float4x4(const float* a) {
  float4x4 m;
  for (int i = 0; i < 4; i++) {
    for (int j = 0; j < 3; j++) m.m[i][j] = *a++;
    m.m[i][3] = 0;
  }
  m.m[3][3] = 1;
  return m;
}

struct GEN_RT_BVH_PRIMITIVE_LEAF_DESCRIPTOR {
  uint32_t ShaderIndex, GeometryRayMask, GeometryIndex, LeafType, GeometryFlags;
};
void unpack_desc(GEN_RT_BVH_PRIMITIVE_LEAF_DESCRIPTOR* d, const uint8_t* p) {
  d->ShaderIndex = rd<uint32_t>(p) & 0x00ffffff;
  d->GeometryRayMask = p[3];
  const uint32_t t = rd<uint32_t>(p + 4);
  d->GeometryIndex = t & 0x0fffffff;
  d->LeafType = (t >> 29) & 1;
  d->GeometryFlags = t >> 30;
}
constexpr uint32_t TYPE_QUAD = 0;

struct GEN_RT_BVH_QUAD_LEAF {
  GEN_RT_BVH_PRIMITIVE_LEAF_DESCRIPTOR LeafDescriptor;
  uint32_t PrimitiveIndex0, PrimitiveIndex1Delta, j0, j1, j2;
  float3 QuadVertex[4];
};
void unpack_quad(GEN_RT_BVH_QUAD_LEAF* d, const uint8_t* p) {
  unpack_desc(&d->LeafDescriptor, p);
  d->PrimitiveIndex0 = rd<uint32_t>(p + 8);
  const uint32_t t = rd<uint32_t>(p + 12);
  d->PrimitiveIndex1Delta = t & 0x0001ffff;
  d->j0 = (t >> 17) & 3;
  d->j1 = (t >> 19) & 3;
  d->j2 = (t >> 21) & 3;
  for (int v = 0; v < 4; ++v)
    d->QuadVertex[v] = {rd<float>(p + 16 + 12 * v), rd<float>(p + 20 + 12 * v), rd<float>(p + 24 + 12 * v)};
}

// set_child_bounds (asu.h:499-508)
void set_child_bounds(const GEN_RT_BVH_INTERNAL_NODE* n, int c, float3* lo, float3* hi) {
  lo->x = n->Origin.x + ldexpf((float)n->ChildLowerXBound[c], n->ChildBoundsExponentX - 8);
  lo->y = n->Origin.y + ldexpf((float)n->ChildLowerYBound[c], n->ChildBoundsExponentY - 8);
  lo->z = n->Origin.z + ldexpf((float)n->ChildLowerZBound[c], n->ChildBoundsExponentZ - 8);
  hi->x = n->Origin.x + ldexpf((float)n->ChildUpperXBound[c], n->ChildBoundsExponentX - 8);
  hi->y = n->Origin.y + ldexpf((float)n->ChildUpperYBound[c], n->ChildBoundsExponentY - 8);
  hi->z = n->Origin.z + ldexpf((float)n->ChildUpperZBound[c], n->ChildBoundsExponentZ - 8);
}

// ------------------------------------------------------- geometry (vrt.cc)
float get_norm(float3 v) { return std::sqrt(v.x * v.x + v.y * v.y + v.z * v.z); }  // :152-155
float3 normalized(float3 v) {  // :162-166
  float norm = get_norm(v);
  return {v.x / norm, v.y / norm, v.z / norm};
}

Ray make_transformed_ray(const Ray& ray, const float4x4& matrix, float* mult) {  // :168-181
  Ray r;
  float4 o4 = matrix * float4{ray.get_origin().x, ray.get_origin().y, ray.get_origin().z, 1};
  float4 d4 = matrix * float4{ray.get_direction().x, ray.get_direction().y, ray.get_direction().z, 0};
  float3 o = {o4.x / o4.w, o4.y / o4.w, o4.z / o4.w};
  float3 d = {d4.x, d4.y, d4.z};
  *mult = get_norm(d);
  d = normalized(d);
  r.make_ray(o, d, ray.get_tmin() * (*mult), ray.get_tmax() * (*mult));
  return r;
}

float magic_max7(float a0, float a1, float b0, float b1, float c0, float c1, float d) {  // :183-189
  float t1 = MIN_MAX(a0, a1, d);
  float t2 = MIN_MAX(b0, b1, t1);
  return MIN_MAX(c0, c1, t2);
}
float magic_min7(float a0, float a1, float b0, float b1, float c0, float c1, float d) {  // :191-197
  float t1 = MAX_MIN(a0, a1, d);
  float t2 = MAX_MIN(b0, b1, t1);
  return MAX_MIN(c0, c1, t2);
}
float3 get_t_bound(float3 box, float3 origin, float3 idir) {  // :199-218
  return {(box.x - origin.x) * idir.x, (box.y - origin.y) * idir.y, (box.z - origin.z) * idir.z};
}
float3 calculate_idir(float3 d) {  // :220-235
  const float ooeps = exp2f(-80.0f);
  float3 r;
  r.x = 1.0f / (fabsf(d.x) > ooeps ? d.x : copysignf(ooeps, d.x));
  r.y = 1.0f / (fabsf(d.y) > ooeps ? d.y : copysignf(ooeps, d.y));
  r.z = 1.0f / (fabsf(d.z) > ooeps ? d.z : copysignf(ooeps, d.z));
  return r;
}
bool ray_box_test(float3 low, float3 high, float3 idir, float3 origin, float tmin, float tmax, float& thit) {  // :237-257
  float3 lo = get_t_bound(low, origin, idir);
  float3 hi = get_t_bound(high, origin, idir);
  float mn = magic_max7(lo.x, hi.x, lo.y, hi.y, lo.z, hi.z, tmin);
  float mx = magic_min7(lo.x, hi.x, lo.y, hi.y, lo.z, hi.z, tmax);
  thit = mn;
  return mn <= mx;
}
bool mt_ray_triangle_test(float3 p0, float3 p1, float3 p2, const Ray& r, float* thit) {  // :3089-3111
  float3 v0v1 = p1 - p0;
  float3 v0v2 = p2 - p0;
  float3 pvec = cross(r.get_direction(), v0v2);
  float det = dot(v0v1, pvec);
  float idet = 1 / det;
  float3 tvec = r.get_origin() - p0;
  float u = dot(tvec, pvec) * idet;
  if (u < 0 || u > 1) return false;
  float3 qvec = cross(tvec, v0v1);
  float v = dot(r.get_direction(), qvec) * idet;
  if (v < 0 || (u + v) > 1) return false;
  *thit = dot(v0v2, qvec) * idet;
  return true;
}
float3 Barycentric(float3 p, float3 a, float3 b, float3 c) {  // :3113-3130
  float3 v0 = b - a, v1 = c - a, v2 = p - a;
  float d00 = dot(v0, v0), d01 = dot(v0, v1), d11 = dot(v1, v1), d20 = dot(v2, v0), d21 = dot(v2, v1);
  float denom = d00 * d11 - d01 * d01;
  float v = (d11 * d20 - d01 * d21) / denom;
  float w = (d00 * d21 - d01 * d20) / denom;
  float u = 1.0f - v - w;
  return {v, w, u};
}

// ------------------------------------------------------------ stack entries
struct StackEntry {  // vulkan_ray_tracing.h:180-208
  const uint8_t* addr = nullptr;
  bool topLevel = false, leaf = false;
  int size = 0;
  bool isBlasRoot = false;
  float worldToObject_tMultiplier = 0;
  const uint8_t* instAddr = nullptr;  // not in the reference: the instance leaf's address, for the hit record
  GEN_RT_BVH_INSTANCE_LEAF instanceLeaf{};
  float4x4 worldToObjectMatrix{}, objectToWorldMatrix{};
  Ray objectRay{};
  StackEntry() {}
  StackEntry(const uint8_t* a, bool t, bool l) : addr(a), topLevel(t), leaf(l) {}
  StackEntry(const uint8_t* a, bool t, bool l, int s) : addr(a), topLevel(t), leaf(l), size(s) {}
  StackEntry(const uint8_t* a, bool t, bool l, int s, bool b) : addr(a), topLevel(t), leaf(l), size(s), isBlasRoot(b) {}
};

struct Tx {
  const uint8_t* address;
  uint32_t type;
};

}  // namespace

// ============================================================ treelets
struct oracle_treelets {
  const uint8_t* base = nullptr;
  // treelet_roots_addr_only after de-dup (vulkan_ray_tracing.cc:1308-1358)
  std::map<const uint8_t*, std::vector<StackEntry>> roots;
  std::map<const uint8_t*, int> root_size;  // size of each root's key entry
  std::map<const uint8_t*, const uint8_t*> node_map;  // node_map_addr_only
  // addrToTreeletID (:468-472)
  const uint8_t* addrToTreeletID(const uint8_t* a) const {
    auto it = node_map.find(a);
    return it == node_map.end() ? nullptr : it->second;
  }
};

namespace {

void fail_msg(const std::string& m) { g_err = m; }

// createTreelets (vulkan_ray_tracing.cc:823-1470) with device_offset = 0.
bool create_treelets(const uint8_t* tlas, int maxBytesPerTreelet, oracle_treelets* out) {
  int remaining_bytes = maxBytesPerTreelet;
  std::map<const uint8_t*, std::vector<StackEntry>> completed;  // completed_treelet_roots_addr_only
  std::map<const uint8_t*, int> completed_size;
  std::deque<StackEntry> pending;  // treelet_roots_pending_work_queue
  std::deque<StackEntry> stack;
  std::deque<int> nodesize_stack;
  std::vector<StackEntry> nodes_in_current_treelet;

  pending.push_back(StackEntry(tlas, true, false, 64));  // :846-848
  GEN_RT_BVH topBVH;
  unpack_bvh(&topBVH, tlas);
  remaining_bytes -= 64;  // :852
  nodes_in_current_treelet.push_back(StackEntry(tlas, true, false, 64));
  const uint8_t* topRootAddr = tlas + topBVH.RootNodeOffset;
  stack.push_back(StackEntry(topRootAddr, true, false, 64));  // :857-860
  nodesize_stack.push_back(64);

  auto close_treelet = [&]() {
    const StackEntry r = pending.front();
    if (completed.find(r.addr) == completed.end()) completed_size[r.addr] = r.size;
    completed[r.addr] = nodes_in_current_treelet;
    pending.pop_front();
    nodes_in_current_treelet.clear();
  };

  while (!pending.empty()) {  // :863
    StackEntry next_node = stack.front();
    const uint8_t* next_node_addr = stack.front().addr;
    stack.pop_front();
    nodesize_stack.pop_front();
    while (next_node_addr != nullptr) {  // :882
      if (next_node.topLevel && !next_node.leaf) {  // :884-944
        const uint8_t* node_addr = next_node_addr;
        GEN_RT_BVH_INTERNAL_NODE node;
        unpack_internal(&node, node_addr);
        remaining_bytes -= 64;
        if (remaining_bytes < 0) return fail_msg("createTreelets asserts: remaining_bytes < 0"), false;
        nodes_in_current_treelet.push_back(next_node);
        const uint8_t* child_addr = node_addr + (node.ChildOffset * 64);
        for (int i = 0; i < 6; i++) {
          if (node.ChildSize[i] > 0) {
            if (node.ChildType[i] != NODE_TYPE_INTERNAL) {
              stack.push_back(StackEntry(child_addr, true, true, 128));
              nodesize_stack.push_back(128 + 64);
            } else {
              stack.push_back(StackEntry(child_addr, true, false, 64));
              nodesize_stack.push_back(64);
            }
          }
          child_addr += node.ChildSize[i] * 64;
        }
      } else if (next_node.topLevel && next_node.leaf) {  // :946-995
        const uint8_t* leaf_addr = next_node_addr;
        GEN_RT_BVH_INSTANCE_LEAF instanceLeaf;
        unpack_instance(&instanceLeaf, leaf_addr);
        remaining_bytes -= 128;
        if (remaining_bytes < 0) return fail_msg("createTreelets asserts: remaining_bytes < 0"), false;
        nodes_in_current_treelet.push_back(next_node);
        GEN_RT_BVH bot;
        unpack_bvh(&bot, leaf_addr + instanceLeaf.BVHAddress);
        remaining_bytes -= 64;
        nodes_in_current_treelet.push_back(StackEntry(leaf_addr + instanceLeaf.BVHAddress, true, true, 64, true));
        if (remaining_bytes < 0) return fail_msg("createTreelets asserts: remaining_bytes < 0"), false;
        const uint8_t* botLevelRootAddr = leaf_addr + instanceLeaf.BVHAddress + bot.RootNodeOffset;
        stack.push_back(StackEntry(botLevelRootAddr, false, false, 64));
        nodesize_stack.push_back(64);
      } else if (!next_node.topLevel && !next_node.leaf) {  // :997-1070
        const uint8_t* node_addr = next_node_addr;
        GEN_RT_BVH_INTERNAL_NODE node;
        unpack_internal(&node, node_addr);
        remaining_bytes -= 64;
        if (remaining_bytes < 0) return fail_msg("createTreelets asserts: remaining_bytes < 0"), false;
        nodes_in_current_treelet.push_back(next_node);
        const uint8_t* child_addr = node_addr + (node.ChildOffset * 64);
        for (int i = 0; i < 6; i++) {
          if (node.ChildSize[i] > 0) {
            if (node.ChildType[i] != NODE_TYPE_INTERNAL) {
              stack.push_back(StackEntry(child_addr, false, true, 64));
              nodesize_stack.push_back(64);
            } else {
              stack.push_back(StackEntry(child_addr, false, false, 64));
              nodesize_stack.push_back(64);
            }
          }
          child_addr += node.ChildSize[i] * 64;
        }
      } else {  // :1072-1114, quad and procedural leaves are both charged 64
        nodes_in_current_treelet.push_back(next_node);
        remaining_bytes -= 64;
        if (remaining_bytes < 0) return fail_msg("createTreelets asserts: remaining_bytes < 0"), false;
      }

      // :1117-1131 (the reference evaluates nodesize_stack.front() before
      // checking emptiness; the outcome depends only on emptiness then)
      if (!nodesize_stack.empty() && remaining_bytes - nodesize_stack.front() >= 0) {
        next_node = stack.front();
        next_node_addr = stack.front().addr;
        stack.pop_front();
        nodesize_stack.pop_front();
      } else if (!nodesize_stack.empty()) {  // :1132-1211
        close_treelet();
        for (size_t i = 0; i < stack.size(); i++) pending.push_back(stack[i]);
        stack.clear();
        nodesize_stack.clear();
        stack.push_back(pending.front());
        nodesize_stack.push_back(128);  // pending_nodesize.front() is never popped
        next_node = StackEntry(nullptr, false, false);
        next_node_addr = nullptr;
        remaining_bytes = maxBytesPerTreelet;
      } else {  // :1212-1268
        close_treelet();
        next_node = StackEntry(nullptr, false, false);
        next_node_addr = nullptr;
        remaining_bytes = maxBytesPerTreelet;
        stack.clear();
        nodesize_stack.clear();
        if (!pending.empty()) {
          stack.push_back(pending.front());
          nodesize_stack.push_back(128);
        }
      }
    }
  }
  // De-dup each member list keeping first occurrences (:1308-1333).
  for (auto& kv : completed) {
    std::vector<StackEntry> dupe_free;
    for (size_t i = 0; i < kv.second.size(); i++) {
      bool found = false;
      for (size_t j = 0; j < dupe_free.size(); j++)
        if (kv.second[i].addr == dupe_free[j].addr) {
          found = true;
          break;
        }
      if (!found) dupe_free.push_back(kv.second[i]);
    }
    kv.second = dupe_free;
  }
  out->roots = completed;
  out->root_size = completed_size;
  // buildNodeToRootMap (:475-489)
  out->node_map.clear();
  for (auto& root : out->roots) {
    out->node_map[root.first] = root.first;
    for (auto& node : root.second) out->node_map[node.addr] = root.first;
  }
  return true;
}

inline uint32_t unit_of(const uint8_t* base, const uint8_t* a) { return (uint32_t)((a - base) / 64); }

struct TraceOut {
  std::vector<Tx> transactions;
  rt_hit hit{};
  // Largest stack sizes the walk reached: traceRay's one stack (peak[0]),
  // or the current / other treelet stacks of traceRayWithTreelets
  // (peak[0] / peak[1]).  Not part of the reference's output; the tests use
  // them to predict which rays exceed a bounded stack.
  uint32_t peak[2] = {0, 0};
  void note(uint32_t k, size_t size) { peak[k] = std::max<uint32_t>(peak[k], (uint32_t)size); }
};

void finish_hit(TraceOut& o, bool hit, float min_thit, const Ray& ray, const GEN_RT_BVH_QUAD_LEAF& closest_leaf,
                const GEN_RT_BVH_INSTANCE_LEAF& closest_instanceLeaf, const Ray& closest_objectRay, float min_thit_object,
                const uint8_t* base, const uint8_t* closest_leaf_addr, const uint8_t* closest_inst_addr) {
  rt_hit& h = o.hit;
  std::memset(&h, 0, sizeof(h));
  if (hit) {  // :2990-3028 / :2202-2240
    h.hit_geometry = 1;
    h.geometry_index = closest_leaf.LeafDescriptor.GeometryIndex;
    h.primitive_index = closest_leaf.PrimitiveIndex0;
    h.instance_index = closest_instanceLeaf.InstanceID;
    float3 ip = ray.get_origin() + make_float3(ray.get_direction().x * min_thit, ray.get_direction().y * min_thit,
                                                ray.get_direction().z * min_thit);
    h.intersection_point[0] = ip.x, h.intersection_point[1] = ip.y, h.intersection_point[2] = ip.z;
    h.world_min_thit = min_thit;
    float3 p[3];
    for (int i = 0; i < 3; i++) p[i] = closest_leaf.QuadVertex[i];
    float3 oip = closest_objectRay.get_origin() + make_float3(closest_objectRay.get_direction().x * min_thit_object,
                                                              closest_objectRay.get_direction().y * min_thit_object,
                                                              closest_objectRay.get_direction().z * min_thit_object);
    float3 b = Barycentric(oip, p[0], p[1], p[2]);
    h.barycentric[0] = b.x, h.barycentric[1] = b.y, h.barycentric[2] = b.z;
    h.closest_leaf = unit_of(base, closest_leaf_addr);
    h.closest_instance = unit_of(base, closest_inst_addr);
  }
  h.n_visits = (uint32_t)o.transactions.size();
}

// traceRay (vulkan_ray_tracing.cc:2309-3076), device_offset = 0, no remap.
void trace_plain(const uint8_t* tlas, uint32_t rayFlags, float3 origin, float Tmin, float3 direction, float Tmax,
                 TraceOut& out) {
  const bool terminateOnFirstHit = rayFlags & RT_RAY_FLAG_TERMINATE_ON_FIRST_HIT;
  const bool skipAnyHitShader = rayFlags & RT_RAY_FLAG_OPAQUE;
  auto& transactions = out.transactions;
  bool hit_procedural = false;
  Ray ray;
  ray.make_ray(origin, direction, Tmin, Tmax);
  float min_thit = ray.dir_tmax.w;
  GEN_RT_BVH_QUAD_LEAF closest_leaf{};
  GEN_RT_BVH_INSTANCE_LEAF closest_instanceLeaf{};
  Ray closest_objectRay{};
  float min_thit_object = 0;
  const uint8_t *closest_leaf_addr = tlas, *closest_inst_addr = tlas;

  GEN_RT_BVH topBVH;
  unpack_bvh(&topBVH, tlas);
  transactions.push_back({tlas, RT_TX_STRUCTURE});
  const uint8_t* topRootAddr = tlas + topBVH.RootNodeOffset;
  std::list<StackEntry> stack;
  {
    float thit;
    if (ray_box_test(topBVH.BoundsMin, topBVH.BoundsMax, calculate_idir(ray.get_direction()), ray.get_origin(),
                     ray.get_tmin(), ray.get_tmax(), thit))
      { stack.push_back(StackEntry(topRootAddr, true, false)); out.note(0, stack.size()); }
  }
  while (!stack.empty()) {  // :2486
    const uint8_t* next_node_addr = nullptr;
    if (!stack.back().leaf) {
      next_node_addr = stack.back().addr;
      stack.pop_back();
    }
    while (next_node_addr != nullptr) {  // :2500-2599
      const uint8_t* node_addr = next_node_addr;
      next_node_addr = nullptr;
      GEN_RT_BVH_INTERNAL_NODE node;
      unpack_internal(&node, node_addr);
      transactions.push_back({node_addr, RT_TX_INTERNAL_NODE});
      bool child_hit[6];
      float thit[6];
      for (int i = 0; i < 6; i++) {
        if (node.ChildSize[i] > 0) {
          float3 idir = calculate_idir(ray.get_direction());
          float3 lo, hi;
          set_child_bounds(&node, i, &lo, &hi);
          child_hit[i] = ray_box_test(lo, hi, idir, ray.get_origin(), ray.get_tmin(), ray.get_tmax(), thit[i]);
          if (child_hit[i] && thit[i] >= min_thit) child_hit[i] = false;
        } else
          child_hit[i] = false;
      }
      const uint8_t* child_addr = node_addr + (node.ChildOffset * 64);
      for (int i = 0; i < 6; i++) {
        if (child_hit[i]) {
          if (node.ChildType[i] != NODE_TYPE_INTERNAL)
            { stack.push_back(StackEntry(child_addr, true, true)); out.note(0, stack.size()); }
          else if (next_node_addr == nullptr)
            next_node_addr = child_addr;
          else
            { stack.push_back(StackEntry(child_addr, true, false)); out.note(0, stack.size()); }
        }
        child_addr += node.ChildSize[i] * 64;
      }
    }
    while (!stack.empty() && stack.back().leaf) {  // :2602
      const uint8_t* leaf_addr = stack.back().addr;
      stack.pop_back();
      GEN_RT_BVH_INSTANCE_LEAF instanceLeaf;
      unpack_instance(&instanceLeaf, leaf_addr);
      transactions.push_back({leaf_addr, RT_TX_INSTANCE_LEAF});
      float4x4 worldToObjectMatrix = instance_leaf_matrix_to_float4x4(instanceLeaf.w2o_run);
      GEN_RT_BVH botLevelASAddr;
      unpack_bvh(&botLevelASAddr, leaf_addr + instanceLeaf.BVHAddress);
      const uint8_t* blasHdr = leaf_addr + instanceLeaf.BVHAddress;
      transactions.push_back({blasHdr, RT_TX_STRUCTURE});
      float worldToObject_tMultiplier;
      Ray objectRay = make_transformed_ray(ray, worldToObjectMatrix, &worldToObject_tMultiplier);
      { stack.push_back(StackEntry(blasHdr + botLevelASAddr.RootNodeOffset, false, false)); out.note(0, stack.size()); }
      while (!stack.empty() && !stack.back().topLevel) {  // :2679
        const uint8_t* nnext = stack.back().addr;
        stack.pop_back();
        while (nnext != nullptr) {
          const uint8_t* node_addr = nnext;
          nnext = nullptr;
          GEN_RT_BVH_INTERNAL_NODE node;
          unpack_internal(&node, node_addr);
          transactions.push_back({node_addr, RT_TX_INTERNAL_NODE});
          bool child_hit[6];
          float thit[6];
          for (int i = 0; i < 6; i++) {
            if (node.ChildSize[i] > 0) {
              float3 idir = calculate_idir(objectRay.get_direction());
              float3 lo, hi;
              set_child_bounds(&node, i, &lo, &hi);
              child_hit[i] = ray_box_test(lo, hi, idir, objectRay.get_origin(), objectRay.get_tmin(),
                                          objectRay.get_tmax(), thit[i]);
              if (child_hit[i] && thit[i] >= min_thit * worldToObject_tMultiplier) child_hit[i] = false;
            } else
              child_hit[i] = false;
          }
          const uint8_t* child_addr = node_addr + (node.ChildOffset * 64);
          for (int i = 0; i < 6; i++) {
            if (child_hit[i]) {
              if (node.ChildType[i] != NODE_TYPE_INTERNAL)
                { stack.push_back(StackEntry(child_addr, false, true)); out.note(0, stack.size()); }
              else if (nnext == nullptr)
                nnext = child_addr;
              else
                { stack.push_back(StackEntry(child_addr, false, false)); out.note(0, stack.size()); }
            }
            child_addr += node.ChildSize[i] * 64;
          }
        }
        while (!stack.empty() && !stack.back().topLevel && stack.back().leaf) {  // :2789
          const uint8_t* leaf = stack.back().addr;
          stack.pop_back();
          GEN_RT_BVH_PRIMITIVE_LEAF_DESCRIPTOR desc;
          unpack_desc(&desc, leaf);
          transactions.push_back({leaf, RT_TX_LEAF_DESCRIPTOR});
          if (desc.LeafType == TYPE_QUAD) {
            GEN_RT_BVH_QUAD_LEAF q;
            unpack_quad(&q, leaf);
            float thit = 0;
            bool hit = mt_ray_triangle_test(q.QuadVertex[0], q.QuadVertex[1], q.QuadVertex[2], objectRay, &thit);
            float world_thit = thit / worldToObject_tMultiplier;
            if (hit && Tmin <= world_thit && world_thit <= Tmax) {  // :2843
              if (skipAnyHitShader && world_thit < min_thit) min_thit = thit / worldToObject_tMultiplier;
              min_thit_object = thit;
              closest_leaf = q;
              closest_instanceLeaf = instanceLeaf;
              closest_objectRay = objectRay;
              closest_leaf_addr = leaf;
              closest_inst_addr = leaf_addr;
              transactions.push_back({leaf, RT_TX_QUAD_LEAF_HIT});
              // Non-opaque rays also go to the any-hit table (:2869-2930):
              // shader dispatch, not restated.
              if (terminateOnFirstHit) stack.clear();
            } else {
              transactions.push_back({leaf, RT_TX_QUAD_LEAF});
            }
          } else {
            hit_procedural = true;
            transactions.push_back({leaf, RT_TX_PROCEDURAL_LEAF});
          }
        }
      }
    }
  }
  finish_hit(out, min_thit < ray.dir_tmax.w, min_thit, ray, closest_leaf, closest_instanceLeaf, closest_objectRay,
             min_thit_object, tlas, closest_leaf_addr, closest_inst_addr);
  if (hit_procedural) out.hit.status |= RT_RAY_HIT_PROCEDURAL;
}

// traceRayWithTreelets (vulkan_ray_tracing.cc:1522-2307), no remap.
// offset_quirk = false: device_offset = 0.  offset_quirk = true: a nonzero
// device_offset.  current_treelet_root starts as a device address (:1707)
// but is then set from a stack entry's host address (:1752), while every
// comparison looks up the child's device address (addrToTreeletID(child_addr
// + device_offset), :1821-1856, :1925-1936, :2015-2046); after the first pop
// no comparison can match, and every child goes to other_treelet_stack.
void trace_treelets(const uint8_t* tlas, const oracle_treelets& T, uint32_t rayFlags, float3 origin, float Tmin,
                    float3 direction, float Tmax, TraceOut& out, bool offset_quirk) {
  const bool terminateOnFirstHit = rayFlags & RT_RAY_FLAG_TERMINATE_ON_FIRST_HIT;
  auto& transactions = out.transactions;
  bool hit_procedural = false;
  Ray ray;
  ray.make_ray(origin, direction, Tmin, Tmax);
  float min_thit = ray.dir_tmax.w;
  GEN_RT_BVH_QUAD_LEAF closest_leaf{};
  GEN_RT_BVH_INSTANCE_LEAF closest_instanceLeaf{};
  Ray closest_objectRay{};
  float min_thit_object = 0;
  const uint8_t *closest_leaf_addr = tlas, *closest_inst_addr = tlas;

  GEN_RT_BVH topBVH;
  unpack_bvh(&topBVH, tlas);
  transactions.push_back({tlas, RT_TX_STRUCTURE});
  const uint8_t* topRootAddr = tlas + topBVH.RootNodeOffset;
  const uint8_t* current_treelet_root = tlas;  // :1707
  bool root_is_device_address = true;           // false once :1752 stores a host address (offset_quirk)
  std::list<StackEntry> current_treelet_stack, other_treelet_stack;
  {
    float thit;
    if (ray_box_test(topBVH.BoundsMin, topBVH.BoundsMax, calculate_idir(ray.get_direction()), ray.get_origin(),
                     ray.get_tmin(), ray.get_tmax(), thit)) {
      if (current_treelet_root == T.addrToTreeletID(topRootAddr))
        current_treelet_stack.push_back(StackEntry(topRootAddr, true, false));
      else
        other_treelet_stack.push_back(StackEntry(topRootAddr, true, false));
      out.note(0, current_treelet_stack.size());
      out.note(1, other_treelet_stack.size());
    }
  }
  auto route = [&](const StackEntry& e) {
    if (root_is_device_address && current_treelet_root == T.addrToTreeletID(e.addr)) {
      current_treelet_stack.push_front(e);
      out.note(0, current_treelet_stack.size());
    } else {
      other_treelet_stack.push_front(e);
      out.note(1, other_treelet_stack.size());
    }
  };
  while (!current_treelet_stack.empty() || !other_treelet_stack.empty()) {  // :1740
    if (current_treelet_stack.empty()) {  // :1748-1754
      current_treelet_stack.push_front(other_treelet_stack.front());
      current_treelet_root = other_treelet_stack.front().addr;
      if (offset_quirk) root_is_device_address = false;
      other_treelet_stack.pop_front();
    }
    StackEntry cur = current_treelet_stack.front();
    current_treelet_stack.pop_front();
    if (cur.topLevel && !cur.leaf) {  // :1758-1869
      GEN_RT_BVH_INTERNAL_NODE node;
      unpack_internal(&node, cur.addr);
      transactions.push_back({cur.addr, RT_TX_INTERNAL_NODE});
      bool child_hit[6];
      float thit[6];
      for (int i = 0; i < 6; i++) {
        if (node.ChildSize[i] > 0) {
          float3 idir = calculate_idir(ray.get_direction());
          float3 lo, hi;
          set_child_bounds(&node, i, &lo, &hi);
          child_hit[i] = ray_box_test(lo, hi, idir, ray.get_origin(), ray.get_tmin(), ray.get_tmax(), thit[i]);
          if (child_hit[i] && thit[i] >= min_thit) child_hit[i] = false;
        } else
          child_hit[i] = false;
      }
      const uint8_t* child_addr = cur.addr + (node.ChildOffset * 64);
      for (int i = 0; i < 6; i++) {
        if (child_hit[i]) {
          if (node.ChildType[i] != NODE_TYPE_INTERNAL)
            route(StackEntry(child_addr, true, true));
          else
            route(StackEntry(child_addr, true, false));
        }
        child_addr += node.ChildSize[i] * 64;
      }
    } else if (cur.topLevel && cur.leaf) {  // :1870-1953
      const uint8_t* leaf_addr = cur.addr;
      GEN_RT_BVH_INSTANCE_LEAF instanceLeaf;
      unpack_instance(&instanceLeaf, leaf_addr);
      transactions.push_back({leaf_addr, RT_TX_INSTANCE_LEAF});
      float4x4 w2o = instance_leaf_matrix_to_float4x4(instanceLeaf.w2o_run);
      float4x4 o2w = instance_leaf_matrix_to_float4x4(instanceLeaf.o2w_run);
      GEN_RT_BVH bot;
      unpack_bvh(&bot, leaf_addr + instanceLeaf.BVHAddress);
      transactions.push_back({leaf_addr + instanceLeaf.BVHAddress, RT_TX_STRUCTURE});
      float mult;
      Ray objectRay = make_transformed_ray(ray, w2o, &mult);
      StackEntry e(leaf_addr + instanceLeaf.BVHAddress + bot.RootNodeOffset, false, false);
      e.worldToObject_tMultiplier = mult;
      e.instanceLeaf = instanceLeaf;
      e.worldToObjectMatrix = w2o;
      e.objectToWorldMatrix = o2w;
      e.objectRay = objectRay;
      e.instAddr = leaf_addr;
      route(e);
    } else if (!cur.topLevel && !cur.leaf) {  // :1954-2070
      GEN_RT_BVH_INTERNAL_NODE node;
      unpack_internal(&node, cur.addr);
      transactions.push_back({cur.addr, RT_TX_INTERNAL_NODE});
      bool child_hit[6];
      float thit[6];
      for (int i = 0; i < 6; i++) {
        if (node.ChildSize[i] > 0) {
          float3 idir = calculate_idir(cur.objectRay.get_direction());
          float3 lo, hi;
          set_child_bounds(&node, i, &lo, &hi);
          child_hit[i] = ray_box_test(lo, hi, idir, cur.objectRay.get_origin(), cur.objectRay.get_tmin(),
                                      cur.objectRay.get_tmax(), thit[i]);
          if (child_hit[i] && thit[i] >= min_thit * cur.worldToObject_tMultiplier) child_hit[i] = false;
        } else
          child_hit[i] = false;
      }
      const uint8_t* child_addr = cur.addr + (node.ChildOffset * 64);
      for (int i = 0; i < 6; i++) {
        if (child_hit[i]) {
          StackEntry e = cur;
          e.addr = child_addr;
          e.leaf = node.ChildType[i] != NODE_TYPE_INTERNAL;
          route(e);
        }
        child_addr += node.ChildSize[i] * 64;
      }
    } else {  // :2071-2196
      const uint8_t* leaf_addr = cur.addr;
      GEN_RT_BVH_PRIMITIVE_LEAF_DESCRIPTOR desc;
      unpack_desc(&desc, leaf_addr);
      transactions.push_back({leaf_addr, RT_TX_LEAF_DESCRIPTOR});
      if (desc.LeafType == TYPE_QUAD) {
        GEN_RT_BVH_QUAD_LEAF q;
        unpack_quad(&q, leaf_addr);
        float thit = 0;
        bool hit = mt_ray_triangle_test(q.QuadVertex[0], q.QuadVertex[1], q.QuadVertex[2], cur.objectRay, &thit);
        float world_thit = thit / cur.worldToObject_tMultiplier;
        if (hit && Tmin <= world_thit && world_thit <= Tmax && world_thit < min_thit) {  // :2127
          min_thit = thit / cur.worldToObject_tMultiplier;
          min_thit_object = thit;
          closest_leaf = q;
          closest_instanceLeaf = cur.instanceLeaf;
          closest_objectRay = cur.objectRay;
          closest_leaf_addr = leaf_addr;
          closest_inst_addr = cur.instAddr;
          transactions.push_back({leaf_addr, RT_TX_QUAD_LEAF_HIT});
          if (terminateOnFirstHit) {
            current_treelet_stack.clear();
            other_treelet_stack.clear();
          }
        } else {
          transactions.push_back({leaf_addr, RT_TX_QUAD_LEAF});
        }
      } else {
        hit_procedural = true;
        transactions.push_back({leaf_addr, RT_TX_PROCEDURAL_LEAF});
      }
    }
  }
  finish_hit(out, min_thit < ray.dir_tmax.w, min_thit, ray, closest_leaf, closest_instanceLeaf, closest_objectRay,
             min_thit_object, tlas, closest_leaf_addr, closest_inst_addr);
  if (hit_procedural) out.hit.status |= RT_RAY_HIT_PROCEDURAL;
}

void trace_range(const uint8_t* blob, const oracle_treelets* tl, const rt_ray* rays, const uint32_t* flags,
                 uint32_t default_flags, uint64_t begin, uint64_t end, int mode, rt_hit* hits, uint32_t* visits,
                 uint32_t* treelets, uint32_t capacity, uint32_t* peaks) {
  TraceOut o;
  for (uint64_t r = begin; r < end; ++r) {
    o.transactions.clear();
    o.peak[0] = o.peak[1] = 0;
    const rt_ray& ry = rays[r];
    const uint32_t f = flags ? flags[r] : default_flags;
    const float3 org = {ry.origin[0], ry.origin[1], ry.origin[2]};
    const float3 dir = {ry.dir[0], ry.dir[1], ry.dir[2]};
    if (mode == 0)
      trace_plain(blob, f, org, ry.tmin, dir, ry.tmax, o);
    else
      trace_treelets(blob, *tl, f, org, ry.tmin, dir, ry.tmax, o, mode == 2);
    if (capacity && o.transactions.size() > capacity) o.hit.status |= RT_RAY_TRACE_OVERFLOW;
    hits[r] = o.hit;
    if (peaks) {
      peaks[2 * r] = o.peak[0];
      peaks[2 * r + 1] = o.peak[1];
    }
    const size_t m = std::min<size_t>(o.transactions.size(), capacity);
    for (size_t j = 0; j < m; ++j) {
      const Tx& t = o.transactions[j];
      if (visits) visits[r * capacity + j] = (unit_of(blob, t.address) << 3) | t.type;
      // printf("RayID,%d", ...) line of :2256-2262
      if (treelets) {
        const uint8_t* id = tl->addrToTreeletID(t.address);
        treelets[r * capacity + j] = id ? unit_of(blob, id) : 0xFFFFFFFFu;
      }
    }
  }
}

}  // namespace

extern "C" {

// The oracle's ray geometry on a batch of cases, in the case and result
// layouts of oracle/ref_pin/pin_geometry.cpp (which runs the reference's own
// functions): op 0 calculate_idir + ray_box_test, 1 mt_ray_triangle_test,
// 2 make_transformed_ray, 3 Barycentric.  Returns 0 or -1.
int oracle_geometry(int op, const float* in, uint32_t n, float* out) {
  static const int kIn[4] = {14, 17, 24, 12}, kOut[4] = {5, 2, 9, 3};
  if (op < 0 || op > 3) {
    g_err = "oracle_geometry: op must be 0..3";
    return -1;
  }
  auto f3 = [](const float* p) { return float3{p[0], p[1], p[2]}; };
  for (uint32_t k = 0; k < n; ++k) {
    const float* c = in + (size_t)k * kIn[op];
    float* o = out + (size_t)k * kOut[op];
    if (op == 0) {
      const float3 idir = calculate_idir(f3(c + 9));
      float thit = -1.0f;
      const bool hit = ray_box_test(f3(c), f3(c + 3), idir, f3(c + 6), c[12], c[13], thit);
      o[0] = idir.x, o[1] = idir.y, o[2] = idir.z, o[3] = hit ? 1.0f : 0.0f, o[4] = thit;
    } else if (op == 1) {
      Ray r;
      r.make_ray(f3(c + 9), f3(c + 12), c[15], c[16]);
      float thit = -1.0f;
      const bool hit = mt_ray_triangle_test(f3(c), f3(c + 3), f3(c + 6), r, &thit);
      o[0] = hit ? 1.0f : 0.0f, o[1] = thit;
    } else if (op == 2) {
      Ray r;
      r.make_ray(f3(c), f3(c + 4), c[3], c[7]);
      float4x4 m;
      for (int i = 0; i < 4; ++i)
        for (int j = 0; j < 4; ++j) m.m[i][j] = c[8 + 4 * i + j];
      float mult = 0.0f;
      const Ray t = make_transformed_ray(r, m, &mult);
      const float3 to = t.get_origin(), td = t.get_direction();
      const float v[9] = {to.x, to.y, to.z, td.x, td.y, td.z, t.get_tmin(), t.get_tmax(), mult};
      for (int i = 0; i < 9; ++i) o[i] = v[i];
    } else {
      const float3 b = Barycentric(f3(c), f3(c + 3), f3(c + 6), f3(c + 9));
      o[0] = b.x, o[1] = b.y, o[2] = b.z;
    }
  }
  return 0;
}

// One node decoded by the oracle's decoders, in the record layout of
// oracle/ref_pin/pin_decoders.cpp (which decodes with the reference header).
int oracle_decode_node(const uint8_t* blob, uint32_t unit, int kind, double* out) {
  const uint8_t* p = blob + (uint64_t)unit * 64;
  std::vector<double> v;
  if (kind == 0) {
    GEN_RT_BVH h;
    unpack_bvh(&h, p);
    v = {(double)h.RootNodeOffset, h.BoundsMin.x, h.BoundsMin.y, h.BoundsMin.z, h.BoundsMax.x, h.BoundsMax.y,
         h.BoundsMax.z};
  } else if (kind == 1) {
    GEN_RT_BVH_INTERNAL_NODE n;
    unpack_internal(&n, p);
    v = {n.Origin.x, n.Origin.y, n.Origin.z, (double)n.ChildOffset, (double)n.NodeType,
         (double)n.ChildBoundsExponentX, (double)n.ChildBoundsExponentY, (double)n.ChildBoundsExponentZ,
         (double)n.NodeRayMask};
    for (int i = 0; i < 6; ++i) v.push_back(n.ChildSize[i]);
    for (int i = 0; i < 6; ++i) v.push_back(n.ChildType[i]);
    for (int i = 0; i < 6; ++i) {
      float3 lo, hi;
      set_child_bounds(&n, i, &lo, &hi);
      v.insert(v.end(), {lo.x, lo.y, lo.z, hi.x, hi.y, hi.z});
    }
  } else if (kind == 2) {
    GEN_RT_BVH_INSTANCE_LEAF l;
    unpack_instance(&l, p);
    const float4x4 w2o = instance_leaf_matrix_to_float4x4(l.w2o_run);
    const float4x4 o2w = instance_leaf_matrix_to_float4x4(l.o2w_run);
    v = {(double)l.ShaderIndex, (double)l.GeometryRayMask, (double)l.InstanceContributionToHitGroupIndex,
         (double)l.LeafType, (double)l.GeometryFlags, (double)l.InstanceFlags, (double)l.BVHAddress,
         (double)l.InstanceID, (double)l.InstanceIndex};
    for (int a = 0; a < 4; ++a)
      for (int b = 0; b < 4; ++b) v.push_back(w2o.m[a][b]);
    for (int a = 0; a < 4; ++a)
      for (int b = 0; b < 4; ++b) v.push_back(o2w.m[a][b]);
    const float4 q = w2o * float4{0.5f, -1.25f, 2.0f, 1.0f};
    const float4 d = w2o * float4{0.25f, 0.75f, -0.5f, 0.0f};
    v.insert(v.end(), {q.x, q.y, q.z, q.w, d.x, d.y, d.z, d.w});
  } else if (kind == 3) {
    GEN_RT_BVH_QUAD_LEAF q;
    unpack_quad(&q, p);
    v = {(double)q.LeafDescriptor.ShaderIndex, (double)q.LeafDescriptor.GeometryRayMask,
         (double)q.LeafDescriptor.GeometryIndex, (double)q.LeafDescriptor.LeafType,
         (double)q.LeafDescriptor.GeometryFlags, (double)q.PrimitiveIndex0, (double)q.PrimitiveIndex1Delta,
         (double)q.j0, (double)q.j1, (double)q.j2};
    for (int k = 0; k < 4; ++k) v.insert(v.end(), {q.QuadVertex[k].x, q.QuadVertex[k].y, q.QuadVertex[k].z});
  } else {
    g_err = "oracle_decode_node: unknown kind";
    return -1;
  }
  for (int i = 0; i < 62; ++i) out[i] = i < (int)v.size() ? v[i] : 0.0;
  return 0;
}

const char* oracle_last_error(void) { return g_err.c_str(); }

oracle_treelets* oracle_form_treelets(const uint8_t* blob, uint64_t n_bytes, int max_bytes) {
  (void)n_bytes;
  auto* t = new oracle_treelets();
  t->base = blob;
  if (!create_treelets(blob, max_bytes, t)) {
    delete t;
    return nullptr;
  }
  return t;
}

void oracle_treelets_free(oracle_treelets* t) { delete t; }

void oracle_treelets_sizes(const oracle_treelets* t, uint32_t* n_treelets, uint64_t* n_members) {
  uint64_t m = 0;
  for (auto& kv : t->roots) m += kv.second.size();
  if (n_treelets) *n_treelets = (uint32_t)t->roots.size();
  if (n_members) *n_members = m;
}

void oracle_treelets_get(const oracle_treelets* t, uint64_t n_units, uint32_t* roots, uint64_t* member_first,
                         uint32_t* members, uint16_t* member_bytes, uint32_t* node_root) {
  uint32_t k = 0;
  uint64_t j = 0;
  if (member_first) member_first[0] = 0;
  for (auto& kv : t->roots) {
    if (roots) roots[k] = unit_of(t->base, kv.first);
    for (auto& e : kv.second) {
      if (members) members[j] = unit_of(t->base, e.addr);
      if (member_bytes) member_bytes[j] = (uint16_t)e.size;
      ++j;
    }
    ++k;
    if (member_first) member_first[k] = j;
  }
  if (node_root) {
    for (uint64_t u = 0; u < n_units; ++u) node_root[u] = 0xFFFFFFFFu;
    for (auto& kv : t->node_map) node_root[unit_of(t->base, kv.first)] = unit_of(t->base, kv.second);
  }
}

int oracle_remap(const oracle_treelets* t, int max_bytes, uint32_t stride, uint64_t n_units, uint64_t* new_addr) {
  // remapBVHToTreeletLayout (:1473-1509), addresses relative to the new layout's base.
  std::map<const uint8_t*, uint64_t> mapping;
  uint64_t i = 0;
  for (auto& root : t->roots) {
    const uint64_t new_root = i * ((uint64_t)max_bytes + stride);
    if (mapping.count(root.first)) {
      g_err = "remapBVHToTreeletLayout asserts: root already mapped";
      return -1;
    }
    mapping[root.first] = new_root;
    uint64_t new_node = new_root + (uint64_t)t->root_size.at(root.first);
    for (auto& node : root.second) {
      if (node.addr != root.first) {
        if (mapping.count(node.addr) == 0) mapping[node.addr] = new_node;
        new_node += node.size;
      }
    }
    i++;
  }
  for (uint64_t u = 0; u < n_units; ++u) new_addr[u] = ~0ull;
  for (auto& kv : mapping) new_addr[unit_of(t->base, kv.first)] = kv.second;
  return 0;
}

int oracle_trace(const uint8_t* blob, uint64_t n_bytes, const oracle_treelets* tl, const rt_ray* rays,
                 const uint32_t* flags, uint32_t default_flags, uint64_t n, int mode, rt_hit* hits, uint32_t* visits,
                 uint32_t* treelets, uint32_t capacity, int threads) {
  return oracle_trace_peaks(blob, n_bytes, tl, rays, flags, default_flags, n, mode, hits, visits, treelets, capacity,
                            nullptr, threads);
}

int oracle_trace_peaks(const uint8_t* blob, uint64_t n_bytes, const oracle_treelets* tl, const rt_ray* rays,
                       const uint32_t* flags, uint32_t default_flags, uint64_t n, int mode, rt_hit* hits,
                       uint32_t* visits, uint32_t* treelets, uint32_t capacity, uint32_t* peaks, int threads) {
  (void)n_bytes;
  if (mode < 0 || mode > 2) {
    g_err = "oracle_trace: mode must be 0, 1 or 2";
    return -1;
  }
  if ((mode != 0 || treelets) && !tl) {
    g_err = "oracle_trace: treelets required";
    return -1;
  }
  if (!visits && !treelets) capacity = 0;
  if (threads <= 1 || n < 256) {
    trace_range(blob, tl, rays, flags, default_flags, 0, n, mode, hits, visits, treelets, capacity, peaks);
    return 0;
  }
  std::vector<std::thread> th;
  const uint64_t chunk = (n + threads - 1) / threads;
  for (int t = 0; t < threads; ++t) {
    const uint64_t b = std::min<uint64_t>(n, t * chunk), e = std::min<uint64_t>(n, b + chunk);
    th.emplace_back(trace_range, blob, tl, rays, flags, default_flags, b, e, mode, hits, visits, treelets, capacity,
                    peaks);
  }
  for (auto& x : th) x.join();
  return 0;
}

// One RT unit, one decision.  queue_variant 0: the decision block of
// rt_unit::cycle (shader.cc:3419-3683).  1: the copy that the pipelined
// treelet queue runs (shader.cc:3780-3932), which has no second-prefetch rule,
// suppresses only a repeat of the last prefetched treelet, and sizes
// heuristic 3 at half the treelet instead of its popularity.  2: the copy the
// treelet queue runs (shader.cc:4020-4060): the whole most popular treelet,
// whatever the heuristic, unless it was the last one prefetched.  flush: the
// queue is cleared before a new treelet's chunks are queued
// (-flush_prefetch_queue_on_new_treelet, :3579-3583 and :3894-3898; the
// treelet queue's copy has no such step).
int oracle_prefetch_decide_ex(const oracle_treelets* tl, const uint32_t* next_unit, uint32_t lanes,
                              const rt_prefetch_params* p, rt_prefetch_state* st, rt_prefetch_decision* out,
                              uint32_t queue_variant, uint32_t flush) {
  const uint8_t* NONE = nullptr;
  auto to_ptr = [&](uint32_t u) -> const uint8_t* { return u == 0xFFFFFFFFu ? nullptr : tl->base + (uint64_t)u * 64; };
  auto to_unit = [&](const uint8_t* a) -> uint32_t { return a ? unit_of(tl->base, a) : 0xFFFFFFFFu; };
  const uint8_t* last_prefetched = to_ptr(st->last_prefetched);
  const uint8_t* last_second = to_ptr(st->last_prefetched_second);
  const uint8_t* last_rejected = to_ptr(st->last_rejected);
  uint64_t queue = st->queue_len;
  std::memset(out, 0, sizeof(*out));
  out->treelet = out->second_treelet = 0xFFFFFFFFu;

  const uint8_t* prefetched_treelet_root = NONE;
  const uint8_t* second_prefetched_treelet_root = NONE;
  std::map<const uint8_t*, int> priority;  // treelet_prefetch_priority
  for (uint32_t i = 0; i < lanes; ++i)
    if (next_unit[i] != 0xFFFFFFFFu) priority[tl->addrToTreeletID(to_ptr(next_unit[i]))] += 1;
  bool submit = false;
  int num_nodes_to_prefetch = 0;
  int max = -1;
  unsigned total_threads = 0;
  for (auto& kv : priority) {
    if (kv.second > max) {
      prefetched_treelet_root = kv.first;
      max = kv.second;
    }
    total_threads += kv.second;
  }
  auto members_of = [&](const uint8_t* r) -> const std::vector<StackEntry>* {
    auto it = tl->roots.find(r);
    return it == tl->roots.end() ? nullptr : &it->second;
  };
  if (queue_variant == 2) {  // the treelet queue's copy (shader.cc:4020-4060)
    // no heuristic, no rejected treelet, no second prefetch, no flush: the
    // whole most popular treelet unless it was the last one prefetched.  An
    // empty histogram names no treelet, whose member list is empty, so the
    // block then queues nothing but still records "no treelet" as the last
    // prefetched one.
    out->treelet = to_unit(prefetched_treelet_root);
    out->count = prefetched_treelet_root ? (uint32_t)priority[prefetched_treelet_root] : 0;
    out->total = total_threads;
    if (last_prefetched != prefetched_treelet_root) {
      const auto* nodes = prefetched_treelet_root ? members_of(prefetched_treelet_root) : nullptr;
      const int n_nodes = nodes ? (int)nodes->size() : 0;
      if ((uint64_t)n_nodes + queue <= p->max_queue) {
        uint32_t chunks = 0;
        for (int j = 0; j < n_nodes; ++j) chunks += ((*nodes)[j].size + 31) / 32;
        queue += chunks;
        out->submitted = prefetched_treelet_root ? 1 : 0;
        out->n_members = (uint32_t)n_nodes;
        out->chunks = chunks;
        last_prefetched = prefetched_treelet_root;
      }
    }
    st->last_prefetched = to_unit(last_prefetched);
    st->queue_len = (uint32_t)queue;
    return 0;
  }
  if (p->heuristic == 0) {
    submit = true;
  } else if (prefetched_treelet_root != NONE) {
    const double percentage = (double)priority[prefetched_treelet_root] / (double)total_threads;
    if (p->heuristic == 1) {
      if (percentage >= p->threshold) {
        last_rejected = NONE;
        submit = true;
      } else {
        if (last_rejected != prefetched_treelet_root) last_rejected = prefetched_treelet_root;
        submit = false;
      }
    } else {
      const auto* m = members_of(prefetched_treelet_root);
      const int n = m ? (int)m->size() : 0;
      const double share = (queue_variant && p->heuristic == 3) ? 0.5 : percentage;
      num_nodes_to_prefetch = (int)(((double)n * share) + 0.5);
      submit = true;
    }
  }
  out->treelet = to_unit(prefetched_treelet_root);
  out->count = prefetched_treelet_root ? (uint32_t)priority[prefetched_treelet_root] : 0;
  out->total = total_threads;
  if (submit && prefetched_treelet_root != NONE) {  // :3562-3640
    const auto* nodes = members_of(prefetched_treelet_root);
    const int n_nodes = nodes ? (int)nodes->size() : 0;
    if (last_prefetched != prefetched_treelet_root && (queue_variant || last_second != prefetched_treelet_root)) {
      const int num = (p->heuristic == 2 || p->heuristic == 3) ? num_nodes_to_prefetch : n_nodes;
      if ((uint64_t)num + queue <= p->max_queue) {
        if (flush) queue = 0;
        const int j0 = (p->heuristic == 3) ? n_nodes - num : 0;
        const int j1 = (p->heuristic == 3) ? n_nodes : num;
        uint32_t chunks = 0;
        for (int j = j0; j < j1; ++j) chunks += ((*nodes)[j].size + 31) / 32;
        queue += chunks;
        out->submitted = 1;
        out->first_member = (uint32_t)j0;
        out->n_members = (uint32_t)(j1 - j0);
        out->chunks = chunks;
        last_prefetched = prefetched_treelet_root;
      }
    }
  }
  if (p->second_prefetch && !queue_variant) {  // :3645-3683
    bool submit_second = false;
    if (queue == 0 && total_threads > 0 && priority.size() > 1) {
      if (last_prefetched == prefetched_treelet_root && prefetched_treelet_root != NONE) {
        int mx = -1;
        for (auto& kv : priority)
          if (kv.second > mx && kv.first != last_prefetched) {
            second_prefetched_treelet_root = kv.first;
            mx = kv.second;
          }
        submit_second = true;
      }
    }
    if (submit_second && second_prefetched_treelet_root != NONE && last_second != second_prefetched_treelet_root) {
      const auto* nodes = members_of(second_prefetched_treelet_root);
      uint32_t chunks = 0;
      if (nodes)
        for (auto& e : *nodes) chunks += (e.size + 31) / 32;
      queue += chunks;
      out->chunks += chunks;
      out->second_treelet = to_unit(second_prefetched_treelet_root);
      last_second = second_prefetched_treelet_root;
    }
  }
  st->last_prefetched = to_unit(last_prefetched);
  st->last_prefetched_second = to_unit(last_second);
  st->last_rejected = to_unit(last_rejected);
  st->queue_len = (uint32_t)queue;
  return 0;
}

// shader.cc:3419-3683, one RT unit, one decision.
int oracle_prefetch_decide(const oracle_treelets* tl, const uint32_t* next_unit, uint32_t lanes,
                           const rt_prefetch_params* p, rt_prefetch_state* st, rt_prefetch_decision* out) {
  return oracle_prefetch_decide_ex(tl, next_unit, lanes, p, st, out, 0, 0);
}

}  // extern "C"

// ---------------------------------------------------------------- RT-unit replay

namespace {

enum Effectiveness { E_TOO_LATE = 0, E_LATE, E_TIMELY, E_TOO_EARLY, E_NEVER_USED, E_UNCLASSIFIED };

struct PrefetchRecord {  // prefetch_block_info (gpu-cache.h:99-113), the fields the classification reads
  uint64_t block;        // 32 B sector address (the sector cache's MSHR address)
  int effectiveness = E_UNCLASSIFIED;
};

// The end-of-run tally of one RT unit's prefetch records (gpu-sim.cc:
// 1749-1795): records are grouped by block address; in a block where some
// record was classified (anything but UNCLASSIFIED and NEVER_USED), the
// unclassified ones count as "unclassified but accessed" and the rest by
// class; in a block where none was, the unclassified ones become NEVER_USED
// and all count by class.
template <class Rec, class Count>
void tally_records(std::vector<Rec>& records, Count* effectiveness, Count& unclassified_but_accessed) {
  std::map<uint64_t, std::vector<Rec*>> by_block;
  for (auto& r : records) by_block[r.block].push_back(&r);
  for (auto& kv : by_block) {
    bool accessed = false;
    for (auto* r : kv.second)
      if (r->effectiveness != E_UNCLASSIFIED && r->effectiveness != E_NEVER_USED) accessed = true;
    for (auto* r : kv.second) {
      if (accessed) {
        if (r->effectiveness == E_UNCLASSIFIED) {
          unclassified_but_accessed++;
          continue;
        }
      } else if (r->effectiveness == E_UNCLASSIFIED) {
        r->effectiveness = E_NEVER_USED;
      }
      effectiveness[r->effectiveness]++;
    }
  }
}

struct SectorState {
  bool valid = false;
  uint64_t ready = 0;  // cycle the data is there
  bool by_prefetch = false;
  int64_t record = -1;  // the prefetch record that filled it
};

struct CacheLine {
  bool used = false;
  uint64_t block = 0;  // 128 B line address
  uint64_t lru = 0;
  SectorState s[4];
};

struct Request {
  uint64_t addr, base;
  bool first_of_tx;
};

struct LaneTrace {
  const uint32_t* row = nullptr;
  uint32_t ptr = 0, end = 0;
  bool issued = false;
};

// rt_unit::schedule_next_warp (shader.cc:4307-4392) over n resident warps
// in uid order (m_current_warps is a std::map keyed by uid): `ready(i)` is
// !is_stalled(), `matches(i)` counts the warp's lanes whose next access lies
// in the last prefetched treelet.  scheduler 1 (OMR): the first ready warp
// with a match; 2 (PMR): the first ready warp with the most matches; either
// falls back, and scheduler 0 or no treelet prefetcher uses, the first ready
// warp.  Returns its position or -1.
template <class Ready, class Matches>
int pick_warp(uint32_t n, uint32_t scheduler, bool treelet_prefetch, Ready ready, Matches matches) {
  if (treelet_prefetch && scheduler == 1) {
    for (uint32_t i = 0; i < n; ++i)
      if (ready(i) && matches(i) > 0) return (int)i;
  } else if (treelet_prefetch && scheduler == 2) {
    int best = -1, best_count = 0;
    for (uint32_t i = 0; i < n; ++i)
      if (ready(i)) {
        const int c = matches(i);
        if (c > best_count) {
          best = (int)i;
          best_count = c;
        }
      }
    if (best >= 0) return best;
  }
  for (uint32_t i = 0; i < n; ++i)
    if (ready(i)) return (int)i;
  return -1;
}

// The Lee MICRO'10 stride prefetcher (shader.cc:4792-4828 as written: the last
// address is only recorded on a warp's first access, and prefetches are
// queued only while the queue holds at least max_prefetch_queue_size
// entries).  step() trains on one demand access and returns true with the
// first prefetch address when two 32-byte prefetches are queued.
struct LeeStride {
  std::map<uint32_t, std::map<int, int>> pws_table;  // warp -> stride -> count
  std::map<uint32_t, uint64_t> pws_last;
  bool step(uint32_t wid, uint64_t next_addr, uint64_t queue_size, uint64_t max_queue, uint64_t* prefetch_addr) {
    if (pws_table.count(wid) == 0) {
      pws_last[wid] = next_addr;
    } else if (pws_table[wid].size() <= 32) {
      const int stride = (int)(uint32_t)(next_addr - pws_last[wid]);
      pws_table[wid][stride]++;
    }
    int largest_stride = 0, largest_count = 0;
    for (auto& kv : pws_table[wid])
      if (kv.second > largest_count) {
        largest_stride = kv.first;
        largest_count = kv.second;
      }
    *prefetch_addr = next_addr + (uint64_t)(int64_t)largest_stride;
    return max_queue <= queue_size;
  }
};

// prefetch_mem_access_q: (request, base) pairs, with a count of the live
// copies of each request address.
struct PrefetchQueue {
  std::deque<std::pair<uint64_t, uint64_t>> q;
  std::unordered_map<uint64_t, uint32_t> live;

  // The removal of queued prefetches of a demand-loaded address
  // (shader.cc:4657-4668, 4779-4789 as written): erasing entry idx and then
  // stepping to idx + 1 skips the entry that moved into its place.  An
  // address with no live copy erases nothing, so the loop is skipped for it.
  uint32_t remove(uint64_t addr) {
    auto c = live.find(addr);
    if (c == live.end() || c->second == 0) return 0;
    uint32_t removed = 0;
    for (size_t idx = 0; idx < q.size(); idx++) {
      if (addr == q[idx].first) {
        q.erase(q.begin() + (long)idx);
        c->second--;
        removed++;
      }
    }
    return removed;
  }
  void push(uint64_t addr, uint64_t base) {
    q.emplace_back(addr, base);
    live[addr]++;
  }
  std::pair<uint64_t, uint64_t> pop() {
    const auto r = q.front();
    q.pop_front();
    live[r.first]--;
    return r;
  }
};

struct UnitWarp {
  uint32_t wid = 0;  // warp id of the stride tables
  LaneTrace lane[32];
  bool in_flight = false, all_sent = false;
  uint64_t ready = 0;
  uint32_t ilat = 0;
  bool done() const {
    for (const auto& l : lane)
      if (l.ptr < l.end) return false;
    return true;
  }
};

constexpr uint32_t kIntersectionLatency[7] = {2, 4, 4, 2, 4, 4, 4};  // -gpgpu_rt_intersection_latency

uint32_t tx_size(uint32_t type) { return type == 2 ? 128u : (type == 3 ? 8u : 64u); }

struct UnitReplay {
  const oracle_treelets* tl;
  const rt_unit_config& cfg;
  uint64_t meta_base, meta_size, n_treelets;
  std::map<const uint8_t*, int> metadata_idx;  // treelet_addr_to_metadata_idx
  rt_unit_stats st{};
  std::vector<CacheLine> lines;
  std::vector<PrefetchRecord> records;
  std::map<uint64_t, int64_t> last_evicted;  // sector -> most recently evicted prefetch record
  PrefetchQueue pq;  // prefetch_mem_access_q
  std::deque<Request> chunk_q;                 // mem_access_q of the warp being served
  UnitWarp* serving = nullptr;
  std::list<UnitWarp> resident;                // m_current_warps, oldest first
  std::deque<std::pair<uint64_t, uint64_t>> metadata_returns;  // (cycle, base)
  uint64_t most_recent_metadata = 0;
  rt_prefetch_state dstate{0xFFFFFFFFu, 0xFFFFFFFFu, 0xFFFFFFFFu, 0};
  LeeStride lee;  // Lee stride tables

  UnitReplay(const oracle_treelets* t, const rt_unit_config& c) : tl(t), cfg(c) {}

  const uint8_t* root_of_addr(uint64_t a) const { return tl->addrToTreeletID(tl->base + a); }

  CacheLine* find(uint64_t block) {
    const uint64_t set = block & (cfg.l1_sets - 1);
    for (uint32_t w = 0; w < cfg.l1_ways; ++w) {
      CacheLine& l = lines[set * cfg.l1_ways + w];
      if (l.used && l.block == block) return &l;
    }
    return nullptr;
  }

  // Allocates the line for `block` (an unused way first, else the least
  // recently used, lowest way on ties), recording evicted prefetched sectors.
  CacheLine* allocate(uint64_t block, uint64_t t) {
    const uint64_t set = block & (cfg.l1_sets - 1);
    CacheLine* victim = nullptr;
    for (uint32_t w = 0; w < cfg.l1_ways && !victim; ++w)
      if (!lines[set * cfg.l1_ways + w].used) victim = &lines[set * cfg.l1_ways + w];
    if (!victim) {
      for (uint32_t w = 0; w < cfg.l1_ways; ++w) {
        CacheLine& l = lines[set * cfg.l1_ways + w];
        if (!victim || l.lru < victim->lru) victim = &l;
      }
      for (int k = 0; k < 4; ++k)
        if (victim->s[k].valid && victim->s[k].by_prefetch) last_evicted[victim->block * 4 + k] = victim->s[k].record;
    }
    *victim = CacheLine();
    victim->used = true;
    victim->block = block;
    victim->lru = t;
    return victim;
  }

  uint64_t demand(uint64_t addr, uint64_t t) {
    const uint64_t sector = addr >> 5, block = addr >> 7;
    const int k = (int)((addr >> 5) & 3);
    st.demand_requests++;
    CacheLine* l = find(block);
    if (l && l->s[k].valid) {
      l->lru = t;
      SectorState& s = l->s[k];
      if (s.ready <= t) {  // HIT
        st.demand_hits++;
        if (s.by_prefetch && records[s.record].effectiveness == E_UNCLASSIFIED) records[s.record].effectiveness = E_TIMELY;
        return t + cfg.hit_latency;
      }
      st.demand_hit_reserved++;  // HIT_RESERVED
      if (s.by_prefetch && records[s.record].effectiveness == E_UNCLASSIFIED) records[s.record].effectiveness = E_LATE;
      return s.ready;
    }
    st.demand_misses++;  // MISS / SECTOR_MISS
    auto ev = last_evicted.find(sector);
    if (ev != last_evicted.end() && records[ev->second].effectiveness == E_UNCLASSIFIED)
      records[ev->second].effectiveness = E_TOO_EARLY;
    if (!l) l = allocate(block, t);
    l->lru = t;
    l->s[k] = SectorState{true, t + cfg.miss_latency, false, -1};
    return t + cfg.miss_latency;
  }

  void prefetch(uint64_t addr, uint64_t base, uint64_t t) {
    const uint64_t block = addr >> 7;
    const int k = (int)((addr >> 5) & 3);
    const int64_t id = (int64_t)records.size();
    records.push_back(PrefetchRecord{addr >> 5});
    st.prefetch_issued++;
    CacheLine* l = find(block);
    if (l && l->s[k].valid) {
      l->lru = t;
      if (l->s[k].ready <= t) {
        st.prefetch_present++;
        // gpu-cache.cc:2101-2116: only a record already classified becomes TOO_LATE
        if (!l->s[k].by_prefetch && records[id].effectiveness != E_UNCLASSIFIED) records[id].effectiveness = E_TOO_LATE;
      } else {
        st.prefetch_merged++;
      }
      return;
    }
    st.prefetch_filled++;
    if (!l) l = allocate(block, t);
    l->lru = t;
    l->s[k] = SectorState{true, t + cfg.miss_latency, true, id};
    if (is_metadata(base)) metadata_returns.emplace_back(t + cfg.miss_latency, base);
  }

  bool is_metadata(uint64_t base) const {
    return cfg.load_metadata && base >= meta_base && base <= meta_base + n_treelets * meta_size;
  }

  uint64_t metadata_addr(const uint8_t* root) {
    return meta_base + (uint64_t)metadata_idx[root] * meta_size;  // operator[]: 0 for a non-root
  }

  void remove_queued(uint64_t addr) { st.prefetch_removed += pq.remove(addr); }

  void enqueue(uint64_t addr, uint64_t base) {
    pq.push(addr, base);
    st.prefetch_queued++;
  }

  void push_member(const StackEntry& m, bool with_metadata) {
    if (with_metadata && cfg.load_metadata) {
      const uint64_t ma = meta_base + (uint64_t)metadata_idx[m.addr] * meta_size;
      for (uint64_t i = 0; i < meta_size / 32; ++i) {
        enqueue(ma + i * 32, ma);
        st.metadata_queued++;
      }
    }
    const uint64_t a = (uint64_t)(m.addr - tl->base);
    for (int i = 0; i < (m.size + 31) / 32; ++i) enqueue(a + 32ull * i, a);
  }

  void stride_prefetch(uint32_t wid, uint64_t next_addr) {
    uint64_t pa = 0;
    if (lee.step(wid, next_addr, pq.q.size(), cfg.decision.max_queue, &pa))
      for (unsigned i = 0; i < 2; ++i) enqueue(pa + i * 32, pa);
  }

  void decide() {
    std::vector<uint32_t> next;
    for (auto& w : resident)
      for (auto& l : w.lane) next.push_back(l.ptr < l.end ? (l.row[l.ptr] >> 3) : 0xFFFFFFFFu);
    dstate.queue_len = (uint32_t)pq.q.size();
    rt_prefetch_decision d;
    oracle_prefetch_decide(tl, next.data(), (uint32_t)next.size(), &cfg.decision, &dstate, &d);
    st.decisions++;
    if (d.submitted) {
      const auto& nodes = tl->roots.at(tl->base + (uint64_t)d.treelet * 64);
      for (uint32_t j = d.first_member; j < d.first_member + d.n_members; ++j) push_member(nodes[j], true);
      st.treelets_prefetched++;
    }
    if (d.second_treelet != 0xFFFFFFFFu) {
      for (const auto& m : tl->roots.at(tl->base + (uint64_t)d.second_treelet * 64)) push_member(m, false);
      st.treelets_prefetched++;
    }
  }

  // rt_unit::schedule_next_warp (shader.cc:4307-4392): pick_warp over the
  // resident warps, oldest (lowest uid) first.
  UnitWarp* schedule() {
    std::vector<UnitWarp*> ws;
    for (auto& w : resident) ws.push_back(&w);
    auto ready = [&](uint32_t i) { return !ws[i]->in_flight && !ws[i]->done(); };
    auto matches = [&](uint32_t i) {
      int c = 0;
      for (const auto& l : ws[i]->lane)
        if (l.ptr < l.end) {
          const uint8_t* r = root_of_addr((uint64_t)(l.row[l.ptr] >> 3) * 64);
          if (dstate.last_prefetched != 0xFFFFFFFFu && r == tl->base + (uint64_t)dstate.last_prefetched * 64) ++c;
        }
      return c;
    };
    const int k = pick_warp((uint32_t)ws.size(), cfg.scheduler, cfg.prefetcher == RT_UNIT_PF_TREELET, ready, matches);
    return k < 0 ? nullptr : ws[k];
  }

  void start_round(UnitWarp* w) {
    std::vector<std::pair<uint64_t, uint32_t>> seen;  // m_next_rt_accesses_set: (address, size)
    uint32_t ilat = 0;
    for (auto& l : w->lane) {
      l.issued = l.ptr < l.end;
      if (!l.issued) continue;
      const uint32_t v = l.row[l.ptr];
      const uint64_t a = (uint64_t)(v >> 3) * 64;
      const uint32_t size = tx_size(v & 7);
      ilat = std::max(ilat, kIntersectionLatency[v & 7]);
      bool dup = false;
      for (auto& p : seen)
        if (p.first == a && p.second == size) dup = true;
      if (dup) continue;
      seen.emplace_back(a, size);
      for (uint32_t i = 0; i < (size + 31) / 32; ++i) chunk_q.push_back(Request{a + 32ull * i, a, i == 0});
    }
    w->in_flight = true;
    w->all_sent = false;
    w->ready = 0;
    w->ilat = ilat;
    serving = w;
  }

  void send_demand(uint64_t t) {
    const Request r = chunk_q.front();
    chunk_q.pop_front();
    if (cfg.prefetcher == RT_UNIT_PF_TREELET || cfg.prefetcher == RT_UNIT_PF_STRIDE) remove_queued(r.addr);
    if (cfg.prefetcher == RT_UNIT_PF_STRIDE && r.first_of_tx) stride_prefetch(serving->wid, r.addr);
    const uint64_t ret = demand(r.addr, t);
    serving->ready = std::max(serving->ready, ret);
    if (chunk_q.empty()) {
      serving->all_sent = true;
      serving->ready += serving->ilat;
      serving = nullptr;
    }
  }

  bool prefetch_issuable() {
    const uint64_t base = pq.q.front().second;
    if (!cfg.wait_metadata || is_metadata(base)) return true;
    return most_recent_metadata == metadata_addr(root_of_addr(base));  // shader.cc:4469-4476
  }

  void run(std::vector<uint32_t> warps, const rt_hit* hits, const uint32_t* visits, uint32_t n, uint32_t capacity) {
    lines.assign((size_t)cfg.l1_sets * cfg.l1_ways, CacheLine());
    size_t next_warp = 0;
    uint32_t local = 0;
    for (uint64_t t = 0;; ++t) {
      for (auto it = resident.begin(); it != resident.end();) {
        if (it->in_flight && it->all_sent && it->ready <= t) {
          for (auto& l : it->lane)
            if (l.issued) {
              l.ptr++;
              l.issued = false;
              st.transactions++;
            }
          it->in_flight = false;
        }
        if (!it->in_flight && it->done()) {
          st.warps++;
          it = resident.erase(it);
        } else {
          ++it;
        }
      }
      while (resident.size() < cfg.max_warps && next_warp < warps.size()) {
        UnitWarp w;
        const uint32_t g = warps[next_warp++];
        w.wid = local++ % cfg.max_warps;
        for (uint32_t i = 0; i < 32; ++i) {
          const uint64_t r = (uint64_t)g * 32 + i;
          if (r < n) {
            w.lane[i].row = visits + r * capacity;
            w.lane[i].end = std::min(hits[r].n_visits, capacity);
          }
        }
        resident.push_back(w);
      }
      if (resident.empty()) {
        st.cycles = t;
        break;
      }
      if (cfg.max_cycles && t >= cfg.max_cycles) {
        st.cycles = t;
        st.status |= 2;
        break;
      }
      while (!metadata_returns.empty() && metadata_returns.front().first <= t) {
        most_recent_metadata = metadata_returns.front().second;
        metadata_returns.pop_front();
      }
      if (cfg.prefetcher == RT_UNIT_PF_TREELET && t % cfg.prefetch_delay == 0) decide();
      if (!chunk_q.empty()) {
        send_demand(t);
      } else if (UnitWarp* w = schedule()) {
        start_round(w);
        send_demand(t);
      } else if (cfg.prefetcher != RT_UNIT_PF_NONE && !pq.q.empty() && prefetch_issuable()) {
        const auto req = pq.pop();
        prefetch(req.first, req.second, t);
      }
    }
    tally_records(records, st.effectiveness, st.unclassified_but_accessed);
  }
};

}  // namespace

// rt_unit::schedule_next_warp over n resident warps (uid order): ready[i]
// = !is_stalled(), next_unit[32 i + lane] = the lane's next access (unit) or
// 0xFFFFFFFF; last_prefetched = root unit or 0xFFFFFFFF.  Returns the chosen
// position or -1.
extern "C" int oracle_schedule_warp(const oracle_treelets* tl, uint32_t scheduler, uint32_t treelet_prefetch,
                                    uint32_t last_prefetched, uint32_t n, const uint8_t* ready,
                                    const uint32_t* next_unit) {
  auto is_ready = [&](uint32_t i) { return ready[i] != 0; };
  auto matches = [&](uint32_t i) {
    int c = 0;
    for (int l = 0; l < 32; ++l) {
      const uint32_t u = next_unit[32 * i + l];
      if (u == 0xFFFFFFFFu || last_prefetched == 0xFFFFFFFFu) continue;
      if (tl->addrToTreeletID(tl->base + (uint64_t)u * 64) == tl->base + (uint64_t)last_prefetched * 64) ++c;
    }
    return c;
  };
  return pick_warp(n, scheduler, treelet_prefetch != 0, is_ready, matches);
}

// A stream of demand accesses through one Lee stride prefetcher and its
// prefetch queue, as the replay drives them.  The queue starts with `prefill`
// entries (request = base = 32 (i + 1)).  Per event k, pops[k] entries
// leave the queue front (issued), the queued copies of next_addr[k] are
// removed, and warp_id[k]'s stride tables train on next_addr[k] and may queue
// two prefetches.  out (uint64), per event: removed, appended, then per
// appended entry (request, base), then the queue length.  Returns the number
// of words written, or -1 when out_cap is too small.
extern "C" int64_t oracle_stride_events(uint32_t n, const uint32_t* warp_id, const uint64_t* next_addr,
                                        const uint32_t* pops, uint32_t max_queue, uint32_t prefill,
                                        uint64_t* out, uint64_t out_cap) {
  LeeStride lee;
  PrefetchQueue pq;
  for (uint32_t i = 0; i < prefill; ++i) pq.push(32ull * (i + 1), 32ull * (i + 1));
  uint64_t w = 0;
  for (uint32_t k = 0; k < n; ++k) {
    for (uint32_t p = 0; p < pops[k] && !pq.q.empty(); ++p) pq.pop();
    const uint32_t removed = pq.remove(next_addr[k]);
    uint64_t pa = 0;
    const bool queue = lee.step(warp_id[k], next_addr[k], pq.q.size(), max_queue, &pa);
    if (w + 8 > out_cap) return -1;
    out[w++] = removed;
    out[w++] = queue ? 2 : 0;
    if (queue)
      for (unsigned i = 0; i < 2; ++i) {
        pq.push(pa + i * 32, pa);
        out[w++] = pa + i * 32;
        out[w++] = pa;
      }
    out[w++] = pq.q.size();
  }
  return (int64_t)w;
}

// The end-of-run tally over one RT unit's n prefetch records (block address,
// class 0-5 as prefetch_request_effectiveness numbers them): out[0..4] the
// count per class, out[5] the unclassified-but-accessed count.
extern "C" void oracle_prefetch_tally(uint32_t n, const uint64_t* block, const uint8_t* effectiveness,
                                      uint64_t* out) {
  std::vector<PrefetchRecord> records(n);
  for (uint32_t i = 0; i < n; ++i) records[i] = PrefetchRecord{block[i], (int)effectiveness[i]};
  for (int k = 0; k < 6; ++k) out[k] = 0;
  tally_records(records, out, out[5]);
}

extern "C" int oracle_unit_replay(const oracle_treelets* tl, int max_treelet_bytes, uint64_t blob_bytes,
                                  const rt_hit* hits, const uint32_t* visits, uint32_t n, uint32_t capacity,
                                  const rt_unit_config* cfg, rt_unit_stats* stats, int threads) {
  if (!tl || !cfg || !stats || cfg->n_rt_units == 0 || cfg->max_warps == 0 || cfg->l1_sets == 0 ||
      cfg->l1_ways == 0 || cfg->prefetch_delay == 0) {
    fail_msg("oracle_unit_replay: bad arguments");
    return -1;
  }
  std::map<const uint8_t*, int> idx;
  int k = 0;
  for (auto& kv : tl->roots) idx[kv.first] = k++;
  const uint32_t n_warps = (n + 31) / 32;
  auto one = [&](uint32_t u) {
    UnitReplay r(tl, *cfg);
    r.meta_base = (blob_bytes + 4095) & ~4095ull;
    r.meta_size = (uint64_t)(max_treelet_bytes / 64) * 4;
    r.n_treelets = tl->roots.size();
    r.metadata_idx = idx;
    std::vector<uint32_t> warps;
    for (uint32_t w = u; w < n_warps; w += cfg->n_rt_units) warps.push_back(w);
    r.run(warps, hits, visits, n, capacity);
    stats[u] = r.st;
  };
  const int nt = std::max(1, std::min<int>(threads, (int)cfg->n_rt_units));
  std::vector<std::thread> pool;
  for (int i = 0; i < nt; ++i)
    pool.emplace_back([&, i] {
      for (uint32_t u = (uint32_t)i; u < cfg->n_rt_units; u += (uint32_t)nt) one(u);
    });
  for (auto& th : pool) th.join();
  return 0;
}
