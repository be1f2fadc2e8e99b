// Decodes every node of a blob with the REFERENCE's own decoder header
// (src/cuda-sim/vulkan_acceleration_structure_util.h, compiled unmodified
// from the reference tree) and prints one 64-value record per node, the
// golden data the oracle's decoders are pinned against.
//
// Build (oracle/ref_pin/Makefile; output only into oracle/_ref/):
//   g++ -std=c++17 -O1 -ffp-contract=off -I oracle/ref_pin/stub -I /usr/local/cuda/include \
//       -I <reference>/src/cuda-sim oracle/ref_pin/pin_decoders.cpp -o oracle/_ref/pin_decoders
// Usage: pin_decoders <blob file>   ->  stdout: binary records of 64 doubles
//   record[0] = kind (0 header, 1 internal, 2 instance leaf, 3 quad leaf), record[1] = unit
//   record[2..] = the decoded values (layout below, identical to oracle_decode_node)
#include <cstdint>
#include <cmath>
#include <vector_types.h>

#include "vulkan_acceleration_structure_util.h"

#include <cstdio>
#include <cstring>
#include <vector>

namespace {

std::vector<uint8_t> blob;

void emit(int kind, uint64_t unit, const std::vector<double>& v) {
  double rec[64] = {0};
  rec[0] = kind;
  rec[1] = (double)unit;
  for (size_t i = 0; i < v.size() && i < 62; ++i) rec[2 + i] = v[i];
  fwrite(rec, sizeof(double), 64, stdout);
}

void header(uint64_t off) {
  GEN_RT_BVH h;
  GEN_RT_BVH_unpack(&h, blob.data() + off);
  emit(0, off / 64, {(double)h.RootNodeOffset, h.BoundsMin.X, h.BoundsMin.Y, h.BoundsMin.Z, h.BoundsMax.X,
                     h.BoundsMax.Y, h.BoundsMax.Z});
}

void walk(uint64_t off, bool top, std::vector<uint8_t>& seen) {
  if (seen[off / 64]) return;
  seen[off / 64] = 1;
  GEN_RT_BVH_INTERNAL_NODE n;
  GEN_RT_BVH_INTERNAL_NODE_unpack(&n, blob.data() + off);
  std::vector<double> v = {n.Origin.X, n.Origin.Y, n.Origin.Z, (double)n.ChildOffset, (double)n.NodeType,
                           (double)n.ChildBoundsExponentX, (double)n.ChildBoundsExponentY,
                           (double)n.ChildBoundsExponentZ, (double)n.NodeRayMask};
  for (int i = 0; i < 6; ++i) v.push_back(n.ChildSize[i]);
  for (int i = 0; i < 6; ++i) v.push_back(n.ChildType[i]);
  for (int i = 0; i < 6; ++i) {
    float3 lo, hi;
    set_child_bounds(&n, i, &lo, &hi);
    v.insert(v.end(), {lo.x, lo.y, lo.z, hi.x, hi.y, hi.z});
  }
  emit(1, off / 64, v);
  uint64_t c = off + (int64_t)n.ChildOffset * 64;
  for (int i = 0; i < 6; ++i) {
    if (n.ChildSize[i] > 0) {
      if (n.ChildType[i] == NODE_TYPE_INTERNAL) {
        walk(c, top, seen);
      } else if (top) {
        if (!seen[c / 64]) {
          seen[c / 64] = 1;
          GEN_RT_BVH_INSTANCE_LEAF l;
          GEN_RT_BVH_INSTANCE_LEAF_unpack(&l, blob.data() + c);
          float4x4 w2o = instance_leaf_matrix_to_float4x4(&l.WorldToObjectm00);
          float4x4 o2w = instance_leaf_matrix_to_float4x4(&l.ObjectToWorldm00);
          std::vector<double> w = {(double)l.ShaderIndex, (double)l.GeometryRayMask,
                                   (double)l.InstanceContributionToHitGroupIndex, (double)l.LeafType,
                                   (double)l.GeometryFlags, (double)l.InstanceFlags, (double)l.BVHAddress,
                                   (double)l.InstanceID, (double)l.InstanceIndex};
          for (int a = 0; a < 4; ++a)
            for (int b = 0; b < 4; ++b) w.push_back(w2o.m[a][b]);
          for (int a = 0; a < 4; ++a)
            for (int b = 0; b < 4; ++b) w.push_back(o2w.m[a][b]);
          const float4 p = w2o * float4{0.5f, -1.25f, 2.0f, 1.0f};
          const float4 d = w2o * float4{0.25f, 0.75f, -0.5f, 0.0f};
          w.insert(w.end(), {p.x, p.y, p.z, p.w, d.x, d.y, d.z, d.w});
          emit(2, c / 64, w);
          const uint64_t hdr = c + l.BVHAddress;
          header(hdr);
          GEN_RT_BVH bh;
          GEN_RT_BVH_unpack(&bh, blob.data() + hdr);
          walk(hdr + bh.RootNodeOffset, false, seen);
        }
      } else {
        if (!seen[c / 64]) {
          seen[c / 64] = 1;
          GEN_RT_BVH_QUAD_LEAF q;
          GEN_RT_BVH_QUAD_LEAF_unpack(&q, blob.data() + c);
          std::vector<double> w = {(double)q.LeafDescriptor.ShaderIndex, (double)q.LeafDescriptor.GeometryRayMask,
                                   (double)q.LeafDescriptor.GeometryIndex, (double)q.LeafDescriptor.LeafType,
                                   (double)q.LeafDescriptor.GeometryFlags, (double)q.PrimitiveIndex0,
                                   (double)q.PrimitiveIndex1Delta, (double)q.j0, (double)q.j1, (double)q.j2};
          for (int k = 0; k < 4; ++k) w.insert(w.end(), {q.QuadVertex[k].X, q.QuadVertex[k].Y, q.QuadVertex[k].Z});
          emit(3, c / 64, w);
        }
      }
    }
    c += n.ChildSize[i] * 64;
  }
}

}  // namespace

int main(int argc, char** argv) {
  if (argc != 2) {
    fprintf(stderr, "usage: pin_decoders <blob>\n");
    return 2;
  }
  FILE* f = fopen(argv[1], "rb");
  if (!f) return 2;
  fseek(f, 0, SEEK_END);
  blob.resize((size_t)ftell(f));
  fseek(f, 0, SEEK_SET);
  if (fread(blob.data(), 1, blob.size(), f) != blob.size()) return 2;
  fclose(f);
  std::vector<uint8_t> seen(blob.size() / 64 + 1, 0);
  header(0);
  GEN_RT_BVH top;
  GEN_RT_BVH_unpack(&top, blob.data());
  walk(top.RootNodeOffset, true, seen);
  return 0;
}
