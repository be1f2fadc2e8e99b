// Host-side BVH builder: triangle meshes + instances -> blob in the
// reference's 6-wide quantized-box layout (format.h).
#pragma once
#include <stdint.h>
#include <string>
#include <vector>

namespace rtb {

struct Mesh {
  std::vector<float> tris;  // 9 floats per triangle: v0, v1, v2
  uint32_t geometry_index = 0;
  uint32_t n() const { return (uint32_t)(tris.size() / 9); }
};

// Row-vector affine transform: world = [x y z 1] * M, M rows 0-2 linear part,
// row 3 translation (the reading convention of float4x4::operator*).
struct Instance {
  uint32_t mesh = 0;
  float o2w[4][3] = {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}, {0, 0, 0}};
  uint32_t instance_id = 0;
};

struct BuildStats {
  uint64_t internal_nodes = 0;
  uint64_t leaves = 0;
  uint64_t instance_leaves = 0;
  uint32_t max_depth = 0;
};

// Builds the whole scene: TLAS header at offset 0, TLAS nodes, then one
// header + node block per mesh.  Meshes that several instances reference are
// stored once (shared BLAS).  Returns false with a message on bad input.
bool build_scene(const std::vector<Mesh>& meshes, const std::vector<Instance>& instances,
                 std::vector<uint8_t>& blob, BuildStats* stats, std::string* err);

}  // namespace rtb
