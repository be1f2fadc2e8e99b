// Runs the REFERENCE's own ray geometry on a batch of cases and prints the
// results: the golden data the oracle's geometry is pinned against.
//
// The reference functions are not copied here.  The Makefile in this folder
// extracts them, unmodified, from the reference tree into oracle/_ref/extract/
// (git-ignored) and this file includes them:
//   geom_minmax.inc   MIN / MAX / MIN_MAX / MAX_MIN    src/cuda-sim/vulkan_ray_tracing.h:53-56
//   geom_ray.inc      struct Ray                       src/abstract_hardware_model.h:333-370
//   geom_vecmath.inc  float3 / float4 operators        src/gpgpu-sim/vector-math.cc:2-82
//   geom_vrt_a.inc    get_norm .. ray_box_test         src/cuda-sim/vulkan_ray_tracing.cc:148-257
//   geom_vrt_b.inc    mt_ray_triangle_test, Barycentric src/cuda-sim/vulkan_ray_tracing.cc:3089-3130
// float4x4 comes from the reference's vulkan_acceleration_structure_util.h,
// included unmodified as for pin_decoders.
//
// Usage: pin_geometry <op> <cases file>  ->  stdout: float32 results
//   op 0 box:  case = lo3 hi3 origin3 dir3 tmin tmax (14)   -> idir3 hit thit (5)
//   op 1 tri:  case = p0 p1 p2 origin3 dir3 tmin tmax (17)  -> hit thit (2); thit is -1 unless written
//   op 2 xform: case = origin3 tmin dir3 tmax m[4][4] (24)  -> origin3 dir3 tmin tmax mult (9)
//   op 3 bary: case = p a b c (12)                          -> v w u (3)
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <vector>
#include <vector_types.h>

#include "vulkan_acceleration_structure_util.h"

#include "geom_minmax.inc"
#include "geom_ray.inc"
#include "geom_vecmath.inc"

// The two geometry functions are static members of VulkanRayTracing.
struct VulkanRayTracing {
  static bool mt_ray_triangle_test(float3 p0, float3 p1, float3 p2, Ray ray_properties, float* thit);
  static float3 Barycentric(float3 p, float3 a, float3 b, float3 c);
};

#include "geom_vrt_a.inc"
#include "geom_vrt_b.inc"

namespace {

const int kIn[4] = {14, 17, 24, 12};

float3 f3(const float* p) { return float3{p[0], p[1], p[2]}; }

void run(int op, const float* c, std::vector<float>& out) {
  if (op == 0) {
    const float3 idir = calculate_idir(f3(c + 9));
    float thit = -1.0f;
    const bool hit = ray_box_test(f3(c), f3(c + 3), idir, f3(c + 6), c[12], c[13], thit);
    out.insert(out.end(), {idir.x, idir.y, idir.z, hit ? 1.0f : 0.0f, thit});
  } else if (op == 1) {
    Ray r;
    r.make_ray(f3(c + 9), f3(c + 12), c[15], c[16]);
    float thit = -1.0f;
    const bool hit = VulkanRayTracing::mt_ray_triangle_test(f3(c), f3(c + 3), f3(c + 6), r, &thit);
    out.insert(out.end(), {hit ? 1.0f : 0.0f, thit});
  } else if (op == 2) {
    Ray r;
    r.make_ray(f3(c), f3(c + 4), c[3], c[7]);
    float4x4 m;
    for (int i = 0; i < 4; ++i)
      for (int j = 0; j < 4; ++j) m.m[i][j] = c[8 + 4 * i + j];
    float mult = 0.0f;
    const Ray t = make_transformed_ray(r, m, &mult);
    const float3 o = t.get_origin(), d = t.get_direction();
    out.insert(out.end(), {o.x, o.y, o.z, d.x, d.y, d.z, t.get_tmin(), t.get_tmax(), mult});
  } else {
    const float3 b = VulkanRayTracing::Barycentric(f3(c), f3(c + 3), f3(c + 6), f3(c + 9));
    out.insert(out.end(), {b.x, b.y, b.z});
  }
}

}  // namespace

int main(int argc, char** argv) {
  if (argc != 3) {
    fprintf(stderr, "usage: pin_geometry <op 0-3> <cases file>\n");
    return 2;
  }
  const int op = atoi(argv[1]);
  if (op < 0 || op > 3) return 2;
  FILE* f = fopen(argv[2], "rb");
  if (!f) return 2;
  std::vector<float> in;
  float buf[4096];
  size_t got;
  while ((got = fread(buf, sizeof(float), 4096, f)) > 0) in.insert(in.end(), buf, buf + got);
  fclose(f);
  if (in.size() % kIn[op]) return 2;
  std::vector<float> out;
  for (size_t k = 0; k < in.size(); k += kIn[op]) run(op, in.data() + k, out);
  fwrite(out.data(), sizeof(float), out.size(), stdout);
  return 0;
}
