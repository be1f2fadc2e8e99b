// FP32 geometry kernels of the traversal, written for host and device.
//
// Each function keeps the reference's operation order so that, with FMA
// contraction off (nvcc --fmad=false, g++ -ffp-contract=off), results are
// bit-identical to the reference's host code:
//   ray_box_test, calculate_idir, magic_max7/min7, get_t_bound
//       src/cuda-sim/vulkan_ray_tracing.cc:183-257
//   MIN / MAX / MIN_MAX / MAX_MIN ternary macros
//       src/cuda-sim/vulkan_ray_tracing.h:53-56
//   mt_ray_triangle_test, Barycentric  vulkan_ray_tracing.cc:3089-3130
//   make_transformed_ray, get_norm, normalized  vulkan_ray_tracing.cc:148-181
//   float4x4::operator*  vulkan_acceleration_structure_util.h:44-56
//   set_child_bounds     vulkan_acceleration_structure_util.h:499-508
//   dot / cross / + / -  src/gpgpu-sim/vector-math.cc:1-82
#pragma once
#include <stdint.h>
#include "format.h"

#include <cmath>
#include <cstring>

namespace rtm {

struct V3 {
  float x, y, z;
};

RT_HD V3 v3(float a, float b, float c) { return V3{a, b, c}; }
RT_HD V3 sub(V3 a, V3 b) { return v3(a.x - b.x, a.y - b.y, a.z - b.z); }
RT_HD V3 add(V3 a, V3 b) { return v3(a.x + b.x, a.y + b.y, a.z + b.z); }
RT_HD V3 cross(V3 a, V3 b) {
  return v3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
RT_HD float dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }

// Ternary min/max: NaN operands select the second argument, unlike fminf.
RT_HD float tmin2(float a, float b) { return (a < b) ? a : b; }
RT_HD float tmax2(float a, float b) { return (a > b) ? a : b; }
RT_HD float min_max(float a, float b, float c) { return tmax2(tmin2(a, b), c); }
RT_HD float max_min(float a, float b, float c) { return tmin2(tmax2(a, b), c); }

RT_HD float bits_to_float(uint32_t u) {
#if defined(__CUDA_ARCH__)
  return __uint_as_float(u);
#else
  float f;
  std::memcpy(&f, &u, 4);
  return f;
#endif
}

RT_HD float fabs_(float x) {
#if defined(__CUDA_ARCH__)
  return fabsf(x);
#else
  return std::fabs(x);
#endif
}

RT_HD float copysign_(float m, float s) {
#if defined(__CUDA_ARCH__)
  return copysignf(m, s);
#else
  return std::copysign(m, s);
#endif
}

RT_HD float sqrt_(float x) {
#if defined(__CUDA_ARCH__)
  return __fsqrt_rn(x);
#else
  return std::sqrt(x);
#endif
}

// 2^k for k in [-149, 127] built from exponent bits (exact).
RT_HD float exp2_int(int k) {
  if (k >= -126) return bits_to_float((uint32_t)(k + 127) << 23);
  return bits_to_float(1u << (k + 149));
}

// q * 2^k for an 8-bit q and k in [-136, 119]: the product has at most
// 8 significant bits, all above 2^-149, so it is exact and equals ldexpf(q, k).
RT_HD float ldexp_u8(uint32_t q, int k) { return (float)q * exp2_int(k); }

// calculate_idir (vulkan_ray_tracing.cc:220-235): 1 / (|d| > 2^-80 ? d : copysign(2^-80, d)).
RT_HD V3 calculate_idir(V3 d) {
  const float ooeps = exp2_int(-80);
  V3 r;
  r.x = 1.0f / (fabs_(d.x) > ooeps ? d.x : copysign_(ooeps, d.x));
  r.y = 1.0f / (fabs_(d.y) > ooeps ? d.y : copysign_(ooeps, d.y));
  r.z = 1.0f / (fabs_(d.z) > ooeps ? d.z : copysign_(ooeps, d.z));
  return r;
}

// ray_box_test (vulkan_ray_tracing.cc:237-257).
RT_HD bool ray_box_test(V3 lo, V3 hi, V3 idir, V3 o, float tmin, float tmax, float& thit) {
  const float lx = (lo.x - o.x) * idir.x, ly = (lo.y - o.y) * idir.y, lz = (lo.z - o.z) * idir.z;
  const float hx = (hi.x - o.x) * idir.x, hy = (hi.y - o.y) * idir.y, hz = (hi.z - o.z) * idir.z;
  // magic_max7 / magic_min7 (vulkan_ray_tracing.cc:183-197)
  float t1 = min_max(lx, hx, tmin);
  float t2 = min_max(ly, hy, t1);
  const float mn = min_max(lz, hz, t2);
  float u1 = max_min(lx, hx, tmax);
  float u2 = max_min(ly, hy, u1);
  const float mx = max_min(lz, hz, u2);
  thit = mn;
  return mn <= mx;
}

// mt_ray_triangle_test (vulkan_ray_tracing.cc:3089-3111): no epsilon on the
// determinant, inclusive u/v bounds, no t > 0 check.
RT_HD bool ray_triangle_test(V3 p0, V3 p1, V3 p2, V3 o, V3 d, float& thit) {
  const V3 e1 = sub(p1, p0);
  const V3 e2 = sub(p2, p0);
  const V3 pvec = cross(d, e2);
  const float det = dot(e1, pvec);
  const float idet = 1.0f / det;
  const V3 tvec = sub(o, p0);
  const float u = dot(tvec, pvec) * idet;
  if (u < 0.0f || u > 1.0f) return false;
  const V3 qvec = cross(tvec, e1);
  const float v = dot(d, qvec) * idet;
  if (v < 0.0f || (u + v) > 1.0f) return false;
  thit = dot(e2, qvec) * idet;
  return true;
}

// Barycentric (vulkan_ray_tracing.cc:3113-3130); returns {v, w, u}.
RT_HD V3 barycentric(V3 p, V3 a, V3 b, V3 c) {
  const V3 v0 = sub(b, a), v1 = sub(c, a), v2 = sub(p, a);
  const float d00 = dot(v0, v0), d01 = dot(v0, v1), d11 = dot(v1, v1);
  const float d20 = dot(v2, v0), d21 = dot(v2, v1);
  const float denom = d00 * d11 - d01 * d01;
  const float v = (d11 * d20 - d01 * d21) / denom;
  const float w = (d00 * d21 - d01 * d20) / denom;
  const float u = 1.0f - v - w;
  return v3(v, w, u);
}

// A 4x3 instance matrix as the walk uses it: m[j][i], rows j = 0..2 linear,
// row 3 translation, column 3 = (0, 0, 0, 1).
struct Mat43 {
  float m[4][3];
};

// float4x4::operator* (asu.h:44-56): res[i] = sum_j m[j][i] * v[j], j = 0..3,
// accumulated left to right starting from 0.
RT_HD void mat_mul_point(const Mat43& M, V3 p, float w, float out[4]) {
  const float vec[4] = {p.x, p.y, p.z, w};
  for (int i = 0; i < 4; ++i) {
    float r = 0.0f;
    for (int j = 0; j < 4; ++j) {
      const float mji = (i < 3) ? M.m[j][i] : (j == 3 ? 1.0f : 0.0f);
      r += mji * vec[j];
    }
    out[i] = r;
  }
}

struct ObjRay {
  V3 o, d;
  float tmin, tmax;
  float mult;  // worldToObject_tMultiplier
};

// make_transformed_ray (vulkan_ray_tracing.cc:168-181) with get_norm /
// normalized (:148-166).
RT_HD ObjRay make_transformed_ray(const Mat43& w2o, V3 o, V3 d, float tmin, float tmax) {
  float to[4], td[4];
  mat_mul_point(w2o, o, 1.0f, to);
  mat_mul_point(w2o, d, 0.0f, td);
  ObjRay r;
  r.o = v3(to[0] / to[3], to[1] / to[3], to[2] / to[3]);
  const V3 dd = v3(td[0], td[1], td[2]);
  const float norm = sqrt_(dd.x * dd.x + dd.y * dd.y + dd.z * dd.z);
  r.mult = norm;
  // normalized() recomputes the same norm; the value is identical.
  r.d = v3(dd.x / norm, dd.y / norm, dd.z / norm);
  r.tmin = tmin * norm;
  r.tmax = tmax * norm;
  return r;
}

}  // namespace rtm
