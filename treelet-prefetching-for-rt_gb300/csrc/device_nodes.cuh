// Device-side node access: 32-byte vector loads of the 64 / 128-byte nodes
// from global memory (read-only path) or from a staged shared-memory image,
// and the decoders for the fields the walk uses (format.h).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "format.h"
#include "rtmath.h"

namespace rtd {

// Raw node words.  Internal nodes and quad leaves use 16 words (64 B).
struct Node64 {
  uint32_t w[16];
};

__device__ __forceinline__ uint4 ld_global_nc(const uint4* p) { return __ldg(p); }

__device__ __forceinline__ uint4 ld_shared_v4(uint32_t saddr) {
  uint4 v;
  asm volatile("ld.shared.v4.u32 {%0, %1, %2, %3}, [%4];" : "=r"(v.x), "=r"(v.y), "=r"(v.z), "=r"(v.w) : "r"(saddr));
  return v;
}

__device__ __forceinline__ uint32_t ld_shared_u32(uint32_t saddr) {
  uint32_t v;
  asm volatile("ld.shared.u32 %0, [%1];" : "=r"(v) : "r"(saddr));
  return v;
}

// One 32-byte read-only load from global memory (256-bit loads exist on
// sm_100 and later, for the global state space only): a 64-byte node takes
// two load instructions instead of four.  p must be 32-byte aligned; nodes are
// 64-byte aligned in the blob.
__device__ __forceinline__ void ld_global_v8(const uint4* p, uint32_t* w) {
  asm("ld.global.nc.v8.u32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
      : "=r"(w[0]), "=r"(w[1]), "=r"(w[2]), "=r"(w[3]), "=r"(w[4]), "=r"(w[5]), "=r"(w[6]), "=r"(w[7])
      : "l"(p));
}

// Loads 64 bytes: from shared memory when saddr != 0, else from global.
__device__ __forceinline__ void load64(const uint4* g, uint32_t saddr, Node64& n) {
  if (!saddr) {
    ld_global_v8(g, n.w);
    ld_global_v8(g + 2, n.w + 8);
    return;
  }
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    const uint4 v = saddr ? ld_shared_v4(saddr + 16u * q) : ld_global_nc(g + q);
    n.w[4 * q + 0] = v.x;
    n.w[4 * q + 1] = v.y;
    n.w[4 * q + 2] = v.z;
    n.w[4 * q + 3] = v.w;
  }
}

__device__ __forceinline__ uint4 load16(const uint4* g, uint32_t saddr, int q) {
  return saddr ? ld_shared_v4(saddr + 16u * q) : ld_global_nc(g + q);
}

__device__ __forceinline__ uint32_t byte_at(const Node64& n, int b) { return (n.w[b >> 2] >> ((b & 3) * 8)) & 0xffu; }
__device__ __forceinline__ float f32_at(const Node64& n, int b) { return __uint_as_float(n.w[b >> 2]); }

// Result of testing one internal node's children against a ray.
struct ChildHits {
  uint32_t hit_mask;    // bit i: child i hit and not culled
  uint32_t child_unit;  // unit index of child 0's block
  uint64_t info;        // child i's info byte (bits 0-1 size, 2-5 type) at bits 8i..8i+7
  __device__ __forceinline__ uint32_t info_of(int i) const { return (uint32_t)(info >> (8 * i)) & 0x3fu; }
};

// Byte b of the node as an exact float: the byte is placed in the mantissa of
// 2^23 with one byte permute, and 2^23 subtracted (both steps exact).
__device__ __forceinline__ float byte_as_float(const Node64& n, int b) {
  const uint32_t sel = (uint32_t)(b & 3) | 0x7540u;  // bytes: q, 0x00, 0x00, 0x4B
  return __uint_as_float(__byte_perm(n.w[b >> 2], 0x4B000000u, sel)) - 8388608.0f;
}

// The six-way min/max of the slab test.  EXACT uses the reference's ternary
// MIN/MAX macros.  FAST uses fminf/fmaxf, which agree with the ternaries
// except on NaN operands and on the sign of a zero result; with a finite ray
// origin and direction no slab value is NaN, and the sign of thit's zero
// never changes a comparison, so both give the same hit / cull decisions.
template <bool FAST>
__device__ __forceinline__ float mn2(float a, float b) {
  if (FAST) return fminf(a, b);
  return rtm::tmin2(a, b);
}
template <bool FAST>
__device__ __forceinline__ float mx2(float a, float b) {
  if (FAST) return fmaxf(a, b);
  return rtm::tmax2(a, b);
}

// One child's slab test from its six plane distances, reduced as magic_max7 /
// magic_min7 (vulkan_ray_tracing.cc:199-218); a hit at thit >= cull is dropped.
template <bool FAST>
__device__ __forceinline__ bool slab_hit(float lx, float ly, float lz, float hx, float hy, float hz, float tmin,
                                         float tmax, float cull) {
  const float t1 = mx2<FAST>(mn2<FAST>(lx, hx), tmin);
  const float t2 = mx2<FAST>(mn2<FAST>(ly, hy), t1);
  const float tn = mx2<FAST>(mn2<FAST>(lz, hz), t2);
  const float u1 = mn2<FAST>(mx2<FAST>(lx, hx), tmax);
  const float u2 = mn2<FAST>(mx2<FAST>(ly, hy), u1);
  const float tf = mn2<FAST>(mx2<FAST>(lz, hz), u2);
  bool h = tn <= tf;
  if (h && tn >= cull) h = false;
  return h;
}

// Two-wide FP32 arithmetic (add / sub / mul / fma .rn.f32x2, sm_100 and
// later): one instruction computes two lanes, each rounded exactly as the
// scalar instruction rounds it (IEEE round to nearest even, subnormals
// kept), so the results are bit for bit those of two scalar operations.  The
// slab test pairs a child's x and y planes in them.
__device__ __forceinline__ unsigned long long f2_pack(float x, float y) {
  unsigned long long r;
  asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(x), "f"(y));
  return r;
}
__device__ __forceinline__ unsigned long long f2_pack_bits(uint32_t x, uint32_t y) {
  unsigned long long r;
  asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "r"(x), "r"(y));
  return r;
}
__device__ __forceinline__ void f2_unpack(unsigned long long r, float& x, float& y) {
  asm("mov.b64 {%0, %1}, %2;" : "=f"(x), "=f"(y) : "l"(r));
}
__device__ __forceinline__ unsigned long long f2_sub(unsigned long long a, unsigned long long b) {
  unsigned long long r;
  asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
  return r;
}
__device__ __forceinline__ unsigned long long f2_mul(unsigned long long a, unsigned long long b) {
  unsigned long long r;
  asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
  return r;
}
__device__ __forceinline__ unsigned long long f2_fma(unsigned long long a, unsigned long long b,
                                                     unsigned long long c) {
  unsigned long long r;
  asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(r) : "l"(a), "l"(b), "l"(c));
  return r;
}

// Bits of byte b of the node placed in the mantissa of 2^23 (byte_as_float
// before its subtraction of 2^23).
__device__ __forceinline__ uint32_t byte_bits(const Node64& n, int b) {
  return __byte_perm(n.w[b >> 2], 0x4B000000u, (uint32_t)(b & 3) | 0x7540u);
}

// Child bound Origin + ldexpf(q, exp - 8) (asu.h:499-508) as one fused
// multiply-add.  q * 2^(exp-8) is exact for an 8-bit q and exp in [-128, 127]
// (at most 8 significant bits, all at or above 2^-149, below 2^127), so the
// reference's ldexpf is exact and its add is the only rounding; fmaf rounds
// the same exact sum once, giving the same bits (signed zeros included: q = 0
// gives +0 * s + Origin either way).  Saves one FP32 operation per bound, 36
// per internal node.  --fmad=false stops only the compiler's own contraction,
// not this explicit fused operation.
__device__ __forceinline__ float child_bound(const Node64& n, int b, float origin, float scale) {
  return __fmaf_rn(byte_as_float(n, b), scale, origin);
}

// The box tests of an internal node (vulkan_ray_tracing.cc:2518-2553 and the
// bottom-level twin :2714-2741): children with ChildSize > 0 are slab-tested
// with the ray's [tmin, tmax]; a hit at thit >= cull is dropped.  Bounds are
// Origin + ldexpf(q, exp - 8) (asu.h:499-508, child_bound), slab values
// (b - o) * idir (vulkan_ray_tracing.cc:199-218), reduced as magic_max7 /
// magic_min7.
template <bool FAST>
__device__ __forceinline__ ChildHits test_children(const Node64& n, uint32_t node_unit, rtm::V3 o, rtm::V3 idir,
                                                   float tmin, float tmax, float cull) {
  ChildHits r;
  const float ox = f32_at(n, 0), oy = f32_at(n, 4), oz = f32_at(n, 8);
  const int child_off = (int)n.w[3];
  const int ex = (int)(int8_t)byte_at(n, 18), ey = (int)(int8_t)byte_at(n, 19), ez = (int)(int8_t)byte_at(n, 20);
  const float sx = rtm::exp2_int(ex - 8), sy = rtm::exp2_int(ey - 8), sz = rtm::exp2_int(ez - 8);
  r.hit_mask = 0;
  r.info = ((uint64_t)n.w[6] << 16) | (n.w[5] >> 16);  // bytes 22..27
  r.info &= 0x3f3f3f3f3f3full;
  r.child_unit = (uint32_t)((int)node_unit + child_off);
  // x and y in two-wide FP32: the same roundings, fewer instructions
  const unsigned long long s_xy = f2_pack(sx, sy), o_xy = f2_pack(ox, oy);
  const unsigned long long org_xy = f2_pack(o.x, o.y), id_xy = f2_pack(idir.x, idir.y);
  const unsigned long long two23 = f2_pack(8388608.0f, 8388608.0f);
#pragma unroll
  for (int i = 0; i < 6; ++i) {
    const uint32_t info = r.info_of(i);
    if (info & 3u) {
      // q as an exact float (bits - 2^23), Origin + q * 2^(e-8) fused, then (b - o) * idir
      const unsigned long long qlo = f2_sub(f2_pack_bits(byte_bits(n, rtf::IN_LO_X + i), byte_bits(n, rtf::IN_LO_Y + i)), two23);
      const unsigned long long qhi = f2_sub(f2_pack_bits(byte_bits(n, rtf::IN_HI_X + i), byte_bits(n, rtf::IN_HI_Y + i)), two23);
      float lx, ly, hx, hy;
      f2_unpack(f2_mul(f2_sub(f2_fma(qlo, s_xy, o_xy), org_xy), id_xy), lx, ly);
      f2_unpack(f2_mul(f2_sub(f2_fma(qhi, s_xy, o_xy), org_xy), id_xy), hx, hy);
      const float lz = (child_bound(n, rtf::IN_LO_Z + i, oz, sz) - o.z) * idir.z;
      const float hz = (child_bound(n, rtf::IN_HI_Z + i, oz, sz) - o.z) * idir.z;
      if (slab_hit<FAST>(lx, ly, lz, hx, hy, hz, tmin, tmax, cull)) r.hit_mask |= 1u << i;
    }
  }
  return r;
}

// True when the slab test may use the FAST min/max (see mn2).
__device__ __forceinline__ bool finite_ray(rtm::V3 o, rtm::V3 d, float tmin, float tmax) {
  return isfinite(o.x) && isfinite(o.y) && isfinite(o.z) && isfinite(d.x) && isfinite(d.y) && isfinite(d.z) &&
         !isnan(tmin) && !isnan(tmax);
}

// Instance leaf fields used by the walk.
struct Instance {
  rtm::Mat43 w2o;
  uint64_t bvh_address;
  uint32_t instance_id;
};

// The same fields when the leaf's first 64 bytes are already loaded in q:
// two more 16-byte loads (bytes 64..79 and 112..127).
__device__ __forceinline__ void instance_from(const Node64& q, const uint4* g, uint32_t saddr, Instance& in) {
  const uint4 d = load16(g, saddr, 4), e = load16(g, saddr, 7);
#pragma unroll
  for (int k = 0; k < 9; ++k) in.w2o.m[k / 3][k % 3] = __uint_as_float(q.w[4 + k]);
  in.w2o.m[3][0] = __uint_as_float(e.y);
  in.w2o.m[3][1] = __uint_as_float(e.z);
  in.w2o.m[3][2] = __uint_as_float(e.w);
  in.bvh_address = (uint64_t)d.x | ((uint64_t)d.y << 32);
  in.instance_id = d.z;
}

__device__ __forceinline__ void load_instance(const uint4* g, uint32_t saddr, Instance& in) {
  const uint4 a = load16(g, saddr, 1), b = load16(g, saddr, 2), c = load16(g, saddr, 3);
  const uint4 d = load16(g, saddr, 4), e = load16(g, saddr, 7);
  // bytes 16..51: world-to-object rows 0-2
  const uint32_t lin[9] = {a.x, a.y, a.z, a.w, b.x, b.y, b.z, b.w, c.x};
#pragma unroll
  for (int k = 0; k < 9; ++k) in.w2o.m[k / 3][k % 3] = __uint_as_float(lin[k]);
  // bytes 116..127: translation row as the reference's struct-order read takes it
  in.w2o.m[3][0] = __uint_as_float(e.y);
  in.w2o.m[3][1] = __uint_as_float(e.z);
  in.w2o.m[3][2] = __uint_as_float(e.w);
  in.bvh_address = (uint64_t)d.x | ((uint64_t)d.y << 32);
  in.instance_id = d.z;
}

}  // namespace rtd
