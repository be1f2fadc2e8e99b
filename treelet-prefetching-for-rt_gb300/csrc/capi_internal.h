// Internal declarations shared by the library's translation units.
#pragma once
#include <stdint.h>

#include <string>
#include <vector>

#include "../../include/treelet_rt.h"
#include "format.h"
#include "rtmath.h"

struct rt_blob {
  std::vector<uint8_t> bytes;
};

struct rt_ctx {
  int device = 0;
};

namespace rti {

void set_error(const std::string& msg);
rt_status fail(rt_status s, const std::string& msg);

// Host-side structural check of a blob; returns false with a message.
bool validate_blob(const uint8_t* b, uint64_t n, std::string* err);

// After the scene's traces have finished: RT_ERR_TIMEOUT if a bounded device
// wait of the last launch gave up, else RT_OK.
rt_status check_device_status(rt_scene* s, const char* who);

// rt_trace_host runs a call of 2^20 rays or more as 4 chunks of 1/8, 3/8,
// 3/8 and 1/8 of the rays (small first and last chunks shorten the copy-in
// before the first trace and the copy-out after the last), one of 2^19 or
// more as 2 halves, and smaller calls whole.  Each chunk costs about one
// launch's tail (tens of microseconds on a full GPU), so more chunks lose.
constexpr uint32_t kHostChunks = 4;
// Rounds of treelet queues a staged launch may run (rt_tuning.queue_rounds).
constexpr uint32_t kMaxQueueRounds = 64;
inline uint32_t host_chunk_bounds(uint32_t n, uint64_t* lo) {
  const uint32_t chunks = n >= (1u << 20) ? 4u : n >= (1u << 19) ? 2u : 1u;
  static const uint32_t kEighths[3][5] = {{0, 8}, {0, 4, 8}, {0, 1, 4, 7, 8}};
  const uint32_t* e = kEighths[chunks == 4 ? 2 : chunks - 1];
  for (uint32_t c = 0; c <= chunks; ++c) lo[c] = (uint64_t)n * e[c] / 8;
  return chunks;
}

// ---- bounce-ray construction (host and device) ----
struct BounceInput {
  uint8_t leaf[64];
  uint8_t inst[128];
};

RT_HD uint32_t pcg_hash(uint32_t v) {
  // PCG-RXS-M-XS hash (Jarzynski & Olano, JCGT 2020).
  uint32_t state = v * 747796405u + 2891336453u;
  uint32_t word = ((state >> ((state >> 28u) + 4u)) ^ state) * 277803737u;
  return (word >> 22u) ^ word;
}

RT_HD float rd32f(const uint8_t* p) {
  uint32_t u = (uint32_t)p[0] | ((uint32_t)p[1] << 8) | ((uint32_t)p[2] << 16) | ((uint32_t)p[3] << 24);
  return rtm::bits_to_float(u);
}

RT_HD rtm::V3 norm3(rtm::V3 v) {
  const float n = rtm::sqrt_(v.x * v.x + v.y * v.y + v.z * v.z);
  return rtm::v3(v.x / n, v.y / n, v.z / n);
}

// Cosine-weighted direction about the geometric normal of the hit triangle
// (flipped to face the incoming ray), origin at the world hit point.
RT_HD void make_bounce(const BounceInput& in, const rt_ray& ray, const rt_hit& h, uint64_t seed, uint64_t index,
                       float tmin, float tmax, rt_ray& out) {
  float M[4][3];
  for (int j = 0; j < 3; ++j)
    for (int k = 0; k < 3; ++k) M[j][k] = rd32f(in.inst + rtf::IL_O2W_LINEAR + 4 * (3 * j + k));
  for (int k = 0; k < 3; ++k) M[3][k] = rd32f(in.inst + rtf::IL_O2W_TRANSLATION + 4 * k);
  rtm::V3 w[3];
  for (int v = 0; v < 3; ++v) {
    const float p[3] = {rd32f(in.leaf + rtf::QL_V0 + 12 * v), rd32f(in.leaf + rtf::QL_V0 + 12 * v + 4),
                        rd32f(in.leaf + rtf::QL_V0 + 12 * v + 8)};
    float q[3];
    for (int k = 0; k < 3; ++k) q[k] = p[0] * M[0][k] + p[1] * M[1][k] + p[2] * M[2][k] + M[3][k];
    w[v] = rtm::v3(q[0], q[1], q[2]);
  }
  rtm::V3 n = rtm::cross(rtm::sub(w[1], w[0]), rtm::sub(w[2], w[0]));
  const float nl = rtm::sqrt_(n.x * n.x + n.y * n.y + n.z * n.z);
  if (!(nl > 0.0f)) {
    out = ray;
    out.tmin = 1.0f;
    out.tmax = 0.0f;
    return;
  }
  n = rtm::v3(n.x / nl, n.y / nl, n.z / nl);
  if (rtm::dot(n, rtm::v3(ray.dir[0], ray.dir[1], ray.dir[2])) > 0.0f) n = rtm::v3(-n.x, -n.y, -n.z);
  // Orthonormal basis (Duff et al., JCGT 2017).
  const float sign = n.z >= 0.0f ? 1.0f : -1.0f;
  const float a = -1.0f / (sign + n.z);
  const float b = n.x * n.y * a;
  const rtm::V3 t = rtm::v3(1.0f + sign * n.x * n.x * a, sign * b, -sign * n.x);
  const rtm::V3 bt = rtm::v3(b, sign + n.y * n.y * a, -n.y);
  const uint32_t h1 = pcg_hash((uint32_t)index ^ pcg_hash((uint32_t)seed ^ (uint32_t)(seed >> 32)));
  const uint32_t h2 = pcg_hash(h1 ^ 0x68bc21ebu);
  const float u1 = (float)(h1 >> 8) * (1.0f / 16777216.0f);
  const float u2 = (float)(h2 >> 8) * (1.0f / 16777216.0f);
  const float r = rtm::sqrt_(u1);
  const float phi = 6.28318530718f * u2;
#if defined(__CUDA_ARCH__)
  float sp, cp;
  sincosf(phi, &sp, &cp);
#else
  const float sp = std::sin(phi), cp = std::cos(phi);
#endif
  const float lx = r * cp, ly = r * sp, lz = rtm::sqrt_(rtm::tmax2(0.0f, 1.0f - u1));
  rtm::V3 d = rtm::v3(t.x * lx + bt.x * ly + n.x * lz, t.y * lx + bt.y * ly + n.y * lz, t.z * lx + bt.z * ly + n.z * lz);
  d = norm3(d);
  out.origin[0] = h.intersection_point[0];
  out.origin[1] = h.intersection_point[1];
  out.origin[2] = h.intersection_point[2];
  out.dir[0] = d.x;
  out.dir[1] = d.y;
  out.dir[2] = d.z;
  out.tmin = tmin;
  out.tmax = tmax;
}

}  // namespace rti
