// Seeded synthetic scenes, camera rays, host bounce rays and blob handles.
//
// The scenes stand in for the LumiBench scenes the reference is run on
// (README.md:87-114), which are not available: random small triangles in the
// unit cube with a ground plane, a displaced heightfield with instanced
// meshes, and clustered Gaussian blobs.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "builder.h"
#include "capi_internal.h"
#include "format.h"
#include "rtmath.h"

namespace {

// PCG32 (O'Neill 2014), one stream per purpose.
struct Pcg32 {
  uint64_t state = 0, inc = 1;
  Pcg32(uint64_t seed, uint64_t stream) {
    inc = (stream << 1u) | 1u;
    next();
    state += seed;
    next();
  }
  uint32_t next() {
    const uint64_t old = state;
    state = old * 6364136223846793005ULL + inc;
    const uint32_t xs = (uint32_t)(((old >> 18u) ^ old) >> 27u);
    const uint32_t rot = (uint32_t)(old >> 59u);
    return (xs >> rot) | (xs << ((32u - rot) & 31u));
  }
  float uniform() { return (float)(next() >> 8) * (1.0f / 16777216.0f); }
  float range(float a, float b) { return a + (b - a) * uniform(); }
  double normal() {  // Box-Muller
    double u1 = ((double)(next() >> 8) + 0.5) * (1.0 / 16777216.0);
    double u2 = (double)(next() >> 8) * (1.0 / 16777216.0);
    return std::sqrt(-2.0 * std::log(u1)) * std::cos(6.283185307179586 * u2);
  }
};

enum Stream : uint64_t { S_CENTRES = 1, S_EDGES = 2, S_INST = 3, S_BLOB = 4, S_MESH = 100 };

void random_tris(rtb::Mesh& m, uint64_t n, uint64_t seed, uint64_t stream, float lo, float hi, float edge) {
  Pcg32 r(seed, stream);
  m.tris.reserve(m.tris.size() + 9 * n);
  for (uint64_t i = 0; i < n; ++i) {
    float c[3], e1[3], e2[3];
    for (int a = 0; a < 3; ++a) c[a] = r.range(lo, hi);
    for (int a = 0; a < 3; ++a) e1[a] = r.range(-edge, edge);
    for (int a = 0; a < 3; ++a) e2[a] = r.range(-edge, edge);
    for (int a = 0; a < 3; ++a) m.tris.push_back(c[a]);
    for (int a = 0; a < 3; ++a) m.tris.push_back(c[a] + e1[a]);
    for (int a = 0; a < 3; ++a) m.tris.push_back(c[a] + e2[a]);
  }
}

void push_tri(rtb::Mesh& m, const float* a, const float* b, const float* c) {
  for (int k = 0; k < 3; ++k) m.tris.push_back(a[k]);
  for (int k = 0; k < 3; ++k) m.tris.push_back(b[k]);
  for (int k = 0; k < 3; ++k) m.tris.push_back(c[k]);
}

// Hash-based value noise in [0, 1) on an integer lattice.
float lattice(uint64_t seed, int x, int z) {
  uint64_t h = seed ^ (0x9E3779B97F4A7C15ULL * (uint64_t)(uint32_t)x) ^ (0xC2B2AE3D27D4EB4FULL * (uint64_t)(uint32_t)z);
  h ^= h >> 33;
  h *= 0xff51afd7ed558ccdULL;
  h ^= h >> 33;
  h *= 0xc4ceb9fe1a85ec53ULL;
  h ^= h >> 33;
  return (float)(h >> 40) * (1.0f / 16777216.0f);
}

float value_noise(uint64_t seed, float x, float z) {
  const int x0 = (int)std::floor(x), z0 = (int)std::floor(z);
  const float fx = x - (float)x0, fz = z - (float)z0;
  const float sx = fx * fx * (3.0f - 2.0f * fx), sz = fz * fz * (3.0f - 2.0f * fz);
  const float a = lattice(seed, x0, z0), b = lattice(seed, x0 + 1, z0);
  const float c = lattice(seed, x0, z0 + 1), d = lattice(seed, x0 + 1, z0 + 1);
  return (a + (b - a) * sx) + ((c + (d - c) * sx) - (a + (b - a) * sx)) * sz;
}

// fBm with 4 octaves, lacunarity 2, gain 0.5, in [-1, 1) scaled by amplitude.
float fbm(uint64_t seed, float x, float z, float amplitude) {
  float sum = 0.0f, amp = 0.5f, freq = 4.0f, norm = 0.0f;
  for (int o = 0; o < 4; ++o) {
    sum += amp * (2.0f * value_noise(seed + (uint64_t)o * 7919u, x * freq, z * freq) - 1.0f);
    norm += amp;
    amp *= 0.5f;
    freq *= 2.0f;
  }
  return amplitude * sum / norm;
}

constexpr float kTerrainSize = 16.0f;

void identity(rtb::Instance& in) {
  const float id[4][3] = {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}, {0, 0, 0}};
  std::memcpy(in.o2w, id, sizeof(id));
}

// Uniform random rotation (Shoemake), scale and translation as a row-vector
// affine transform.
void random_transform(Pcg32& r, float s_lo, float s_hi, const float t_lo[3], const float t_hi[3], float out[4][3]) {
  const double u1 = r.uniform(), u2 = r.uniform(), u3 = r.uniform();
  const double a = std::sqrt(1 - u1), b = std::sqrt(u1);
  const double qx = a * std::sin(6.283185307179586 * u2), qy = a * std::cos(6.283185307179586 * u2);
  const double qz = b * std::sin(6.283185307179586 * u3), qw = b * std::cos(6.283185307179586 * u3);
  // column-vector rotation R; row-vector form uses R^T
  const double R[3][3] = {{1 - 2 * (qy * qy + qz * qz), 2 * (qx * qy - qz * qw), 2 * (qx * qz + qy * qw)},
                          {2 * (qx * qy + qz * qw), 1 - 2 * (qx * qx + qz * qz), 2 * (qy * qz - qx * qw)},
                          {2 * (qx * qz - qy * qw), 2 * (qy * qz + qx * qw), 1 - 2 * (qx * qx + qy * qy)}};
  const double s = r.range(s_lo, s_hi);
  for (int j = 0; j < 3; ++j)
    for (int k = 0; k < 3; ++k) out[j][k] = (float)(s * R[k][j]);
  for (int k = 0; k < 3; ++k) out[3][k] = r.range(t_lo[k], t_hi[k]);
}

bool finish(std::vector<rtb::Mesh>& meshes, std::vector<rtb::Instance>& inst, rt_blob** out) {
  auto* b = new rt_blob();
  std::string err;
  if (!rtb::build_scene(meshes, inst, b->bytes, nullptr, &err)) {
    delete b;
    rti::set_error("rt_gen_scene: " + err);
    return false;
  }
  *out = b;
  return true;
}

rtm::V3 normalize3(rtm::V3 v) {
  const float n = std::sqrt(v.x * v.x + v.y * v.y + v.z * v.z);
  return rtm::v3(v.x / n, v.y / n, v.z / n);
}

float rd_f32(const uint8_t* p) {
  float f;
  std::memcpy(&f, p, 4);
  return f;
}

}  // namespace

extern "C" {

rt_status rt_gen_scene(uint32_t kind, uint64_t n_tris, uint64_t seed, rt_blob** out) {
  if (!out) return rti::fail(RT_ERR_INVALID, "rt_gen_scene: out is NULL");
  *out = nullptr;
  std::vector<rtb::Mesh> meshes;
  std::vector<rtb::Instance> inst;
  switch (kind) {
    case RT_SCENE_CUBE_PLANE: {
      if (n_tris == 0) n_tris = 16384;
      meshes.resize(1);
      random_tris(meshes[0], n_tris, seed, S_CENTRES, 0.0f, 1.0f, 0.02f);
      const float p0[3] = {-1, 0, -1}, p1[3] = {2, 0, -1}, p2[3] = {2, 0, 2}, p3[3] = {-1, 0, 2};
      push_tri(meshes[0], p0, p1, p2);
      push_tri(meshes[0], p0, p2, p3);
      inst.resize(1);
      identity(inst[0]);
      break;
    }
    case RT_SCENE_CUBE: {
      if (n_tris == 0) n_tris = 16384;
      meshes.resize(1);
      random_tris(meshes[0], n_tris, seed, S_CENTRES, 0.0f, 1.0f, 0.02f);
      inst.resize(1);
      identity(inst[0]);
      break;
    }
    case RT_SCENE_TERRAIN_INSTANCES: {
      if (n_tris == 0) n_tris = 2ull * 1024 * 1024;
      const uint32_t g = std::max<uint32_t>(1, (uint32_t)std::lround(std::sqrt((double)n_tris / 2.0)));
      meshes.resize(65);
      rtb::Mesh& t = meshes[0];
      t.tris.reserve(9ull * 2 * g * g);
      std::vector<float> h((size_t)(g + 1) * (g + 1));
      for (uint32_t z = 0; z <= g; ++z)
        for (uint32_t x = 0; x <= g; ++x)
          h[(size_t)z * (g + 1) + x] = fbm(seed, (float)x / g, (float)z / g, 0.1f) * kTerrainSize;
      for (uint32_t z = 0; z < g; ++z)
        for (uint32_t x = 0; x < g; ++x) {
          const float cs = kTerrainSize / (float)g;
          const float a[3] = {x * cs, h[(size_t)z * (g + 1) + x], z * cs};
          const float b[3] = {(x + 1) * cs, h[(size_t)z * (g + 1) + x + 1], z * cs};
          const float c[3] = {(x + 1) * cs, h[(size_t)(z + 1) * (g + 1) + x + 1], (z + 1) * cs};
          const float d[3] = {x * cs, h[(size_t)(z + 1) * (g + 1) + x], (z + 1) * cs};
          push_tri(t, a, b, c);
          push_tri(t, a, c, d);
        }
      for (uint32_t m = 1; m < 65; ++m) {
        random_tris(meshes[m], 10000, seed, S_MESH + m, -0.5f, 0.5f, 0.02f);
        meshes[m].geometry_index = 0;
      }
      inst.resize(65);
      identity(inst[0]);
      inst[0].mesh = 0;
      inst[0].instance_id = 0;
      Pcg32 r(seed, S_INST);
      const float tlo[3] = {0.0f, 0.0f, 0.0f}, thi[3] = {kTerrainSize, 1.5f, kTerrainSize};
      for (uint32_t i = 1; i < 65; ++i) {
        inst[i].mesh = i;
        inst[i].instance_id = i;
        random_transform(r, 0.5f, 2.0f, tlo, thi, inst[i].o2w);
      }
      break;
    }
    case RT_SCENE_BLOBS: {
      if (n_tris == 0) n_tris = 4ull * 1024 * 1024;
      meshes.resize(1);
      Pcg32 rc(seed, S_CENTRES);
      double centre[16][3];
      for (int b = 0; b < 16; ++b)
        for (int a = 0; a < 3; ++a) centre[b][a] = rc.uniform();
      Pcg32 rb(seed, S_BLOB);
      Pcg32 re(seed, S_EDGES);
      rtb::Mesh& m = meshes[0];
      m.tris.reserve(9 * n_tris);
      for (uint64_t i = 0; i < n_tris; ++i) {
        const int b = (int)(i % 16);
        float c[3];
        for (int a = 0; a < 3; ++a) c[a] = (float)(centre[b][a] + 0.05 * rb.normal());
        float e1[3], e2[3];
        for (int a = 0; a < 3; ++a) e1[a] = re.range(-0.005f, 0.005f);
        for (int a = 0; a < 3; ++a) e2[a] = re.range(-0.005f, 0.005f);
        const float v1[3] = {c[0] + e1[0], c[1] + e1[1], c[2] + e1[2]};
        const float v2[3] = {c[0] + e2[0], c[1] + e2[1], c[2] + e2[2]};
        push_tri(m, c, v1, v2);
      }
      inst.resize(1);
      identity(inst[0]);
      break;
    }
    case RT_SCENE_SHARED_BLAS: {
      if (n_tris == 0) n_tris = 512;
      meshes.resize(1);
      random_tris(meshes[0], n_tris, seed, S_CENTRES, -0.5f, 0.5f, 0.05f);
      inst.resize(4);
      for (uint32_t i = 0; i < 4; ++i) {
        identity(inst[i]);
        inst[i].mesh = 0;
        inst[i].instance_id = 10 + i;
        inst[i].o2w[3][0] = (float)(i % 2) * 1.25f;
        inst[i].o2w[3][1] = (float)(i / 2) * 1.25f;
        inst[i].o2w[3][2] = 0.0f;
      }
      break;
    }
    default:
      return rti::fail(RT_ERR_INVALID, "rt_gen_scene: unknown scene kind " + std::to_string(kind));
  }
  if (!finish(meshes, inst, out)) return RT_ERR_INVALID;
  return RT_OK;
}

rt_status rt_blob_build(const float* tris, const uint32_t* mesh_first, uint32_t n_meshes, const uint32_t* inst_mesh,
                        const float* inst_o2w, const uint32_t* inst_id, uint32_t n_instances, rt_blob** out) {
  if (!out || !tris || !mesh_first || !inst_mesh || !inst_o2w || !inst_id || n_meshes == 0 || n_instances == 0)
    return rti::fail(RT_ERR_INVALID, "rt_blob_build: NULL argument or empty scene");
  *out = nullptr;
  std::vector<rtb::Mesh> meshes(n_meshes);
  for (uint32_t m = 0; m < n_meshes; ++m) {
    if (mesh_first[m + 1] < mesh_first[m]) return rti::fail(RT_ERR_INVALID, "rt_blob_build: mesh_first not ascending");
    meshes[m].tris.assign(tris + 9ull * mesh_first[m], tris + 9ull * mesh_first[m + 1]);
  }
  std::vector<rtb::Instance> inst(n_instances);
  for (uint32_t i = 0; i < n_instances; ++i) {
    inst[i].mesh = inst_mesh[i];
    inst[i].instance_id = inst_id[i];
    for (int j = 0; j < 4; ++j)
      for (int k = 0; k < 3; ++k) inst[i].o2w[j][k] = inst_o2w[12ull * i + 3 * j + k];
  }
  if (!finish(meshes, inst, out)) return RT_ERR_INVALID;
  return RT_OK;
}

rt_status rt_blob_wrap(const void* bytes, uint64_t n_bytes, rt_blob** out) {
  if (!out || (!bytes && n_bytes)) return rti::fail(RT_ERR_INVALID, "rt_blob_wrap: NULL argument");
  auto* b = new rt_blob();
  b->bytes.assign((const uint8_t*)bytes, (const uint8_t*)bytes + n_bytes);
  *out = b;
  return RT_OK;
}

rt_status rt_blob_data(const rt_blob* blob, const uint8_t** bytes, uint64_t* n_bytes) {
  if (!blob || !bytes || !n_bytes) return rti::fail(RT_ERR_INVALID, "rt_blob_data: NULL argument");
  *bytes = blob->bytes.data();
  *n_bytes = blob->bytes.size();
  return RT_OK;
}

void rt_blob_free(rt_blob* blob) { delete blob; }

rt_status rt_scene_default_camera(uint32_t kind, rt_camera* cam) {
  if (!cam) return rti::fail(RT_ERR_INVALID, "rt_scene_default_camera: NULL");
  rt_camera c{};
  c.up[1] = 1.0f;
  c.vfov_deg = 60.0f;
  switch (kind) {
    case RT_SCENE_CUBE_PLANE:
    case RT_SCENE_CUBE:
    case RT_SCENE_BLOBS:
      c.eye[0] = 0.5f, c.eye[1] = 0.5f, c.eye[2] = -1.5f;
      c.target[0] = 0.5f, c.target[1] = 0.5f, c.target[2] = 0.5f;
      break;
    case RT_SCENE_TERRAIN_INSTANCES:
      // 75 degrees below the horizon: the whole 60-degree frustum lands on the terrain
      c.eye[0] = 0.5f * kTerrainSize, c.eye[1] = 0.5625f * kTerrainSize, c.eye[2] = 0.3125f * kTerrainSize;
      c.target[0] = 0.5f * kTerrainSize, c.target[1] = 0.0f, c.target[2] = 0.4632f * kTerrainSize;
      break;
    case RT_SCENE_SHARED_BLAS:
      c.eye[0] = 0.625f, c.eye[1] = 0.625f, c.eye[2] = -3.0f;
      c.target[0] = 0.625f, c.target[1] = 0.625f, c.target[2] = 0.0f;
      break;
    default:
      return rti::fail(RT_ERR_INVALID, "rt_scene_default_camera: unknown kind");
  }
  *cam = c;
  return RT_OK;
}

rt_status rt_gen_camera_rays(const rt_camera* cam, uint32_t width, uint32_t height, uint32_t spp,
                             uint64_t jitter_seed, float tmin, float tmax, rt_ray* out) {
  if (!cam || !out || width == 0 || height == 0 || spp == 0)
    return rti::fail(RT_ERR_INVALID, "rt_gen_camera_rays: bad argument");
  const rtm::V3 eye = rtm::v3(cam->eye[0], cam->eye[1], cam->eye[2]);
  const rtm::V3 fwd = normalize3(rtm::sub(rtm::v3(cam->target[0], cam->target[1], cam->target[2]), eye));
  const rtm::V3 upv = rtm::v3(cam->up[0], cam->up[1], cam->up[2]);
  const rtm::V3 right = normalize3(rtm::cross(fwd, upv));
  const rtm::V3 up = rtm::cross(right, fwd);
  const float th = std::tan(0.5f * cam->vfov_deg * 3.14159265358979f / 180.0f);
  const float aspect = (float)width / (float)height;
  const uint32_t tiles_x = (width + 7) / 8, tiles_y = (height + 3) / 4;
  uint64_t k = 0;
  for (uint32_t s = 0; s < spp; ++s) {
    Pcg32 r(jitter_seed, 1000 + s);
    for (uint32_t ty = 0; ty < tiles_y; ++ty)
      for (uint32_t tx = 0; tx < tiles_x; ++tx)
        for (uint32_t py = 0; py < 4; ++py)
          for (uint32_t px = 0; px < 8; ++px) {
            const uint32_t x = tx * 8 + px, y = ty * 4 + py;
            if (x >= width || y >= height) continue;
            float jx = 0.5f, jy = 0.5f;
            if (jitter_seed) {
              jx = r.uniform();
              jy = r.uniform();
            }
            const float sx = (2.0f * ((float)x + jx) / (float)width - 1.0f) * aspect * th;
            const float sy = (1.0f - 2.0f * ((float)y + jy) / (float)height) * th;
            rtm::V3 d = rtm::add(fwd, rtm::add(rtm::v3(right.x * sx, right.y * sx, right.z * sx),
                                               rtm::v3(up.x * sy, up.y * sy, up.z * sy)));
            d = normalize3(d);
            rt_ray& o = out[k++];
            o.origin[0] = eye.x, o.origin[1] = eye.y, o.origin[2] = eye.z;
            o.dir[0] = d.x, o.dir[1] = d.y, o.dir[2] = d.z;
            o.tmin = tmin;
            o.tmax = tmax;
          }
  }
  return RT_OK;
}

rt_status rt_gen_bounce_rays_host(const rt_blob* blob, const rt_ray* rays, const rt_hit* hits, uint64_t n,
                                  uint64_t seed, float tmin, float tmax, rt_ray* out) {
  if (!blob || !rays || !hits || !out) return rti::fail(RT_ERR_INVALID, "rt_gen_bounce_rays_host: NULL");
  const uint8_t* B = blob->bytes.data();
  const uint64_t nb = blob->bytes.size();
  for (uint64_t i = 0; i < n; ++i) {
    rt_ray& o = out[i];
    const rt_hit& h = hits[i];
    if (!h.hit_geometry || (uint64_t)h.closest_leaf * 64 + 64 > nb || (uint64_t)h.closest_instance * 64 + 128 > nb) {
      o = rays[i];
      o.tmin = 1.0f;
      o.tmax = 0.0f;
      continue;
    }
    rti::BounceInput in;
    std::memcpy(in.leaf, B + (uint64_t)h.closest_leaf * 64, 64);
    std::memcpy(in.inst, B + (uint64_t)h.closest_instance * 64, 128);
    rti::make_bounce(in, rays[i], h, seed, i, tmin, tmax, o);
  }
  return RT_OK;
}

}  // extern "C"
