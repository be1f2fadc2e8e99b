// sample_gen: writes the CPU-baseline sample of the terrain workload to files,
// so that the reference's own walk (pin_traversal --time) can be timed in a
// process that loads none of the library's shared objects.
//
//   sample_gen <out dir> <width> <height> <spp> <seed> <sample rays> <threads>
//
// Writes <out dir>/blob (the scene: the 1024 x 1024 fBm heightfield, 2^21
// triangles, with 64 instanced 10K-triangle meshes) and <out dir>/rays: about
// <sample rays> / 2 camera rays spread evenly over the frame (pixel-centre
// jitter seed <seed>, tmin 1e-4, tmax 1e30) followed by their cosine bounce
// rays.  The bounce rays need each primary ray's closest leaf and instance;
// the oracle's restatement of traceRay (pinned to the reference's own walk)
// finds them.  The scene and ray generators are the library's host code,
// compiled in; this program is test infrastructure for the CPU baseline.
#include <cstdio>
#include <cstdlib>
#include <string>
#include <vector>

#include "../include/treelet_rt.h"
#include "oracle_rt.h"

namespace rti {
// the library's error recorder, for the generators compiled in here
void set_error(const std::string& msg) { std::fprintf(stderr, "sample_gen: %s\n", msg.c_str()); }
rt_status fail(rt_status s, const std::string& msg) {
  set_error(msg);
  return s;
}
}  // namespace rti

namespace {

bool write_file(const std::string& path, const void* data, size_t n) {
  FILE* f = std::fopen(path.c_str(), "wb");
  if (!f) return false;
  const bool ok = std::fwrite(data, 1, n, f) == n;
  return std::fclose(f) == 0 && ok;
}

}  // namespace

int main(int argc, char** argv) {
  if (argc != 8) {
    std::fprintf(stderr, "usage: sample_gen <out dir> <width> <height> <spp> <seed> <sample rays> <threads>\n");
    return 2;
  }
  const std::string dir = argv[1];
  const uint32_t w = (uint32_t)std::strtoul(argv[2], nullptr, 10), h = (uint32_t)std::strtoul(argv[3], nullptr, 10);
  const uint32_t spp = (uint32_t)std::strtoul(argv[4], nullptr, 10);
  const uint64_t seed = std::strtoull(argv[5], nullptr, 10);
  const uint64_t want = std::strtoull(argv[6], nullptr, 10);
  const int threads = std::atoi(argv[7]);
  rt_blob* blob = nullptr;
  if (rt_gen_scene(RT_SCENE_TERRAIN_INSTANCES, 2ull * 1024 * 1024, seed, &blob) != RT_OK) return 1;
  const uint8_t* bytes = nullptr;
  uint64_t nb = 0;
  rt_blob_data(blob, &bytes, &nb);
  rt_camera cam;
  rt_scene_default_camera(RT_SCENE_TERRAIN_INSTANCES, &cam);
  const uint64_t n_prim = (uint64_t)w * h * spp;
  std::vector<rt_ray> prim(n_prim);
  if (rt_gen_camera_rays(&cam, w, h, spp, seed, 1e-4f, 1e30f, prim.data()) != RT_OK) return 1;
  // primary rays spread evenly over the frame (the indices numpy's
  // linspace(0, n - 1, k).astype(int64) picks)
  const uint64_t k = want / 2;
  std::vector<rt_ray> rays(2 * k);
  for (uint64_t i = 0; i < k; ++i) {
    const double x = k > 1 ? (double)i * (double)(n_prim - 1) / (double)(k - 1) : 0.0;
    rays[i] = prim[(uint64_t)x];
  }
  std::vector<rt_hit> hits(k);
  if (oracle_trace(bytes, nb, nullptr, rays.data(), nullptr, RT_RAY_FLAG_OPAQUE, k, 0, hits.data(), nullptr, nullptr,
                   0, threads) != 0)
    return 1;
  if (rt_gen_bounce_rays_host(blob, rays.data(), hits.data(), k, seed + 100, 1e-4f, 1e30f, rays.data() + k) != RT_OK)
    return 1;
  if (!write_file(dir + "/blob", bytes, nb) || !write_file(dir + "/rays", rays.data(), sizeof(rt_ray) * rays.size()))
    return 1;
  rt_blob_free(blob);
  std::printf("%llu %llu\n", (unsigned long long)k, (unsigned long long)k);
  return 0;
}
