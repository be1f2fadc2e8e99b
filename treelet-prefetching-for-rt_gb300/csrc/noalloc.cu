// rt_trace_host_noalloc: the host-buffer trace without any device allocation.
//
// rt_trace_host stages the caller's host rays and hit records through a
// device buffer that the library allocates (and grows) with cudaMalloc.  Some
// callers cannot allow that: a simulator that calls the traversal per warp
// from its own cycle loop, where an allocation (an implicit device
// synchronisation) per call is not acceptable; a process whose device memory
// is handed out entirely by its own allocator; code that must not change the
// device's memory map while other work is in flight.  This entry point stages
// through one fixed array in device global memory instead, reserved when the
// library is loaded.
//
// Limits and sharing:
//  * At most RT_NOALLOC_MAX_RAYS (32768) rays per call; larger batches are
//    rejected with RT_ERR_TOO_LARGE.  The array is 3,276,800 bytes and every
//    GPU that loads the library holds it until the process exits.
//  * Every call on a device uses the same array.  Calls whose work overlaps
//    on the GPU (from several host threads, or several scenes on one device)
//    race on it; callers must serialise them.
//  * The call runs on the calling thread's per-thread default stream, while
//    the scene's ray hand-out counter, trace counters and status word are
//    shared with every other trace of that scene (rt_trace, rt_trace_host,
//    rt_trace_batch).  A call that overlaps any other trace of the same scene
//    on the GPU races on those as well: serialise them too.
//  * The caller's current device is restored before the call returns.
//  * The array keeps the last call's contents.  Nothing in it needs to start
//    at zero: each call overwrites the rays and flags it uses and the kernel
//    writes every hit record it returns.
//  * The first call on a device looks the array's device address up
//    (cudaGetSymbolAddress); make that first call before any stream capture.
#include <cuda_runtime.h>

#include <mutex>
#include <string>

#include "capi_internal.h"

namespace {

constexpr uint32_t kMaxRays = RT_NOALLOC_MAX_RAYS;
constexpr size_t kRayBytes = sizeof(rt_ray) * (size_t)kMaxRays;     // 1 MiB
constexpr size_t kFlagBytes = sizeof(uint32_t) * (size_t)kMaxRays;  // 128 KiB
constexpr size_t kHitBytes = sizeof(rt_hit) * (size_t)kMaxRays;     // 2 MiB
constexpr size_t kScratchBytes = kRayBytes + kFlagBytes + kHitBytes;
static_assert(kRayBytes % 256 == 0 && kFlagBytes % 256 == 0, "scratch sections stay 256-byte aligned");

// The staging array.  In host code this name is only a stand-in for the
// symbol: its device address comes from cudaGetSymbolAddress below.
static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex g_setup_mutex;
void* g_scratch_addr[kMaxDevices] = {};

// Device address of the array on `device` (which must be current).
rt_status scratch_address(int device, unsigned char** out) {
  if (device < 0 || device >= kMaxDevices) return rti::fail(RT_ERR_INVALID, "rt_trace_host_noalloc: device ordinal");
  std::lock_guard<std::mutex> lock(g_setup_mutex);
  if (!g_scratch_addr[device]) {
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p)
      return rti::fail(RT_ERR_CUDA, std::string("rt_trace_host_noalloc: cudaGetSymbolAddress: ") + cudaGetErrorString(e));
    g_scratch_addr[device] = p;
  }
  *out = static_cast<unsigned char*>(g_scratch_addr[device]);
  return RT_OK;
}

}  // namespace

namespace {

rt_status trace_noalloc(rt_scene* scene, int device, const rt_ray* rays, const uint32_t* flags,
                        uint32_t default_flags, uint32_t n, uint32_t mode, rt_hit* hits) {
  cudaError_t e = cudaSetDevice(device);
  if (e != cudaSuccess) return rti::fail(RT_ERR_CUDA, std::string("rt_trace_host_noalloc: ") + cudaGetErrorString(e));
  unsigned char* base = nullptr;
  rt_status st = scratch_address(device, &base);
  if (st != RT_OK) return st;
  rt_ray* d_rays = reinterpret_cast<rt_ray*>(base);
  uint32_t* d_flags = flags ? reinterpret_cast<uint32_t*>(base + kRayBytes) : nullptr;
  rt_hit* d_hits = reinterpret_cast<rt_hit*>(base + kRayBytes + kFlagBytes);
  cudaStream_t s = cudaStreamPerThread;
  e = cudaMemcpyAsync(d_rays, rays, sizeof(rt_ray) * (size_t)n, cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess && flags)
    e = cudaMemcpyAsync(d_flags, flags, sizeof(uint32_t) * (size_t)n, cudaMemcpyHostToDevice, s);
  if (e != cudaSuccess) return rti::fail(RT_ERR_CUDA, std::string("rt_trace_host_noalloc: ") + cudaGetErrorString(e));
  st = rt_trace(scene, d_rays, d_flags, default_flags, n, mode, d_hits, nullptr, s);
  if (st != RT_OK) return st;
  e = cudaMemcpyAsync(hits, d_hits, sizeof(rt_hit) * (size_t)n, cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return rti::fail(RT_ERR_CUDA, std::string("rt_trace_host_noalloc: ") + cudaGetErrorString(e));
  // a bounded wait inside the kernel that gave up (results stay valid:
  // staging was switched off for the rest of that launch)
  return rti::check_device_status(scene, "rt_trace_host_noalloc");
}

}  // namespace

extern "C" rt_status rt_trace_host_noalloc(rt_scene* scene, const rt_ray* rays, const uint32_t* flags,
                                           uint32_t default_flags, uint32_t n, uint32_t mode, rt_hit* hits) {
  if (!scene) return rti::fail(RT_ERR_INVALID, "rt_trace_host_noalloc: NULL scene");
  if (n == 0) return RT_OK;
  if (!rays || !hits) return rti::fail(RT_ERR_INVALID, "rt_trace_host_noalloc: NULL rays or hits");
  if (n > kMaxRays)
    return rti::fail(RT_ERR_TOO_LARGE, "rt_trace_host_noalloc: " + std::to_string(n) +
                                           " rays exceed the fixed staging array (at most " +
                                           std::to_string(kMaxRays) + " rays per call)");
  // The scene's device is the device of its blob.
  const void* dblob = nullptr;
  uint64_t nbytes = 0;
  rt_status st = rt_scene_device_blob(scene, &dblob, &nbytes);
  if (st != RT_OK) return st;
  cudaPointerAttributes attr{};
  cudaError_t e = cudaPointerGetAttributes(&attr, dblob);
  if (e != cudaSuccess) return rti::fail(RT_ERR_CUDA, std::string("rt_trace_host_noalloc: ") + cudaGetErrorString(e));
  int caller_device = 0;
  e = cudaGetDevice(&caller_device);
  if (e != cudaSuccess) return rti::fail(RT_ERR_CUDA, std::string("rt_trace_host_noalloc: ") + cudaGetErrorString(e));
  st = trace_noalloc(scene, attr.device, rays, flags, default_flags, n, mode, hits);
  // the caller's current device, as it was on entry
  e = cudaSetDevice(caller_device);
  if (st == RT_OK && e != cudaSuccess)
    return rti::fail(RT_ERR_CUDA, std::string("rt_trace_host_noalloc: ") + cudaGetErrorString(e));
  return st;
}
