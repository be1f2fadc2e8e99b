/* treelet_rt.h - C ABI of the GB300 ray-traversal library.
 *
 * This is the drop-in boundary for the reference simulator's functional
 * ray-traversal path.  In the reference, the PTX `trace_ray` op
 * (src/cuda-sim/instructions.cc:7135-7255) calls, once per ray,
 *
 *   VulkanRayTracing::traceRay(...)               src/cuda-sim/vulkan_ray_tracing.h:329-341
 *   VulkanRayTracing::traceRayWithTreelets(...)   src/cuda-sim/vulkan_ray_tracing.h:343-356
 *
 * which form treelets on the first call (createTreelets,
 * src/cuda-sim/vulkan_ray_tracing.cc:823-1470), walk the BVH, store a
 * Traversal_data record (src/cuda-sim/vulkan_rt_thread_data.h:43-58) and hand
 * an ordered list of node memory transactions to the RT-unit timing model
 * (thread->set_rt_transactions, vulkan_ray_tracing.cc:2252, :3040).  The
 * timing model then looks treelets up through addrToTreeletID /
 * treelet_roots_addr_only (vulkan_ray_tracing.cc:456-489) and makes
 * treelet-prefetch decisions (src/gpgpu-sim/shader.cc:3419-3633).
 *
 * Here the same work is batched: a caller passes device arrays of rays and
 * receives device arrays of hit records and access traces.  All functions
 * return an rt_status; rt_last_error() gives the message of the last failure
 * on the calling thread.  Nothing aborts and no device code traps.
 *
 * Addresses: a node is named by its byte offset in the scene blob divided
 * by 64 (its "unit index"); the blob is one address space (the reference's
 * host-to-device offsets are 0 unless rt_scene_set_device_offset says
 * otherwise).  A treelet is named by its root's unit index,
 * exactly as the reference names a treelet by its root address.
 */
#ifndef TREELET_RT_H
#define TREELET_RT_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum rt_status {
  RT_OK = 0,
  RT_ERR_INVALID = 1,   /* bad argument */
  RT_ERR_CUDA = 2,      /* a CUDA runtime call failed */
  RT_ERR_OOM = 3,       /* allocation failed */
  RT_ERR_BLOB = 4,      /* scene blob failed validation */
  RT_ERR_STATE = 5,     /* call order violated (e.g. trace before treelets) */
  RT_ERR_TOO_LARGE = 6, /* size beyond a documented limit */
  RT_ERR_TIMEOUT = 7,   /* a bounded device wait gave up */
  RT_ERR_NO_DEVICE = 8  /* no CUDA device / kernels not loadable */
} rt_status;

/* Ray flags: SPIR-V RayFlags (SPV_KHR_ray_tracing). */
#define RT_RAY_FLAG_OPAQUE 0x1u
#define RT_RAY_FLAG_NO_OPAQUE 0x2u
#define RT_RAY_FLAG_TERMINATE_ON_FIRST_HIT 0x4u
#define RT_RAY_FLAG_SKIP_CLOSEST_HIT 0x8u

/* Traversal modes. */
#define RT_MODE_PLAIN 0u   /* traceRay order (vulkan_ray_tracing.cc:2309-3076) */
#define RT_MODE_TREELET 1u /* traceRayWithTreelets order (vulkan_ray_tracing.cc:1522-2307) */
#define RT_MODE_STAGED 2u  /* treelet order; treelets staged into shared memory */

/* Transaction types in a visit trace (TransactionType,
 * src/abstract_hardware_model.h:201-211). */
#define RT_TX_STRUCTURE 0u
#define RT_TX_INTERNAL_NODE 1u
#define RT_TX_INSTANCE_LEAF 2u
#define RT_TX_LEAF_DESCRIPTOR 3u
#define RT_TX_QUAD_LEAF 4u
#define RT_TX_QUAD_LEAF_HIT 5u
#define RT_TX_PROCEDURAL_LEAF 6u

/* Per-ray status bits in rt_hit.status. */
#define RT_RAY_TRACE_OVERFLOW 0x1u /* more transactions than trace capacity */
#define RT_RAY_STACK_OVERFLOW 0x2u /* traversal stack full: result invalid */
#define RT_RAY_HIT_PROCEDURAL 0x4u /* a procedural leaf was reached */
#define RT_RAY_BAD_NODE 0x8u       /* a child pointer left the blob: result invalid */

/* A ray: the reference's Ray {origin_tmin, dir_tmax}
 * (src/abstract_hardware_model.h:333-370). 32 bytes. */
typedef struct rt_ray {
  float origin[3];
  float tmin;
  float dir[3];
  float tmax;
} rt_ray;

/* Hit record: the fields of Traversal_data / Hit_data
 * (src/cuda-sim/vulkan_rt_thread_data.h:29-58) that traversal produces,
 * plus trace bookkeeping.  64 bytes. */
typedef struct rt_hit {
  uint32_t hit_geometry;     /* 1 if min_thit < Tmax */
  uint32_t geometry_index;   /* closest leaf's GeometryIndex */
  uint32_t primitive_index;  /* closest leaf's PrimitiveIndex0 */
  uint32_t instance_index;   /* closest instance leaf's InstanceID */
  float world_min_thit;
  float barycentric[3];      /* {v, w, u} as Barycentric() returns */
  float intersection_point[3];
  uint32_t n_visits;         /* transactions of this ray (full count) */
  uint32_t status;           /* RT_RAY_* bits */
  uint32_t closest_leaf;     /* unit index of the closest quad leaf */
  uint32_t closest_instance; /* unit index of its instance leaf */
  uint32_t reserved;
} rt_hit;

/* Caller-owned device buffers for the access traces.  Either pointer may be
 * NULL (that trace is not written).  Row r holds ray r's first `capacity`
 * transactions in order.
 *   visits[r * capacity + j]   = unit_index << 3 | transaction type
 *   treelets[r * capacity + j] = treelet root unit index of that transaction
 *                                (the reference's "RayID,<ids>" line,
 *                                vulkan_ray_tracing.cc:2256-2262) */
typedef struct rt_trace_buf {
  uint32_t* visits;
  uint32_t* treelets;
  uint32_t capacity;
} rt_trace_buf;

typedef struct rt_blob rt_blob;   /* host scene blob */
typedef struct rt_ctx rt_ctx;     /* device context */
typedef struct rt_scene rt_scene; /* device-resident scene */

/* ---------------- errors ---------------- */
const char* rt_last_error(void);
const char* rt_version(void);

/* ---------------- host scene blobs ---------------- */

/* Synthetic scene kinds (seeded).  See rt_gen_scene. */
#define RT_SCENE_CUBE_PLANE 0u        /* n random small triangles in the unit cube + 2-triangle ground plane */
#define RT_SCENE_TERRAIN_INSTANCES 1u /* heightfield (n triangles) + 64 instanced 10K-triangle meshes */
#define RT_SCENE_BLOBS 2u             /* n small triangles in 16 Gaussian blobs (sigma 0.05) */
#define RT_SCENE_CUBE 3u              /* n random small triangles in the unit cube */
#define RT_SCENE_SHARED_BLAS 4u       /* one n-triangle mesh instanced 4 times (shared BLAS) */

rt_status rt_gen_scene(uint32_t kind, uint64_t n_tris, uint64_t seed, rt_blob** out);

/* Builds a blob from caller meshes and instances.  tris holds 9 floats per
 * triangle; mesh m owns triangles [mesh_first[m], mesh_first[m+1]).  Each
 * instance i references mesh inst_mesh[i] with object-to-world transform
 * inst_o2w[12*i .. 12*i+11] (row-vector convention: rows 0-2 linear part,
 * row 3 translation) and InstanceID inst_id[i]. */
rt_status rt_blob_build(const float* tris, const uint32_t* mesh_first, uint32_t n_meshes,
                        const uint32_t* inst_mesh, const float* inst_o2w, const uint32_t* inst_id,
                        uint32_t n_instances, rt_blob** out);

/* Wraps existing bytes (copied) in the reference layout. */
rt_status rt_blob_wrap(const void* bytes, uint64_t n_bytes, rt_blob** out);
rt_status rt_blob_data(const rt_blob* blob, const uint8_t** bytes, uint64_t* n_bytes);
void rt_blob_free(rt_blob* blob);

/* Pinhole camera rays on the host: W x H pixels, spp samples each,
 * pixel-centre samples when jitter_seed == 0, else jittered.  Rays are
 * ordered sample-major, then 8x4 pixel tiles (one warp per tile, the
 * launch tiling of vkCmdTraceRaysKHR, vulkan_ray_tracing.cc:3503-3588). */
typedef struct rt_camera {
  float eye[3];
  float target[3];
  float up[3];
  float vfov_deg;
} rt_camera;
rt_status rt_scene_default_camera(uint32_t kind, rt_camera* cam);
rt_status rt_gen_camera_rays(const rt_camera* cam, uint32_t width, uint32_t height, uint32_t spp,
                             uint64_t jitter_seed, float tmin, float tmax, rt_ray* out);

/* Cosine-weighted bounce rays about the geometric normal at each hit (host).
 * Rays whose hit_geometry is 0 get an empty interval (tmin = 1, tmax = 0). */
rt_status rt_gen_bounce_rays_host(const rt_blob* blob, const rt_ray* rays, const rt_hit* hits, uint64_t n,
                                  uint64_t seed, float tmin, float tmax, rt_ray* out);

/* Validates a blob: header, child pointers in range, child sizes/types legal.
 * Returns RT_ERR_BLOB with a message on the first problem. */
rt_status rt_blob_validate(const rt_blob* blob);

/* ---------------- device context and scenes ---------------- */
rt_status rt_ctx_create(int device, rt_ctx** out);
rt_status rt_ctx_destroy(rt_ctx* ctx);

/* Uploads a blob (validated first). */
rt_status rt_scene_create(rt_ctx* ctx, const rt_blob* blob, rt_scene** out);
rt_status rt_scene_destroy(rt_scene* scene);
/* Device pointer and size of the uploaded blob. */
rt_status rt_scene_device_blob(const rt_scene* scene, const void** dptr, uint64_t* n_bytes);

/* ---------------- treelets ---------------- */

/* Treelet partition of the scene with a byte budget per treelet
 * (createTreelets, vulkan_ray_tracing.cc:823-1470, with the node -> treelet
 * map of buildNodeToRootMap, :475-489).  Must precede RT_MODE_TREELET /
 * RT_MODE_STAGED traces.  Re-forming replaces the previous partition. */
typedef struct rt_treelet_info {
  uint32_t n_treelets;
  uint32_t max_treelet_bytes;
  uint64_t member_entries;  /* sum of member-list lengths after de-dup */
  uint64_t image_bytes;     /* bytes of all staged treelet images */
  uint32_t largest_image;   /* bytes of the largest treelet image */
  uint32_t reserved;
} rt_treelet_info;
rt_status rt_treelets_form(rt_scene* scene, uint32_t max_treelet_bytes, rt_treelet_info* info);

/* Host copies of the partition:
 *   roots[k]        root unit index of treelet k (k ascending root address =
 *                   treelet_addr_to_metadata_idx order, vulkan_ray_tracing.cc:1310-1334)
 *   member_first[k] start of treelet k's members in `members`, k = 0..n (n+1 entries)
 *   members[...]    member unit indices in formation order, de-duplicated
 *   member_bytes[..] size charged for each member (64 / 128)
 *   node_root[u]    treelet root of unit u (addrToTreeletID) or 0xFFFFFFFF
 * Any pointer may be NULL.  Sizes: n_treelets, n_treelets + 1,
 * member_entries, member_entries, blob bytes / 64. */
rt_status rt_treelets_get(const rt_scene* scene, uint32_t* roots, uint64_t* member_first, uint32_t* members,
                          uint16_t* member_bytes, uint32_t* node_root);

/* The same partition on the host only, without a device (for tools and
 * tests): form, read back (same layout as rt_treelets_get), remap, free. */
typedef struct rt_partition rt_partition;
rt_status rt_partition_form(const rt_blob* blob, uint32_t max_treelet_bytes, rt_partition** out,
                            rt_treelet_info* info);
rt_status rt_partition_get(const rt_partition* p, uint32_t* roots, uint64_t* member_first, uint32_t* members,
                           uint16_t* member_bytes, uint32_t* node_root);
rt_status rt_partition_remap(const rt_partition* p, uint32_t stride, uint64_t* new_addr);
void rt_partition_free(rt_partition* p);
/* Routing bits of the treelet-ordered walk per unit (n_units entries; no
 * reference counterpart, they restate the addrToTreeletID comparisons of
 * traceRayWithTreelets, vulkan_ray_tracing.cc:1821-1856, per node): bit i:
 * internal child i shares the node's treelet root; bit 6 + i: child i's
 * treelet root is the node; bits 12 / 13: the same for an instance leaf's
 * BLAS root.  `blob` must be the one the partition was formed on. */
rt_status rt_partition_route(const rt_partition* p, const rt_blob* blob, uint16_t* route);
/* The pinned image for `order` (NULL: default order) and `budget` bytes:
 * out == NULL only reports its size in *n_bytes; else out receives *n_bytes
 * bytes.  *root_soff: record of the TLAS root in 16-byte units, 0 if absent. */
rt_status rt_partition_pinned(const rt_partition* p, const rt_blob* blob, const uint32_t* order, uint32_t n_order,
                              uint32_t budget, void* out, uint64_t* n_bytes, uint32_t* root_soff);

/* Treelet-contiguous relayout (remapBVHToTreeletLayout,
 * vulkan_ray_tracing.cc:1473-1509): new_addr[u] for every unit, or
 * 0xFFFFFFFFFFFFFFFF for units not placed; treelet k starts at
 * k * (max_treelet_bytes + stride).  Returns RT_ERR_STATE where the reference
 * asserts (a treelet root already placed inside an earlier treelet). */
rt_status rt_treelets_remap(const rt_scene* scene, uint32_t stride, uint64_t* new_addr);

/* ---------------- tracing ---------------- */

/* Traces n rays.  All array arguments are device pointers on the scene's
 * device; `flags` may be NULL (every ray uses default_flags).  `trace` may be
 * NULL.  Stream-ordered on `stream` (a cudaStream_t, NULL = default stream). */
rt_status rt_trace(rt_scene* scene, const rt_ray* rays, const uint32_t* flags, uint32_t default_flags, uint32_t n,
                   uint32_t mode, rt_hit* hits, const rt_trace_buf* trace, void* stream);

/* The same with host arrays: copies rays in and hits (and traces, whose
 * pointers are then host pointers) out; synchronous.  When `hits` is
 * page-locked, mapped host memory (cudaHostAlloc, or cudaHostRegister with
 * mapping) and no trace is asked for, the kernel writes the hit records
 * straight into it and there is no copy-out; if `rays` (and `flags`) are
 * page-locked too, the kernel also reads them where they are, and the call is
 * one launch with no copies.  Otherwise a call of 2^19 rays or more runs as up
 * to 4 chunks on the scene's own streams, so that copies of one chunk overlap
 * the trace of another (page-locked host arrays let them overlap fully).
 * Results and the counters of rt_trace_stats_get cover the whole call, as for
 * one rt_trace. */
rt_status rt_trace_host(rt_scene* scene, const rt_ray* rays, const uint32_t* flags, uint32_t default_flags,
                        uint32_t n, uint32_t mode, rt_hit* hits, const rt_trace_buf* trace);

/* rt_trace_host with the access traces packed: ray r's transactions are
 * entries offsets[r] .. offsets[r+1]-1 of `visits` / `treelets` (either may be
 * NULL, not both), its first min(n_visits, row_capacity) transactions in
 * order, as the reference keeps one variable-length access list per ray
 * (the per-thread transaction lists that traceRayWithTreelets fills,
 * vulkan_ray_tracing.cc:2256-2262).  Only the used entries cross PCIe/C2C,
 * not n x row_capacity.  `offsets` holds n + 1 entries; `capacity` is the
 * entries `visits` and `treelets` each hold.  *total receives the entries
 * written; when it exceeds `capacity`, hits, offsets and *total are still
 * filled, the arrays' contents are unspecified and the call returns
 * RT_ERR_TOO_LARGE (call again with arrays of *total entries).  Calls of
 * 2^19 rays or more run as chunks whose packing and copies overlap the next
 * chunk's trace (page-locked arrays let the copies run at full speed).
 * n x row_capacity must stay below 2^32 and n at most 2^24.  Synchronous. */
rt_status rt_trace_host_packed(rt_scene* scene, const rt_ray* rays, const uint32_t* flags, uint32_t default_flags,
                               uint32_t n, uint32_t mode, uint32_t row_capacity, rt_hit* hits, uint64_t* offsets,
                               uint32_t* visits, uint32_t* treelets, uint64_t capacity, uint64_t* total);

/* rt_trace_host for callers that cannot allocate device memory: no
 * counterpart in the reference.  A simulator calling the traversal per warp
 * from its cycle loop, or a process whose device memory belongs to its own
 * allocator, cannot have the library cudaMalloc a staging buffer (an
 * allocation synchronises the device).  This call stages rays, flags and hit
 * records through one fixed device array of 3,276,800 bytes that the library
 * reserves at load time (held on every GPU that loads it until exit), so it
 * takes at most RT_NOALLOC_MAX_RAYS rays per call and returns
 * RT_ERR_TOO_LARGE above that.  All calls on a device share the array:
 * calls that overlap on the GPU race, so serialise them.  The first call on a
 * device looks up the array's address; make it before any stream capture.
 * No visit traces.  Synchronous. */
#define RT_NOALLOC_MAX_RAYS 32768u
rt_status rt_trace_host_noalloc(rt_scene* scene, const rt_ray* rays, const uint32_t* flags, uint32_t default_flags,
                                uint32_t n, uint32_t mode, rt_hit* hits);

/* Predicted next treelets for RT_MODE_STAGED (no reference counterpart):
 * hints[8 * t + octant] is the dense treelet expected after dense treelet t
 * for rays whose direction falls in the octant (bit 0: x > 0, bit 1: y > 0,
 * bit 2: z > 0).  With hints set, a warp stages the treelet its lanes are
 * predicted to reach after their next one instead of the next one itself.
 * NULL clears them.  Host array of 8 x n_treelets entries; staging never
 * changes a result. */
rt_status rt_scene_set_stage_hints(rt_scene* scene, const uint32_t* hints);

/* Traversal tuning; 0 keeps the current value, RT_TUNING_OFF switches a
 * feature off where noted.  None of these changes any result, only speed. */
#define RT_TUNING_OFF 0xFFFFFFFFu
typedef struct rt_tuning {
  uint32_t block_threads;     /* threads per CTA for RT_MODE_PLAIN / RT_MODE_TREELET (32..256) */
  uint32_t staged_threads;    /* threads per CTA for RT_MODE_STAGED (32..256) */
  uint32_t staged_epoch;      /* node visits of a warp between staging votes */
  uint32_t staged_slots;      /* shared-memory treelet slots per warp (1..8; RT_TUNING_OFF: none) */
  uint32_t refill_lanes;      /* idle lanes of a warp that make it fetch new rays (1..32) */
  uint32_t staged_slot_bytes; /* bytes per slot: a treelet's first bytes when smaller than it */
  uint32_t staged_min_votes;  /* lanes of a warp that must want a treelet to stage it (1..32) */
  uint32_t stack_depth;       /* traversal stack entries per ray: 48, 96 or 160 (deeper rays are flagged) */
  uint32_t pinned_bytes;      /* shared memory per CTA for pinned treelets (256..229376; RT_TUNING_OFF: none) */
  uint32_t wait_tries;        /* probes of a CTA's wait for its pinned treelets before it stops staging
                                 (1..2^24; the first probe does not block); the wait for copies still in
                                 flight when a CTA exits always keeps the default limit (2^22) */
  uint32_t queue_rounds;      /* RT_MODE_STAGED: rounds of treelet queues (1..64; RT_TUNING_OFF: none, the
                                 walk with pinned treelets and warp slots).  With queues, rays wait in
                                 per-treelet queues between treelets; each round a warp stages one
                                 treelet into shared memory and runs the stints of the rays queued on
                                 it; after the last round the rays left finish without queues.  The
                                 scene keeps the queues' device memory (about 64 + 8 * stack_depth + 16
                                 bytes per ray) from the first such launch on. */
  uint32_t short_stack;       /* RT_MODE_PLAIN over one scene: 1 keeps the bottom 16 entries of each ray's
                                 stack in shared memory, lane-interleaved per warp (a warp-synchronous
                                 short stack: entry k of the warp's 32 rays in one row of 32 banks),
                                 the deeper ones in local memory; RT_TUNING_OFF (the default): the whole
                                 stack in local memory, about 40% faster on a GB300 */
} rt_tuning;
rt_status rt_scene_set_tuning(rt_scene* scene, const rt_tuning* t);
rt_status rt_scene_get_tuning(const rt_scene* scene, rt_tuning* t);

/* Pinned treelets (RT_MODE_STAGED; no reference counterpart).  Each CTA of a
 * staged launch copies the pinned image into shared memory once, with
 * cp.async.bulk, and serves every read of a pinned node from it for the
 * whole launch.  The image holds the pinned nodes' own bytes with their
 * route bits and the records of their pinned children, so results are
 * unchanged.  Treelets are pinned in `order`
 * (dense ids, most wanted first) while they fit in tuning.pinned_bytes;
 * order == NULL restores the default order: the TLAS treelet, then treelets
 * by the surface-area probability of their root. */
rt_status rt_scene_set_pin_order(rt_scene* scene, const uint32_t* order, uint32_t n);
typedef struct rt_pinned_info {
  uint32_t bytes;       /* image size (0: nothing pinned) */
  uint32_t n_treelets;  /* treelets pinned */
  uint32_t n_records;   /* nodes pinned */
  uint32_t root_pinned; /* 1 if the TLAS root node is pinned */
} rt_pinned_info;
/* The image the next staged launch uses, built now if needed. */
rt_status rt_scene_pinned_info(rt_scene* scene, rt_pinned_info* info);

/* The reference's device_offset: the shift from the host copy of the
 * acceleration structure to the simulated device address that traceRay
 * receives (vulkan_ray_tracing.cc:1549-1572).  Only zero versus nonzero
 * changes a result.  0 (the default) gives the treelet order as intended.
 * With a nonzero offset the reference stores a host address in
 * current_treelet_root at the first pop from the other-treelet stack
 * (:1752) but compares it with device treelet roots (:1821-1856,
 * :1925-1936, :2015-2046), so from then on every child goes to the
 * other-treelet stack; RT_MODE_TREELET and RT_MODE_STAGED then reproduce
 * that order.  RT_MODE_PLAIN is unaffected.  Visit traces name blob units
 * either way (the reference's transaction address is unit * 64 plus the
 * offset). */
rt_status rt_scene_set_device_offset(rt_scene* scene, uint64_t device_offset);

/* Counters of the last rt_trace on this scene (read after the stream is
 * synchronised): node bytes read by the walk, bytes copied into shared memory
 * by treelet staging, node reads served from shared memory / global memory. */
typedef struct rt_trace_stats {
  uint64_t node_bytes;
  uint64_t staged_bytes;
  uint64_t smem_reads;
  uint64_t gmem_reads;
  uint64_t stagings;
  uint64_t device_status; /* nonzero: a bounded wait gave up (staging was switched off) */
} rt_trace_stats;
rt_status rt_trace_stats_get(rt_scene* scene, rt_trace_stats* out);

/* Device version of rt_gen_bounce_rays_host (stream-ordered). */
rt_status rt_gen_bounce_rays(rt_scene* scene, const rt_ray* rays, const rt_hit* hits, uint32_t n, uint64_t seed,
                             float tmin, float tmax, rt_ray* out, void* stream);

/* ---------------- many scenes, one launch ---------------- */

/* A batch traces rays of many scenes in ONE persistent work-queue launch
 * (no reference counterpart: the reference traces one ray per call).  Item k
 * covers rays [ray_begin[k], ray_begin[k+1]) of the concatenated ray and hit
 * arrays and uses scenes[item_scene[k]].  Modes PLAIN and TREELET run as one
 * launch over every item with the batch's tuning; RT_MODE_STAGED runs each
 * item as its scene's own staged launch (its pinned treelets and tuning,
 * without treelet queues), in item order on the stream, because a CTA's
 * shared memory holds one scene's treelets.  TREELET and STAGED need
 * rt_treelets_form on every scene.  The batch owns its queue and counter
 * memory; the scenes must outlive it. */
typedef struct rt_batch rt_batch;
rt_status rt_batch_create(rt_ctx* ctx, rt_scene* const* scenes, uint32_t n_scenes, rt_batch** out);
rt_status rt_batch_destroy(rt_batch* b);
rt_status rt_batch_set_items(rt_batch* b, const uint32_t* ray_begin, const uint32_t* item_scene, uint32_t n_items);
rt_status rt_batch_set_tuning(rt_batch* b, const rt_tuning* t);
rt_status rt_trace_batch(rt_batch* b, const rt_ray* rays, const uint32_t* flags, uint32_t default_flags,
                         uint32_t mode, rt_hit* hits, void* stream);
/* Records rt_trace_batch with these buffers into a CUDA graph owned by the
 * batch (replacing any previous one); rt_batch_graph_launch replays it.  For
 * RT_MODE_STAGED the call first runs the batch once, uncaptured, so that every
 * staged kernel's launch shape is set before recording. */
rt_status rt_batch_graph_capture(rt_batch* b, const rt_ray* rays, const uint32_t* flags, uint32_t default_flags,
                                 uint32_t mode, rt_hit* hits, void* stream);
rt_status rt_batch_graph_launch(rt_batch* b, void* stream);

/* ---------------- learned treelet predictor ---------------- */

/* No reference counterpart: a small MLP that predicts the treelet a ray
 * enters after its current one, trained on the traversal's own treelet
 * traces, used to pick treelets to stage before the rays reach them.
 *   input  : ray origin (3), direction (3), a 16-dim embedding of the current treelet
 *   hidden : 64 -> GELU -> 64 -> GELU (BF16 weights, FP32 accumulate)
 *   output : one logit per treelet of the scene
 * Training runs on the GPU (forward, softmax cross-entropy, backward, Adam). */
typedef struct rt_mlp_sample {
  float origin[3];
  float dir[3];
  uint32_t current; /* dense treelet index (rank of its root in rt_treelets_get's roots) */
  uint32_t target;  /* dense index of the next treelet (ignored by rt_mlp_topk) */
} rt_mlp_sample;    /* 32 bytes */

#define RT_MLP_HIDDEN 64u
#define RT_MLP_EMBED 16u
#define RT_MLP_MAX_BATCH 4096u

typedef struct rt_mlp rt_mlp;
rt_status rt_mlp_create(rt_ctx* ctx, uint32_t n_treelets, uint64_t seed, rt_mlp** out);
rt_status rt_mlp_destroy(rt_mlp* m);
/* Parameter count and host copies (FP32 master values), in the order
 * E[n_treelets][16], W1[22][64], b1[64], W2[64][64], b2[64], W3[64][n], b3[n]. */
rt_status rt_mlp_num_params(const rt_mlp* m, uint64_t* n);
rt_status rt_mlp_get_params(const rt_mlp* m, float* host);
rt_status rt_mlp_set_params(rt_mlp* m, const float* host);
/* Mean cross-entropy and its gradient (same order as the parameters) on a
 * device batch of n <= RT_MLP_MAX_BATCH samples, without updating; grads may be NULL. */
rt_status rt_mlp_loss_grad(rt_mlp* m, const rt_mlp_sample* samples, uint32_t n, float* loss, float* grads_host);
/* One Adam step (lr, beta1 0.9, beta2 0.999) on a device batch; *loss receives the batch loss. */
rt_status rt_mlp_train_step(rt_mlp* m, const rt_mlp_sample* samples, uint32_t n, float lr, float* loss);
/* Top-4 treelets per sample, highest logit first (device output, n x 4). */
rt_status rt_mlp_topk(rt_mlp* m, const rt_mlp_sample* samples, uint32_t n, uint32_t* top4);

/* ---------------- treelet-prefetch decision ---------------- */

/* Heuristics of -treelet_prefetch_heuristic (src/gpgpu-sim/gpu-sim.cc:389-466). */
#define RT_PREFETCH_ALWAYS 0u      /* most popular treelet, always */
#define RT_PREFETCH_POPULARITY 1u  /* only if its share >= threshold */
#define RT_PREFETCH_PARTIAL 2u     /* round(share * nodes) nodes from the start */
#define RT_PREFETCH_LATTER 3u      /* the same count from the end */
#define RT_NO_TREELET 0xFFFFFFFFu

/* Which copy of the decision runs (rt_prefetch_params.variant).  The RT unit
 * has three: the decision block of rt_unit::cycle (shader.cc:3419-3683), the
 * copy the pipelined treelet queue runs (-pipelined_treelet_queue,
 * shader.cc:3780-3932: no second-prefetch rule, only the last prefetched
 * treelet suppressed, heuristic LATTER sized at half the treelet), and the
 * copy the treelet queue runs (-treelet_queue, shader.cc:4020-4060: the whole
 * most popular treelet for every heuristic unless it was the last one
 * prefetched; with no pending access it queues nothing and records "no
 * treelet" as the last one).  RT_PREFETCH_FLUSH_ON_NEW_TREELET may be or-ed in:
 * -flush_prefetch_queue_on_new_treelet clears the queue before a new
 * treelet's requests (shader.cc:3579-3583, :3894-3898; the treelet queue's
 * copy has no such step, so there it changes nothing). */
#define RT_PREFETCH_MAIN_BLOCK 0u
#define RT_PREFETCH_PIPELINED_QUEUE 1u
#define RT_PREFETCH_TREELET_QUEUE 2u
#define RT_PREFETCH_FLUSH_ON_NEW_TREELET 4u

typedef struct rt_prefetch_params {
  uint32_t heuristic;       /* RT_PREFETCH_* */
  uint32_t max_queue;       /* -max_prefetch_queue_size */
  double threshold;         /* -treelet_prefetch_threshold */
  uint32_t second_prefetch; /* -prefetch_next_treelet_when_queue_empty */
  uint32_t variant;         /* RT_PREFETCH_MAIN_BLOCK / _PIPELINED_QUEUE / _TREELET_QUEUE, | _FLUSH_ON_NEW_TREELET */
} rt_prefetch_params;

/* Per-RT-unit state carried from one decision to the next. */
typedef struct rt_prefetch_state {
  uint32_t last_prefetched;        /* root unit or RT_NO_TREELET */
  uint32_t last_prefetched_second; /* root unit or RT_NO_TREELET */
  uint32_t last_rejected;          /* root unit or RT_NO_TREELET */
  uint32_t queue_len;              /* 32 B requests waiting in the unit's prefetch queue */
} rt_prefetch_state;

typedef struct rt_prefetch_decision {
  uint32_t treelet;        /* most popular treelet root, or RT_NO_TREELET */
  uint32_t count;          /* lanes whose next access is in it */
  uint32_t total;          /* lanes with a next access */
  uint32_t submitted;      /* 1 if its nodes were queued */
  uint32_t first_member;   /* queued members: [first_member, first_member + n_members) */
  uint32_t n_members;      /*   of the treelet's member list (rt_treelets_get order) */
  uint32_t chunks;         /* 32 B requests queued */
  uint32_t second_treelet; /* treelet queued by the second-prefetch rule, or RT_NO_TREELET */
} rt_prefetch_decision;

/* One decision per RT unit (shader.cc:3419-3683, or the copy params->variant
 * names): n_units groups of `lanes` next-access unit indices (RT_NO_TREELET =
 * lane idle).  Device arrays; state is read and updated in place.  Needs
 * rt_treelets_form. */
rt_status rt_prefetch_decide(rt_scene* scene, const uint32_t* next_unit, uint32_t n_units, uint32_t lanes,
                             const rt_prefetch_params* params, rt_prefetch_state* state, rt_prefetch_decision* out,
                             void* stream);

/* ---------------- RT-unit trace replay ---------------- */

/* Replays the visit traces of a traced batch through a model of the
 * reference's RT units and their treelet prefetching, with no reference
 * counterpart as one call: it restates the RT unit's request loop
 * (shader.cc:4394-4450, one 32-byte request per cycle, prefetches only on
 * cycles without a demand request, shader.cc:4118-4130, :4453-4501), warp
 * selection (treelet_scheduler 0/1/2, shader.cc:4307-4392), the
 * treelet-prefetch decision every prefetch_delay cycles (shader.cc:3419-3683,
 * with the metadata loads of load_treelet_metadata and the strict wait of
 * wait_for_metadata_load), the Lee MICRO'10 stride prefetcher
 * (shader.cc:4792-4826), the removal of queued prefetches a demand request
 * covers (shader.cc:4657-4681, :4765-4790), and the prefetch classification
 * of gpu-cache.cc:1953-2116 with the final tally of gpu-sim.cc:1749-1790.
 * The memory behind it is this library's own simple model: one sectored L1
 * per RT unit (128 B lines, 32 B sectors, LRU), a fixed hit latency and a
 * fixed miss latency, merging of requests to a sector in flight.
 *
 * Warp w (rays 32w .. 32w + 31 of the batch) runs on RT unit w % n_rt_units,
 * units take their warps in order, at most max_warps at a time.  A warp
 * issues, per round, the next transaction of each lane that has one
 * (identical (address, size) pairs once), split into 32 B requests; the
 * round completes when its last request's data is back, plus the longest
 * intersection latency of its transaction types (2,4,4,2,4,4,4 cycles by
 * transaction type, -gpgpu_rt_intersection_latency).  Transaction addresses
 * are unit * 64 with the sizes of rt_trace's visit entries.  Treelet k's
 * metadata (max_treelet_bytes / 16 bytes, vulkan_ray_tracing.cc:1601-1602)
 * sits at (blob bytes rounded up to 4 KiB) + k * that size; a member that is
 * not a treelet root loads treelet 0's, as the reference's map lookup does. */
#define RT_UNIT_PF_NONE 0u
#define RT_UNIT_PF_TREELET 1u
#define RT_UNIT_PF_STRIDE 2u   /* Lee MICRO'10 */
#define RT_UNIT_SCHED_FIRST 0u /* first ready warp (treelet_scheduler 0) */
#define RT_UNIT_SCHED_OMR 1u   /* first ready warp with a lane headed into the last prefetched treelet */
#define RT_UNIT_SCHED_PMR 2u   /* ready warp with the most such lanes */
typedef struct rt_unit_config {
  uint32_t n_rt_units;       /* RT units */
  uint32_t max_warps;        /* resident warps per unit (-gpgpu_rt_max_warps, 1..16) */
  uint32_t l1_sets;          /* L1 sets (power of two) */
  uint32_t l1_ways;          /* L1 ways (1..32) */
  uint32_t hit_latency;      /* cycles from request to data on a hit (>= 1) */
  uint32_t miss_latency;     /* cycles from request to data on a miss (>= 1, <= 4096) */
  uint32_t prefetcher;       /* RT_UNIT_PF_* */
  uint32_t scheduler;        /* RT_UNIT_SCHED_* (OMR / PMR need the treelet prefetcher) */
  rt_prefetch_params decision; /* treelet prefetcher: heuristic, max queue, threshold, second prefetch
                                  (the main decision block: variant must be 0) */
  uint32_t prefetch_delay;   /* cycles between decisions (>= 1) */
  uint32_t load_metadata;    /* queue each member's treelet metadata before it (-load_treelet_metadata) */
  uint32_t wait_metadata;    /* strict wait for the metadata (-wait_for_metadata_load) */
  uint32_t max_cycles;       /* per unit, 0 = no limit */
} rt_unit_config;

/* Effectiveness classes, numbered as prefetch_request_effectiveness
 * (abstract_hardware_model.h:247-254). */
#define RT_PF_TOO_LATE 0u
#define RT_PF_LATE 1u
#define RT_PF_TIMELY 2u
#define RT_PF_TOO_EARLY 3u
#define RT_PF_NEVER_USED 4u

typedef struct rt_unit_stats {
  uint64_t cycles;              /* cycle after the unit's last warp left */
  uint64_t warps, transactions; /* warps run, lane transactions consumed */
  uint64_t demand_requests;     /* 32 B demand requests */
  uint64_t demand_hits, demand_hit_reserved, demand_misses;
  uint64_t prefetch_queued, prefetch_issued, prefetch_removed; /* 32 B prefetch requests */
  uint64_t prefetch_present, prefetch_merged, prefetch_filled; /* what an issued prefetch found */
  uint64_t decisions, treelets_prefetched, metadata_queued;
  uint64_t effectiveness[5];         /* RT_PF_* tally at the end */
  uint64_t unclassified_but_accessed;
  uint64_t status;              /* bit 0: a model table filled up; bit 1: max_cycles reached */
} rt_unit_stats;

/* hits / visits are the device outputs of rt_trace on `n` rays (visits with
 * `capacity` entries per ray; a ray replays min(n_visits, capacity) of them).
 * stats: device array of n_rt_units records.  Needs rt_treelets_form.  One
 * CUDA thread models one RT unit; the call allocates the units' tables,
 * synchronises `stream` and frees them before it returns. */
rt_status rt_unit_replay(rt_scene* scene, const rt_hit* hits, const uint32_t* visits, uint32_t n, uint32_t capacity,
                         const rt_unit_config* config, rt_unit_stats* stats, void* stream);

#ifdef __cplusplus
}
#endif
#endif /* TREELET_RT_H */
