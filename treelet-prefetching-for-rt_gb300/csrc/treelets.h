// Treelet partition of a blob (host, array based) and the staged images
// that the shared-memory traversal copies with cp.async.bulk.
#pragma once
#include <stdint.h>

#include <string>
#include <vector>

namespace rtt {

constexpr uint32_t kNoTreelet = 0xFFFFFFFFu;
constexpr uint32_t kSlotBits = 10;  // image slots of 64 B: images up to 64 KiB
constexpr uint32_t kMaxDense = 1u << (32 - kSlotBits);

struct Partition {
  uint32_t max_bytes = 0;
  std::vector<uint32_t> roots;         // root unit of treelet k, ascending
  std::vector<uint16_t> root_bytes;    // size of the root entry (64 / 128)
  std::vector<uint64_t> member_first;  // k -> first member, size n+1
  std::vector<uint32_t> members;       // member units, formation order, de-duplicated
  std::vector<uint16_t> member_bytes;  // charged size of each member
  std::vector<uint32_t> node_root;     // unit -> treelet root unit (addrToTreeletID)
  // Staged images: treelet k's members' bytes back to back.
  std::vector<uint64_t> image_off;     // k -> byte offset in the image store (64 B aligned), size n+1
  std::vector<uint32_t> node_loc;      // unit -> (dense treelet << kSlotBits) | 64 B slot in its image
  uint64_t image_bytes = 0;
  uint32_t largest_image = 0;
};

// createTreelets (vulkan_ray_tracing.cc:823-1470) + buildNodeToRootMap
// (:475-489) over a blob in one address space.  Returns false with a message
// where the reference would assert (budget too small for a root, bad node).
bool form_treelets(const uint8_t* blob, uint64_t n_bytes, uint32_t max_bytes, Partition& out, std::string* err);

// Fills the image store (size out.image_bytes) from the blob.
void build_images(const uint8_t* blob, const Partition& p, std::vector<uint8_t>& store);

// Routing bits of the treelet-ordered walk, per unit.  traceRayWithTreelets
// pushes a child onto the current-treelet stack when addrToTreeletID(child)
// equals current_treelet_root (vulkan_ray_tracing.cc:1821-1856).  A node
// popped from the current-treelet stack has root(node) == current_treelet_root;
// a node popped from the other stack becomes current_treelet_root itself
// (:1748-1754).  So, for an internal node u and its child slot i:
//   bit i       root(child i) == root(u)   (u came off the current stack)
//   bit 6 + i   root(child i) == u         (u came off the other stack)
// and for an instance leaf bits 12 and 13, the same two tests for its BLAS
// root.  Units are taken modulo 2^29 as the walk's stack entries hold them;
// children outside the blob have no root (kNoTreelet), as in the walk.
constexpr uint32_t kRouteOtherShift = 6;
constexpr uint32_t kRouteInstShift = 12;
constexpr uint32_t kEntryUnitMask = (1u << 29) - 1u;
void route_masks(const uint8_t* blob, uint64_t n_bytes, const Partition& p, std::vector<uint16_t>& out);

// Treelets pinned in shared memory for a whole staged launch (pinned.h).
struct Pinned {
  std::vector<uint8_t> bytes;  // the image, a multiple of 128 bytes; empty when nothing is pinned
  uint32_t root_soff = 0;      // record of the TLAS root node, 0 if it is not pinned
  uint32_t n_treelets = 0;
  uint32_t n_records = 0;
};

// Dense treelet ids by estimated visit frequency: the TLAS treelet first,
// then by the probability that a ray reaching the root box reaches the
// treelet's root, estimated as a product of child / parent box surface-area
// ratios down the tree (an instance's BLAS root inherits the instance leaf's).
void default_pin_order(const uint8_t* blob, uint64_t n_bytes, std::vector<uint32_t>& order, const Partition& p);

// Pins treelets in `order` (dense ids; repeats and ids out of range are
// skipped) while their records fit in `budget` bytes: every member that is
// an internal node, instance leaf or primitive leaf reached in exactly one
// role.  Child pointers of a record name a child's record when the child is
// pinned too.
void build_pinned(const uint8_t* blob, uint64_t n_bytes, const Partition& p, const std::vector<uint16_t>& route,
                  const std::vector<uint32_t>& order, uint32_t budget, Pinned& out);

// remapBVHToTreeletLayout (vulkan_ray_tracing.cc:1473-1509).
bool remap_layout(const Partition& p, uint64_t n_units, uint32_t stride, std::vector<uint64_t>& new_addr,
                  std::string* err);

}  // namespace rtt
