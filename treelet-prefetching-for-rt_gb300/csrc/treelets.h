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

// remapBVHToTreeletLayout (vulkan_ray_tracing.cc:1473-1509).
bool remap_layout(const Partition& p, uint64_t n_units, uint32_t stride, std::vector<uint64_t>& new_addr,
                  std::string* err);

}  // namespace rtt
