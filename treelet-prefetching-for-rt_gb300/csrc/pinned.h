// Shared-memory records of pinned treelets.
//
// The staged traversal keeps the most-visited treelets resident in shared
// memory for the whole launch.  A record holds a node's own 64 bytes (so the
// walk reads and tests it exactly as it would from the blob) plus what the
// walk would otherwise fetch from other tables: the node's unit, its route
// bits and the records of its pinned children.  Records are 16-byte aligned
// and named by their offset in 16-byte units ("soff"); soff 0 is never a
// record.
#pragma once
#include <stdint.h>

namespace rtp {

// internal node, 80 B: the blob's 64 bytes with bytes 16..17 (NodeType and
// the pad byte, which the walk does not read) replaced by the node's route
// bits, then a 16-byte tail
constexpr uint32_t IN_ROUTE = 16;        // u16 route bits of the node
constexpr uint32_t IN_UNIT = 64;         // u32 unit of the node
constexpr uint32_t IN_CHILD_SOFF = 68;   // u16 x6: record of child i, 0 if the child is not pinned
constexpr uint32_t kInternalBytes = 80;

// instance leaf, 64 B (decoded: the walk's effective world-to-object rows)
constexpr uint32_t IL_UNIT = 0;        // u32 unit of the leaf
constexpr uint32_t IL_HDR_UNIT = 4;    // u32 unit of its BLAS header
constexpr uint32_t IL_BROOT_UNIT = 8;  // u32 unit of the BLAS root node (as the walk forms it)
constexpr uint32_t IL_ROUTE = 12;      // u16 route bits of the leaf, u16 record of the BLAS root
constexpr uint32_t IL_W2O = 16;        // f32 x12: effective world-to-object rows 0..3
constexpr uint32_t kInstanceBytes = 64;

// primitive (quad / procedural) leaf, 64 B: the blob's bytes with word 0
// (shader index and mask, not read by the walk) replaced by the unit
constexpr uint32_t kPrimBytes = 64;

// largest image: soff is 16 bits
constexpr uint32_t kMaxBytes = 65536u * 16u;

}  // namespace rtp
