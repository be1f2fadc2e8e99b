// Byte layout of the 6-wide quantized-box BVH blob that the traversal reads.
//
// The layout is the one decoded by the reference's
// src/cuda-sim/vulkan_acceleration_structure_util.h (GEN_RT_BVH :89-107,
// GEN_RT_BVH_INTERNAL_NODE :109-207, GEN_RT_BVH_INSTANCE_LEAF :226-387,
// PRIMITIVE_LEAF_DESCRIPTOR :389-424, QUAD_LEAF :426-466,
// PROCEDURAL_LEAF :468-497).  It has to match byte for byte so that a blob
// built for the reference walks identically here; the offsets below are
// written out from those decoders.
//
// A node "address" in this library is its byte offset inside one contiguous
// blob (a single address space: the reference's host->device offsets are 0).
// Every node starts on a 64-byte boundary, so a node is also named by its
// "unit index" = byte offset / 64.  Instance leaves span two units.
#pragma once
#include <stdint.h>

#if defined(__CUDACC__)
#define RT_HD __host__ __device__ __forceinline__
#else
#define RT_HD inline
#endif

namespace rtf {

// Sizes charged per transaction (TransactionType, src/abstract_hardware_model.h:201-211,
// sizes from the *_length * 4 expressions in src/cuda-sim/vulkan_ray_tracing.cc).
constexpr uint32_t kUnit = 64;
constexpr uint32_t kHeaderBytes = 64;          // GEN_RT_BVH_length * 4
constexpr uint32_t kInternalBytes = 64;        // GEN_RT_BVH_INTERNAL_NODE_length * 4
constexpr uint32_t kInstanceLeafBytes = 128;   // GEN_RT_BVH_INSTANCE_LEAF_length * 4
constexpr uint32_t kLeafDescBytes = 8;         // GEN_RT_BVH_PRIMITIVE_LEAF_DESCRIPTOR_length * 4
constexpr uint32_t kQuadLeafBytes = 64;        // GEN_RT_BVH_QUAD_LEAF_length * 4
constexpr uint32_t kProceduralLeafBytes = 64;  // GEN_RT_BVH_PROCEDURAL_LEAF_length * 4

// Child types stored in bits 2..5 of an internal node's child-info byte.
enum ChildType : uint32_t {
  CT_INTERNAL = 0,
  CT_INSTANCE = 1,
  CT_PROCEDURAL = 3,
  CT_QUAD = 4,
};

// Transaction types, numbered as TransactionType (abstract_hardware_model.h:201-211).
enum TxType : uint32_t {
  TX_STRUCTURE = 0,
  TX_INTERNAL = 1,
  TX_INSTANCE_LEAF = 2,
  TX_LEAF_DESC = 3,
  TX_QUAD_LEAF = 4,
  TX_QUAD_LEAF_HIT = 5,
  TX_PROCEDURAL_LEAF = 6,
};

RT_HD uint32_t tx_bytes(uint32_t t) {
  // STRUCTURE, INTERNAL, INSTANCE_LEAF, LEAF_DESC, QUAD, QUAD_HIT, PROCEDURAL
  return t == TX_INSTANCE_LEAF ? 128u : (t == TX_LEAF_DESC ? 8u : 64u);
}

// ---- GEN_RT_BVH header (64 B) ----
constexpr uint32_t HDR_ROOT_OFFSET = 0;  // u64, bytes, relative to the header
constexpr uint32_t HDR_BOUNDS_MIN = 8;   // f32 x3
constexpr uint32_t HDR_BOUNDS_MAX = 20;  // f32 x3

// ---- internal node (64 B) ----
constexpr uint32_t IN_ORIGIN = 0;        // f32 x3
constexpr uint32_t IN_CHILD_OFFSET = 12; // i32, in 64 B units, relative to the node
constexpr uint32_t IN_NODE_TYPE = 16;    // u8
constexpr uint32_t IN_EXP = 18;          // i8 x3 (X, Y, Z)
constexpr uint32_t IN_RAY_MASK = 21;     // u8 (not used by the walk)
constexpr uint32_t IN_CHILD_INFO = 22;   // u8 x6: bits 0-1 size (64 B units), bits 2-5 type
constexpr uint32_t IN_LO_X = 28;         // u8 x6 each
constexpr uint32_t IN_HI_X = 34;
constexpr uint32_t IN_LO_Y = 40;
constexpr uint32_t IN_HI_Y = 46;
constexpr uint32_t IN_LO_Z = 52;
constexpr uint32_t IN_HI_Z = 58;

// ---- instance leaf (128 B) ----
constexpr uint32_t IL_SHADER_MASK = 0;     // u24 shader index | u8 geometry ray mask
constexpr uint32_t IL_HITGROUP_FLAGS = 4;  // u24 hit-group contribution | u8 (leaf type, geometry flags)
constexpr uint32_t IL_START_NODE = 8;      // u48 (unused by the walk)
constexpr uint32_t IL_INSTANCE_FLAGS = 14; // u8
constexpr uint32_t IL_W2O_LINEAR = 16;     // f32 x9, rows 0-2 of the world-to-object matrix
constexpr uint32_t IL_SLOT_52 = 52;        // f32 x3, decoded as WorldToObjectm30..32
constexpr uint32_t IL_BVH_ADDRESS = 64;    // u64, bytes from this leaf to the BLAS header
constexpr uint32_t IL_INSTANCE_ID = 72;    // u32
constexpr uint32_t IL_INSTANCE_INDEX = 76; // u32
constexpr uint32_t IL_O2W_LINEAR = 80;     // f32 x9, rows 0-2 of the object-to-world matrix
constexpr uint32_t IL_SLOT_116 = 116;      // f32 x3, decoded as ObjectToWorldm30..32
// The reference reads each 4x3 matrix as 12 consecutive floats of its
// decoded struct (instance_leaf_matrix_to_float4x4, asu.h:210-224), and the
// struct lists ObjectToWorldm30..32 right after WorldToObjectm22.  The
// effective matrices the walk uses are therefore:
//   world-to-object = rows from bytes 16..51, translation row from bytes 116..127
//   object-to-world = rows from bytes 80..115, translation row from bytes 52..63
constexpr uint32_t IL_W2O_TRANSLATION = IL_SLOT_116;
constexpr uint32_t IL_O2W_TRANSLATION = IL_SLOT_52;

// ---- primitive leaf descriptor (first 8 B of a quad / procedural leaf) ----
constexpr uint32_t PL_SHADER_MASK = 0;  // u24 shader index | u8 geometry ray mask
constexpr uint32_t PL_GEOM = 4;         // u32: geometry index bits 0-27, leaf type bit 29, flags 30-31

// ---- quad leaf (64 B) ----
constexpr uint32_t QL_PRIM0 = 8;        // u32 PrimitiveIndex0
constexpr uint32_t QL_PRIM1 = 12;       // u32: PrimitiveIndex1Delta bits 0-16, j0/j1/j2 bits 17-22
constexpr uint32_t QL_V0 = 16;          // f32 x3 x4 vertices; only v0..v2 are tested
constexpr uint32_t QL_V1 = 28;
constexpr uint32_t QL_V2 = 40;
constexpr uint32_t QL_V3 = 52;

// ---- procedural leaf (64 B) ----
constexpr uint32_t PR_COUNT = 8;        // u32: NumPrimitives bits 0-3, LastPrimitive bits 19-31
constexpr uint32_t PR_PRIMS = 12;       // u32 x13

RT_HD uint32_t child_size_units(uint8_t info) { return info & 0x3u; }
RT_HD uint32_t child_type(uint8_t info) { return (uint32_t)(info & 0x3fu) >> 2; }
RT_HD uint32_t leaf_type_of(uint32_t geom_word) { return (geom_word >> 29) & 1u; }  // 0 = quad
RT_HD uint32_t geometry_index_of(uint32_t geom_word) { return geom_word & 0x0fffffffu; }

// SPIR-V ray flags (SPV_KHR_ray_tracing).  The walk honours Opaque,
// TerminateOnFirstHit and SkipClosestHitShader; cull flags and masks are
// ignored, as in the reference.
constexpr uint32_t RAY_FLAG_OPAQUE = 0x1;
constexpr uint32_t RAY_FLAG_NO_OPAQUE = 0x2;
constexpr uint32_t RAY_FLAG_TERMINATE_ON_FIRST_HIT = 0x4;
constexpr uint32_t RAY_FLAG_SKIP_CLOSEST_HIT = 0x8;

// Packed trace entry: unit index << 3 | transaction type.
RT_HD uint32_t pack_visit(uint32_t unit, uint32_t type) { return (unit << 3) | type; }
RT_HD uint32_t visit_unit(uint32_t v) { return v >> 3; }
RT_HD uint32_t visit_type(uint32_t v) { return v & 7u; }

}  // namespace rtf
