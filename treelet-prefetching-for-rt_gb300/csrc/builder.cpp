// Binned-SAH BVH builder emitting the reference's 6-wide node layout.
//
// 1. A binary BVH is built top-down over primitive centroids with 16 SAH bins
//    per split (one primitive per leaf: the layout has one triangle per quad
//    leaf, vulkan_ray_tracing.cc:2824 asserts PrimitiveIndex1Delta == 0).
// 2. It is collapsed to 6-wide nodes by repeatedly opening the child with the
//    largest surface area.
// 3. Nodes are laid out depth first: each node's children form one
//    contiguous block (the walk advances child_addr by ChildSize * 64,
//    vulkan_ray_tracing.cc:2555-2593), internal children of a block are then
//    laid out in order.
// 4. Child boxes are quantized to 8 bits per side against the node origin with
//    a per-axis power-of-two scale, rounded outward so that the dequantized
//    box (Origin + ldexpf(q, exp - 8), asu.h:499-508) contains the exact box.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstring>
#include <string>
#include <thread>

#include "builder.h"
#include "format.h"
#include "rtmath.h"

namespace rtb {
namespace {

struct AABB {
  float lo[3] = {INFINITY, INFINITY, INFINITY};
  float hi[3] = {-INFINITY, -INFINITY, -INFINITY};
  void grow(const AABB& b) {
    for (int a = 0; a < 3; ++a) {
      lo[a] = std::min(lo[a], b.lo[a]);
      hi[a] = std::max(hi[a], b.hi[a]);
    }
  }
  void grow(const float* p) {
    for (int a = 0; a < 3; ++a) {
      lo[a] = std::min(lo[a], p[a]);
      hi[a] = std::max(hi[a], p[a]);
    }
  }
  double area() const {
    double d[3];
    for (int a = 0; a < 3; ++a) d[a] = std::max(0.0, (double)hi[a] - (double)lo[a]);
    return 2.0 * (d[0] * d[1] + d[1] * d[2] + d[0] * d[2]);
  }
};

struct BNode {
  AABB box;
  int32_t left = -1, right = -1;  // children, or -1
  int32_t prim = -1;              // primitive index for a leaf
};

struct Binary {
  std::vector<BNode> nodes;
  int32_t root = -1;
};

// Builds a binary SAH tree over the given primitive boxes.
void build_binary(const std::vector<AABB>& prim_box, Binary& out) {
  const uint32_t n = (uint32_t)prim_box.size();
  out.nodes.clear();
  out.nodes.reserve(2 * (size_t)n);
  std::vector<uint32_t> idx(n);
  std::vector<float> cen(3 * (size_t)n);
  for (uint32_t i = 0; i < n; ++i) {
    idx[i] = i;
    for (int a = 0; a < 3; ++a) cen[3 * (size_t)i + a] = 0.5f * (prim_box[i].lo[a] + prim_box[i].hi[a]);
  }
  struct Task {
    uint32_t begin, end;
    int32_t node;
  };
  std::vector<Task> work;
  out.nodes.emplace_back();
  out.root = 0;
  work.push_back({0, n, 0});
  constexpr int kBins = 16;
  while (!work.empty()) {
    Task t = work.back();
    work.pop_back();
    AABB box, cbox;
    for (uint32_t i = t.begin; i < t.end; ++i) {
      box.grow(prim_box[idx[i]]);
      cbox.grow(&cen[3 * (size_t)idx[i]]);
    }
    out.nodes[t.node].box = box;
    const uint32_t count = t.end - t.begin;
    if (count == 1) {
      out.nodes[t.node].prim = (int32_t)idx[t.begin];
      continue;
    }
    int axis = 0;
    float ext[3];
    for (int a = 0; a < 3; ++a) ext[a] = cbox.hi[a] - cbox.lo[a];
    if (ext[1] > ext[axis]) axis = 1;
    if (ext[2] > ext[axis]) axis = 2;
    uint32_t mid;
    if (!(ext[axis] > 0.0f)) {
      mid = t.begin + count / 2;
    } else {
      AABB bb[kBins];
      uint32_t bc[kBins] = {0};
      const double scale = (double)kBins / (double)ext[axis];
      auto bin_of = [&](uint32_t p) {
        int b = (int)(((double)cen[3 * (size_t)p + axis] - (double)cbox.lo[axis]) * scale);
        return std::min(std::max(b, 0), kBins - 1);
      };
      for (uint32_t i = t.begin; i < t.end; ++i) {
        const int b = bin_of(idx[i]);
        bc[b]++;
        bb[b].grow(prim_box[idx[i]]);
      }
      double right_area[kBins];
      uint32_t right_cnt[kBins];
      AABB acc;
      uint32_t cnt = 0;
      for (int b = kBins - 1; b > 0; --b) {
        acc.grow(bb[b]);
        cnt += bc[b];
        right_area[b] = acc.area();
        right_cnt[b] = cnt;
      }
      AABB lacc;
      uint32_t lcnt = 0;
      double best = INFINITY;
      int best_b = -1;
      for (int b = 1; b < kBins; ++b) {
        lacc.grow(bb[b - 1]);
        lcnt += bc[b - 1];
        if (lcnt == 0 || right_cnt[b] == 0) continue;
        const double cost = lacc.area() * lcnt + right_area[b] * right_cnt[b];
        if (cost < best) {
          best = cost;
          best_b = b;
        }
      }
      if (best_b < 0) {
        mid = t.begin + count / 2;
        std::nth_element(idx.begin() + t.begin, idx.begin() + mid, idx.begin() + t.end,
                         [&](uint32_t a, uint32_t b) {
                           const float ca = cen[3 * (size_t)a + axis], cb = cen[3 * (size_t)b + axis];
                           return ca < cb || (ca == cb && a < b);
                         });
      } else {
        auto it = std::stable_partition(idx.begin() + t.begin, idx.begin() + t.end,
                                        [&](uint32_t p) { return bin_of(p) < best_b; });
        mid = (uint32_t)(it - idx.begin());
        if (mid == t.begin || mid == t.end) mid = t.begin + count / 2;
      }
    }
    const int32_t l = (int32_t)out.nodes.size();
    out.nodes.emplace_back();
    const int32_t r = (int32_t)out.nodes.size();
    out.nodes.emplace_back();
    out.nodes[t.node].left = l;
    out.nodes[t.node].right = r;
    work.push_back({mid, t.end, r});
    work.push_back({t.begin, mid, l});
  }
}

// Children of a wide node: binary-node ids (leaves or internal).
void collapse_children(const Binary& b, int32_t node, std::vector<int32_t>& ch) {
  ch.clear();
  const BNode& n = b.nodes[node];
  if (n.prim >= 0) {
    ch.push_back(node);
    return;
  }
  ch.push_back(n.left);
  ch.push_back(n.right);
  while (ch.size() < 6) {
    int best = -1;
    double best_area = -1.0;
    for (int i = 0; i < (int)ch.size(); ++i) {
      const BNode& c = b.nodes[ch[i]];
      if (c.prim >= 0) continue;
      const double a = c.box.area();
      if (a > best_area) {
        best_area = a;
        best = i;
      }
    }
    if (best < 0) break;
    const int32_t open = ch[best];
    ch[best] = b.nodes[open].left;
    ch.insert(ch.begin() + best + 1, b.nodes[open].right);
  }
}

void put_u32(uint8_t* p, uint32_t v) { std::memcpy(p, &v, 4); }
void put_i32(uint8_t* p, int32_t v) { std::memcpy(p, &v, 4); }
void put_u64(uint8_t* p, uint64_t v) { std::memcpy(p, &v, 8); }
void put_f32(uint8_t* p, float v) { std::memcpy(p, &v, 4); }

float dequant(float origin, uint32_t q, int e) {
  return origin + std::ldexp((float)q, e - 8);
}

// Quantizes one axis of up to 6 child boxes.  Returns the exponent.
int quantize_axis(float origin, float node_hi, const float* clo, const float* chi, int nc, uint8_t* qlo,
                  uint8_t* qhi) {
  const double extent = (double)node_hi - (double)origin;
  int e;
  if (!(extent > 0.0)) {
    e = -128;
  } else {
    int p;
    std::frexp(extent / 255.0, &p);  // extent/255 in [2^(p-1), 2^p)
    e = p + 8;
    e = std::max(-128, std::min(127, e));
  }
  for (;; ++e) {
    bool ok = true;
    for (int c = 0; c < nc && ok; ++c) {
      const double s = std::ldexp(1.0, e - 8);
      long lo = (long)std::floor(((double)clo[c] - (double)origin) / s);
      lo = std::max(0L, std::min(255L, lo));
      while (lo > 0 && dequant(origin, (uint32_t)lo, e) > clo[c]) --lo;
      long hi = (long)std::ceil(((double)chi[c] - (double)origin) / s);
      hi = std::max(0L, hi);
      while (hi <= 255 && dequant(origin, (uint32_t)hi, e) < chi[c]) ++hi;
      if (hi > 255) {
        ok = false;
        break;
      }
      qlo[c] = (uint8_t)lo;
      qhi[c] = (uint8_t)hi;
    }
    if (ok || e >= 127) return e;
  }
}

struct WideChild {
  AABB box;
  uint32_t type;   // rtf::ChildType
  uint32_t units;  // size in 64 B units
  int32_t ref;     // binary node id (internal) or primitive id (leaf)
};

// Writes an internal node at byte offset `off` with children block at `block`.
void write_internal(uint8_t* blob, uint64_t off, uint64_t block, const AABB& box,
                    const std::vector<WideChild>& ch) {
  uint8_t* p = blob + off;
  std::memset(p, 0, 64);
  for (int a = 0; a < 3; ++a) put_f32(p + rtf::IN_ORIGIN + 4 * a, box.lo[a]);
  put_i32(p + rtf::IN_CHILD_OFFSET, (int32_t)((int64_t)(block - off) / 64));
  p[rtf::IN_NODE_TYPE] = 0;
  p[rtf::IN_RAY_MASK] = 0xff;
  const int nc = (int)ch.size();
  float clo[6], chi[6];
  uint8_t qlo[6] = {0}, qhi[6] = {0};
  const uint32_t lo_off[3] = {rtf::IN_LO_X, rtf::IN_LO_Y, rtf::IN_LO_Z};
  const uint32_t hi_off[3] = {rtf::IN_HI_X, rtf::IN_HI_Y, rtf::IN_HI_Z};
  for (int a = 0; a < 3; ++a) {
    for (int c = 0; c < nc; ++c) {
      clo[c] = ch[c].box.lo[a];
      chi[c] = ch[c].box.hi[a];
    }
    const int e = quantize_axis(box.lo[a], box.hi[a], clo, chi, nc, qlo, qhi);
    p[rtf::IN_EXP + a] = (uint8_t)(int8_t)e;
    for (int c = 0; c < nc; ++c) {
      p[lo_off[a] + c] = qlo[c];
      p[hi_off[a] + c] = qhi[c];
    }
  }
  for (int c = 0; c < nc; ++c) p[rtf::IN_CHILD_INFO + c] = (uint8_t)((ch[c].units & 3u) | (ch[c].type << 2));
}

void write_header(uint8_t* blob, uint64_t off, uint64_t root_off, const AABB& box) {
  uint8_t* p = blob + off;
  std::memset(p, 0, 64);
  put_u64(p + rtf::HDR_ROOT_OFFSET, root_off - off);
  for (int a = 0; a < 3; ++a) {
    put_f32(p + rtf::HDR_BOUNDS_MIN + 4 * a, box.lo[a]);
    put_f32(p + rtf::HDR_BOUNDS_MAX + 4 * a, box.hi[a]);
  }
}

void write_quad(uint8_t* blob, uint64_t off, const float* tri, uint32_t prim, uint32_t geom) {
  uint8_t* p = blob + off;
  std::memset(p, 0, 64);
  put_u32(p + rtf::PL_SHADER_MASK, 0xff000000u);
  put_u32(p + rtf::PL_GEOM, (geom & 0x0fffffffu) | (1u << 30));  // quad, opaque geometry
  put_u32(p + rtf::QL_PRIM0, prim);
  put_u32(p + rtf::QL_PRIM1, (0u << 17) | (1u << 19) | (2u << 21));
  for (int v = 0; v < 3; ++v)
    for (int a = 0; a < 3; ++a) put_f32(p + rtf::QL_V0 + 12 * v + 4 * a, tri[3 * v + a]);
  for (int a = 0; a < 3; ++a) put_f32(p + rtf::QL_V3 + 4 * a, tri[6 + a]);
}

// Inverse of a row-vector affine transform, in double.
void invert_affine(const float m[4][3], double inv[4][3]) {
  // world = p * L + t  =>  p = (world - t) * L^-1
  const double a = m[0][0], b = m[0][1], c = m[0][2];
  const double d = m[1][0], e = m[1][1], f = m[1][2];
  const double g = m[2][0], h = m[2][1], i = m[2][2];
  const double A = e * i - f * h, B = -(d * i - f * g), C = d * h - e * g;
  const double det = a * A + b * B + c * C;
  const double r = 1.0 / det;
  double L[3][3] = {{A * r, -(b * i - c * h) * r, (b * f - c * e) * r},
                    {B * r, (a * i - c * g) * r, -(a * f - c * d) * r},
                    {C * r, -(a * h - b * g) * r, (a * e - b * d) * r}};
  for (int j = 0; j < 3; ++j)
    for (int k = 0; k < 3; ++k) inv[j][k] = L[j][k];
  for (int k = 0; k < 3; ++k) {
    double s = 0;
    for (int j = 0; j < 3; ++j) s += (double)m[3][j] * L[j][k];
    inv[3][k] = -s;
  }
}

void write_instance(uint8_t* blob, uint64_t off, uint64_t blas_hdr, const Instance& in, uint32_t index) {
  uint8_t* p = blob + off;
  std::memset(p, 0, 128);
  put_u32(p + rtf::IL_SHADER_MASK, 0xff000000u);
  put_u32(p + rtf::IL_HITGROUP_FLAGS, 0u);
  double w2o[4][3];
  invert_affine(in.o2w, w2o);
  for (int j = 0; j < 3; ++j)
    for (int k = 0; k < 3; ++k) {
      put_f32(p + rtf::IL_W2O_LINEAR + 4 * (3 * j + k), (float)w2o[j][k]);
      put_f32(p + rtf::IL_O2W_LINEAR + 4 * (3 * j + k), in.o2w[j][k]);
    }
  // Translation rows go where the reference's struct-order matrix read
  // picks them up (format.h: IL_W2O_TRANSLATION / IL_O2W_TRANSLATION).
  for (int k = 0; k < 3; ++k) {
    put_f32(p + rtf::IL_W2O_TRANSLATION + 4 * k, (float)w2o[3][k]);
    put_f32(p + rtf::IL_O2W_TRANSLATION + 4 * k, in.o2w[3][k]);
  }
  put_u64(p + rtf::IL_BVH_ADDRESS, blas_hdr - off);
  put_u32(p + rtf::IL_INSTANCE_ID, in.instance_id);
  put_u32(p + rtf::IL_INSTANCE_INDEX, index);
}

AABB tri_box(const float* t) {
  AABB b;
  b.grow(t);
  b.grow(t + 3);
  b.grow(t + 6);
  return b;
}

// World box of a transformed object box, widened by a relative epsilon.
AABB transform_box(const AABB& ob, const float m[4][3]) {
  AABB w;
  for (int c = 0; c < 8; ++c) {
    const double p[3] = {(c & 1) ? ob.hi[0] : ob.lo[0], (c & 2) ? ob.hi[1] : ob.lo[1],
                         (c & 4) ? ob.hi[2] : ob.lo[2]};
    float q[3];
    for (int k = 0; k < 3; ++k) {
      double s = m[3][k];
      for (int j = 0; j < 3; ++j) s += p[j] * (double)m[j][k];
      q[k] = (float)s;
    }
    w.grow(q);
  }
  for (int a = 0; a < 3; ++a) {
    const float pad = 1e-5f * std::max(1.0f, std::max(std::fabs(w.lo[a]), std::fabs(w.hi[a])));
    w.lo[a] -= pad;
    w.hi[a] += pad;
  }
  return w;
}

// Lays out one tree (TLAS or BLAS) depth first starting at `root_off`.
// `leaf_units` is the size of a leaf child (1 for quads, 2 for instances).
// `emit_leaf(prim, offset)` writes a leaf.  Returns the end offset.
template <class EmitLeaf>
uint64_t layout_tree(uint8_t* blob, bool write, const Binary& b, uint64_t root_off, uint32_t leaf_type,
                     uint32_t leaf_units, EmitLeaf&& emit_leaf, BuildStats* st, uint32_t depth0) {
  struct Item {
    int32_t bnode;
    uint64_t off;
    uint32_t depth;
  };
  std::vector<Item> stack;
  stack.push_back({b.root, root_off, depth0});
  uint64_t cursor = root_off + 64;
  std::vector<int32_t> ch;
  std::vector<WideChild> wc;
  std::vector<Item> next;
  while (!stack.empty()) {
    Item it = stack.back();
    stack.pop_back();
    collapse_children(b, it.bnode, ch);
    wc.clear();
    for (int32_t c : ch) {
      const BNode& n = b.nodes[c];
      WideChild w;
      w.box = n.box;
      if (n.prim >= 0) {
        w.type = leaf_type;
        w.units = leaf_units;
        w.ref = n.prim;
      } else {
        w.type = rtf::CT_INTERNAL;
        w.units = 1;
        w.ref = c;
      }
      wc.push_back(w);
    }
    const uint64_t block = cursor;
    if (write) write_internal(blob, it.off, block, b.nodes[it.bnode].box, wc);
    if (st) {
      st->internal_nodes++;
      st->max_depth = std::max(st->max_depth, it.depth);
    }
    next.clear();
    uint64_t c_off = block;
    for (const WideChild& w : wc) {
      if (w.type == rtf::CT_INTERNAL) {
        next.push_back({w.ref, c_off, it.depth + 1});
      } else {
        if (write) emit_leaf((uint32_t)w.ref, c_off);
        if (st) st->leaves++;
      }
      c_off += 64ull * w.units;
    }
    cursor = c_off;
    for (auto r = next.rbegin(); r != next.rend(); ++r) stack.push_back(*r);
  }
  return cursor;
}

}  // namespace

bool build_scene(const std::vector<Mesh>& meshes, const std::vector<Instance>& instances,
                 std::vector<uint8_t>& blob, BuildStats* stats, std::string* err) {
  if (instances.empty()) {
    if (err) *err = "scene has no instances";
    return false;
  }
  for (const Instance& in : instances) {
    if (in.mesh >= meshes.size() || meshes[in.mesh].n() == 0) {
      if (err) *err = "instance references a missing or empty mesh";
      return false;
    }
  }
  // Only meshes that some instance uses get a BLAS.
  std::vector<int> used(meshes.size(), 0);
  for (const Instance& in : instances) used[in.mesh] = 1;

  std::vector<Binary> blas(meshes.size());
  std::vector<AABB> blas_box(meshes.size());
  {
    std::vector<std::thread> th;
    const unsigned hw = std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
    std::vector<size_t> order;
    for (size_t m = 0; m < meshes.size(); ++m)
      if (used[m]) order.push_back(m);
    std::sort(order.begin(), order.end(), [&](size_t a, size_t b) { return meshes[a].n() > meshes[b].n(); });
    std::atomic_size_t next{0};
    auto worker = [&]() {
      for (;;) {
        const size_t k = next.fetch_add(1);
        if (k >= order.size()) return;
        const size_t m = order[k];
        const Mesh& mesh = meshes[m];
        std::vector<AABB> pb(mesh.n());
        for (uint32_t t = 0; t < mesh.n(); ++t) pb[t] = tri_box(&mesh.tris[9 * (size_t)t]);
        build_binary(pb, blas[m]);
        blas_box[m] = blas[m].nodes[blas[m].root].box;
      }
    };
    for (unsigned i = 0; i < hw; ++i) th.emplace_back(worker);
    for (auto& t : th) t.join();
  }
  std::vector<AABB> inst_box(instances.size());
  for (size_t i = 0; i < instances.size(); ++i) inst_box[i] = transform_box(blas_box[instances[i].mesh], instances[i].o2w);
  Binary tlas;
  build_binary(inst_box, tlas);

  BuildStats st;
  // Pass 1: sizes.  TLAS header at 0, TLAS root at 64.
  auto noop = [](uint32_t, uint64_t) {};
  uint64_t end = layout_tree(nullptr, false, tlas, 64, rtf::CT_INSTANCE, 2, noop, nullptr, 1);
  std::vector<uint64_t> hdr_off(meshes.size(), 0);
  for (size_t m = 0; m < meshes.size(); ++m) {
    if (!used[m]) continue;
    hdr_off[m] = end;
    end = layout_tree(nullptr, false, blas[m], end + 64, rtf::CT_QUAD, 1, noop, nullptr, 1);
  }
  if (end / 64 >= (1ull << 29)) {
    if (err) *err = "scene exceeds 32 GiB (unit index must fit 29 bits)";
    return false;
  }
  blob.assign(end, 0);
  uint8_t* B = blob.data();
  write_header(B, 0, 64, tlas.nodes[tlas.root].box);
  uint32_t inst_counter = 0;
  layout_tree(
      B, true, tlas, 64, rtf::CT_INSTANCE, 2,
      [&](uint32_t prim, uint64_t off) {
        const Instance& in = instances[prim];
        write_instance(B, off, hdr_off[in.mesh], in, prim);
        inst_counter++;
      },
      &st, 1);
  st.instance_leaves = st.leaves;
  st.leaves = 0;
  for (size_t m = 0; m < meshes.size(); ++m) {
    if (!used[m]) continue;
    write_header(B, hdr_off[m], hdr_off[m] + 64, blas_box[m]);
    const Mesh& mesh = meshes[m];
    layout_tree(
        B, true, blas[m], hdr_off[m] + 64, rtf::CT_QUAD, 1,
        [&](uint32_t prim, uint64_t off) { write_quad(B, off, &mesh.tris[9 * (size_t)prim], prim, mesh.geometry_index); },
        &st, 1);
  }
  if (stats) *stats = st;
  return true;
}

}  // namespace rtb
