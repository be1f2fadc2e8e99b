// Array-based restatement of the reference's greedy treelet partition.
//
// createTreelets (src/cuda-sim/vulkan_ray_tracing.cc:823-1470) walks the BVH
// breadth first from a pending root, charging each node's bytes against the
// budget, until the next frontier node does not fit; then every frontier node
// becomes a pending root (FIFO) and the walk restarts from the oldest pending
// root.  Charges: header 64, internal node 64, instance leaf 128 plus its
// BLAS header 64, primitive leaf 64; the fit check looks ahead with 192 for
// an instance leaf and 64 otherwise.  The first treelet is rooted at the TLAS
// header.  A root completed twice keeps its last member list (std::map
// assignment); member lists are de-duplicated keeping first occurrences; the
// node -> root map is filled in ascending root order so the largest root
// containing a node wins (buildNodeToRootMap, :475-489).
#include "treelets.h"

#include <algorithm>
#include <cstring>
#include <deque>
#include <unordered_map>

#include "format.h"
#include "pinned.h"
#include "rtmath.h"

namespace rtt {
namespace {

struct Entry {
  uint32_t unit;
  uint8_t top, leaf;
  uint16_t size;   // StackEntry::size
  uint16_t look;   // nodesize_stack value (fit check)
};

template <class T>
T rd(const uint8_t* b, uint64_t off) {
  T v;
  std::memcpy(&v, b + off, sizeof(T));
  return v;
}

}  // namespace

bool form_treelets(const uint8_t* blob, uint64_t n_bytes, uint32_t max_bytes, Partition& out, std::string* err) {
  auto bad = [&](const std::string& m) {
    if (err) *err = m;
    return false;
  };
  if (n_bytes < 128 || (n_bytes % 64) != 0) return bad("blob too small or not a multiple of 64 bytes");
  if (max_bytes < 192) return bad("max_treelet_bytes must be at least 192 (an instance leaf and its BLAS header)");
  if (max_bytes > (1u << (kSlotBits + 6))) return bad("max_treelet_bytes above 65536 is not supported");
  const uint64_t n_units = n_bytes / 64;
  out = Partition();
  out.max_bytes = max_bytes;

  // completed root -> member list (last completion wins)
  std::unordered_map<uint32_t, uint32_t> completed_idx;  // root -> index into lists
  std::vector<uint32_t> completed_root;
  std::vector<uint16_t> completed_root_size;
  std::vector<std::vector<std::pair<uint32_t, uint16_t>>> completed_members;

  std::deque<Entry> pq;     // treelet_roots_pending_work_queue
  std::deque<Entry> stack;  // currently considered nodes (FIFO)
  std::vector<std::pair<uint32_t, uint16_t>> nct;  // nodes_in_current_treelet

  const uint64_t root_off = rd<uint64_t>(blob, rtf::HDR_ROOT_OFFSET);
  if (root_off % 64 || root_off >= n_bytes) return bad("TLAS RootNodeOffset out of range");
  int64_t remaining = (int64_t)max_bytes - 64;
  pq.push_back(Entry{0, 1, 0, 64, 128});
  nct.push_back({0u, (uint16_t)64});
  stack.push_back(Entry{(uint32_t)(root_off / 64), 1, 0, 64, 64});

  auto complete = [&]() {
    const Entry& r = pq.front();
    auto it = completed_idx.find(r.unit);
    if (it == completed_idx.end()) {
      completed_idx.emplace(r.unit, (uint32_t)completed_root.size());
      completed_root.push_back(r.unit);
      completed_root_size.push_back(r.size);
      completed_members.push_back(nct);
    } else {
      completed_members[it->second] = nct;
    }
    pq.pop_front();
    nct.clear();
  };

  auto check_unit = [&](uint64_t u, uint32_t units) { return u + units <= n_units; };

  while (!pq.empty()) {
    Entry node = stack.front();
    stack.pop_front();
    for (;;) {
      if (!check_unit(node.unit, node.top && node.leaf ? 2 : 1)) return bad("node outside the blob");
      const uint64_t off = (uint64_t)node.unit * 64;
      if (node.top && !node.leaf) {
        remaining -= 64;
        if (remaining < 0) return bad("treelet budget exceeded by a root");
        nct.push_back({node.unit, node.size});
        const int32_t child_off = rd<int32_t>(blob, off + rtf::IN_CHILD_OFFSET);
        int64_t c = (int64_t)node.unit + child_off;
        for (int i = 0; i < 6; ++i) {
          const uint8_t info = blob[off + rtf::IN_CHILD_INFO + i];
          const uint32_t sz = rtf::child_size_units(info);
          if (sz > 0) {
            if (c < 0) return bad("child pointer before the blob");
            if (rtf::child_type(info) != rtf::CT_INTERNAL) {
              stack.push_back(Entry{(uint32_t)c, 1, 1, 128, 192});
            } else {
              stack.push_back(Entry{(uint32_t)c, 1, 0, 64, 64});
            }
          }
          c += sz;
        }
      } else if (node.top && node.leaf) {
        remaining -= 128;
        nct.push_back({node.unit, node.size});
        const uint64_t bvh = rd<uint64_t>(blob, off + rtf::IL_BVH_ADDRESS);
        const uint64_t hdr = off + bvh;
        if (hdr % 64 || hdr + 64 > n_bytes) return bad("instance BVHAddress out of range");
        remaining -= 64;
        if (remaining < 0) return bad("treelet budget exceeded by a root");
        nct.push_back({(uint32_t)(hdr / 64), (uint16_t)64});
        const uint64_t broot = hdr + rd<uint64_t>(blob, hdr + rtf::HDR_ROOT_OFFSET);
        if (broot % 64 || broot + 64 > n_bytes) return bad("BLAS RootNodeOffset out of range");
        stack.push_back(Entry{(uint32_t)(broot / 64), 0, 0, 64, 64});
      } else if (!node.top && !node.leaf) {
        remaining -= 64;
        if (remaining < 0) return bad("treelet budget exceeded by a root");
        nct.push_back({node.unit, node.size});
        const int32_t child_off = rd<int32_t>(blob, off + rtf::IN_CHILD_OFFSET);
        int64_t c = (int64_t)node.unit + child_off;
        for (int i = 0; i < 6; ++i) {
          const uint8_t info = blob[off + rtf::IN_CHILD_INFO + i];
          const uint32_t sz = rtf::child_size_units(info);
          if (sz > 0) {
            if (c < 0) return bad("child pointer before the blob");
            if (rtf::child_type(info) != rtf::CT_INTERNAL)
              stack.push_back(Entry{(uint32_t)c, 0, 1, 64, 64});
            else
              stack.push_back(Entry{(uint32_t)c, 0, 0, 64, 64});
          }
          c += sz;
        }
      } else {
        nct.push_back({node.unit, node.size});
        remaining -= 64;  // quad and procedural leaves are both charged 64
        if (remaining < 0) return bad("treelet budget exceeded by a root");
      }
      if (!stack.empty() && remaining - (int64_t)stack.front().look >= 0) {
        node = stack.front();
        stack.pop_front();
        continue;
      }
      if (!stack.empty()) {
        complete();
        for (const Entry& e : stack) pq.push_back(e);
        stack.clear();
        stack.push_back(pq.front());
      } else {
        complete();
        if (!pq.empty()) stack.push_back(pq.front());
      }
      remaining = max_bytes;
      break;
    }
  }

  // Ascending root order (treelet_addr_to_metadata_idx).
  const uint32_t n = (uint32_t)completed_root.size();
  std::vector<uint32_t> order(n);
  for (uint32_t i = 0; i < n; ++i) order[i] = i;
  std::sort(order.begin(), order.end(), [&](uint32_t a, uint32_t b) { return completed_root[a] < completed_root[b]; });
  out.roots.resize(n);
  out.root_bytes.resize(n);
  out.member_first.assign(n + 1, 0);
  std::vector<uint32_t> stamp(n_units, kNoTreelet);
  for (uint32_t k = 0; k < n; ++k) {
    const uint32_t i = order[k];
    out.roots[k] = completed_root[i];
    out.root_bytes[k] = completed_root_size[i];
    for (const auto& m : completed_members[i]) {
      if (stamp[m.first] == k) continue;
      stamp[m.first] = k;
      out.members.push_back(m.first);
      out.member_bytes.push_back(m.second);
    }
    out.member_first[k + 1] = out.members.size();
  }
  out.node_root.assign(n_units, kNoTreelet);
  std::vector<uint32_t> node_dense(n_units, kNoTreelet);
  for (uint32_t k = 0; k < n; ++k) {
    out.node_root[out.roots[k]] = out.roots[k];
    node_dense[out.roots[k]] = k;
    for (uint64_t j = out.member_first[k]; j < out.member_first[k + 1]; ++j) {
      out.node_root[out.members[j]] = out.roots[k];
      node_dense[out.members[j]] = k;
    }
  }
  // Images: members back to back; node_loc points into the image of the
  // treelet the node maps to.
  out.image_off.assign(n + 1, 0);
  out.node_loc.assign(n_units, kNoTreelet);
  uint64_t pos = 0;
  for (uint32_t k = 0; k < n; ++k) {
    out.image_off[k] = pos;
    uint64_t b = 0;
    for (uint64_t j = out.member_first[k]; j < out.member_first[k + 1]; ++j) {
      const uint32_t u = out.members[j];
      if (node_dense[u] == k && out.node_loc[u] == kNoTreelet && k < kMaxDense)
        out.node_loc[u] = (k << kSlotBits) | (uint32_t)(b / 64);
      b += out.member_bytes[j];
    }
    out.largest_image = std::max<uint32_t>(out.largest_image, (uint32_t)b);
    pos += b;
  }
  out.image_off[n] = pos;
  out.image_bytes = pos;
  return true;
}

void build_images(const uint8_t* blob, const Partition& p, std::vector<uint8_t>& store) {
  store.assign(p.image_bytes, 0);
  const uint32_t n = (uint32_t)p.roots.size();
  for (uint32_t k = 0; k < n; ++k) {
    uint64_t pos = p.image_off[k];
    for (uint64_t j = p.member_first[k]; j < p.member_first[k + 1]; ++j) {
      std::memcpy(store.data() + pos, blob + (uint64_t)p.members[j] * 64, p.member_bytes[j]);
      pos += p.member_bytes[j];
    }
  }
}

void route_masks(const uint8_t* blob, uint64_t n_bytes, const Partition& p, std::vector<uint16_t>& out) {
  const uint64_t n_units = n_bytes / 64;
  out.assign(n_units, 0);
  auto root_of = [&](uint32_t u) {
    u &= kEntryUnitMask;
    return u < n_units ? p.node_root[u] : kNoTreelet;
  };
  // bit `same` if the child shares u's root, bit `other` if its root is u
  auto bits = [&](uint32_t u, uint32_t child, uint32_t same, uint32_t other) -> uint16_t {
    const uint32_t rc = root_of(child);
    uint16_t m = 0;
    if (rc == p.node_root[u]) m |= (uint16_t)(1u << same);
    if (rc == u) m |= (uint16_t)(1u << other);
    return m;
  };
  // every unit a walk can pop: reachable internal nodes and instance leaves
  std::vector<uint8_t> seen(n_units, 0);
  std::vector<std::pair<uint32_t, uint8_t>> work;  // unit, kind (0 internal top, 1 internal bottom, 2 instance)
  const uint64_t root_off = rd<uint64_t>(blob, rtf::HDR_ROOT_OFFSET);
  if (root_off % 64 == 0 && root_off / 64 < n_units) work.push_back({(uint32_t)(root_off / 64), 0});
  while (!work.empty()) {
    const auto [u, kind] = work.back();
    work.pop_back();
    if (u >= n_units || seen[u] & (1u << kind)) continue;
    seen[u] |= (uint8_t)(1u << kind);
    const uint64_t off = (uint64_t)u * 64;
    if (kind == 2) {
      if (u + 1 >= n_units) continue;
      const uint64_t hdr = off + rd<uint64_t>(blob, off + rtf::IL_BVH_ADDRESS);
      if (hdr % 64 || hdr / 64 >= n_units) continue;
      const uint64_t broot = hdr + rd<uint64_t>(blob, hdr + rtf::HDR_ROOT_OFFSET);
      const uint32_t bu = (uint32_t)(broot >> 6);  // the walk's unit of the BLAS root
      out[u] |= bits(u, bu, kRouteInstShift, kRouteInstShift + 1);
      work.push_back({bu & kEntryUnitMask, 1});
      continue;
    }
    // child units as the walk forms them: 32-bit node + offset, then + sizes
    uint32_t c = (uint32_t)((int32_t)u + rd<int32_t>(blob, off + rtf::IN_CHILD_OFFSET));
    for (int i = 0; i < 6; ++i) {
      const uint8_t info = blob[off + rtf::IN_CHILD_INFO + i];
      const uint32_t sz = rtf::child_size_units(info);
      if (sz > 0) {
        out[u] |= bits(u, c, i, kRouteOtherShift + i);
        const bool internal = rtf::child_type(info) == rtf::CT_INTERNAL;
        if (internal) work.push_back({c & kEntryUnitMask, kind});
        else if (kind == 0) work.push_back({c & kEntryUnitMask, 2});
      }
      c += sz;
    }
  }
}

namespace {

// Roles in which the walk can pop a unit.
constexpr uint8_t kTopInternal = 1, kBotInternal = 2, kInstance = 4, kPrim = 8;

// Breadth-first pass over every unit a walk can pop, from the TLAS root: the
// roles each unit is reached in and, optionally, the node it was first
// reached from (kNoTreelet for the root) and its surface-area visit
// probability along that first path.
void reach(const uint8_t* blob, uint64_t n_bytes, std::vector<uint8_t>& role, std::vector<double>* prob,
           std::vector<uint32_t>* parent = nullptr) {
  const uint64_t n_units = n_bytes / 64;
  role.assign(n_units, 0);
  if (prob) prob->assign(n_units, 0.0);
  if (parent) parent->assign(n_units, kNoTreelet);
  std::deque<uint32_t> q;
  uint32_t from = kNoTreelet;
  auto add = [&](uint32_t u, uint8_t r, double pr) {
    u &= kEntryUnitMask;
    if (u >= n_units || (r == kInstance && u + 1 >= n_units) || (role[u] & r)) return;
    if (!role[u]) {
      if (prob) (*prob)[u] = pr;
      if (parent) (*parent)[u] = from;
    }
    role[u] |= r;
    q.push_back(u);
  };
  const uint64_t root_off = rd<uint64_t>(blob, rtf::HDR_ROOT_OFFSET);
  if (root_off % 64 == 0) add((uint32_t)(root_off / 64), kTopInternal, 1.0);
  std::vector<uint8_t> done(n_units, 0);
  while (!q.empty()) {
    const uint32_t u = q.front();
    from = u;
    q.pop_front();
    const uint8_t todo = role[u] & ~done[u];
    done[u] |= todo;
    const double pu = prob ? (*prob)[u] : 0.0;
    const uint64_t off = (uint64_t)u * 64;
    if (todo & kInstance) {
      const uint64_t hdr = off + rd<uint64_t>(blob, off + rtf::IL_BVH_ADDRESS);
      if (hdr % 64 == 0 && hdr / 64 < n_units) {
        const uint64_t broot = hdr + rd<uint64_t>(blob, hdr + rtf::HDR_ROOT_OFFSET);
        add((uint32_t)(broot >> 6), kBotInternal, pu);
      }
    }
    for (uint8_t lvl : {kTopInternal, kBotInternal}) {
      if (!(todo & lvl)) continue;
      const float ox = rd<float>(blob, off + 0), oy = rd<float>(blob, off + 4), oz = rd<float>(blob, off + 8);
      const float sx = rtm::exp2_int((int)(int8_t)blob[off + rtf::IN_EXP + 0] - 8);
      const float sy = rtm::exp2_int((int)(int8_t)blob[off + rtf::IN_EXP + 1] - 8);
      const float sz = rtm::exp2_int((int)(int8_t)blob[off + rtf::IN_EXP + 2] - 8);
      double area[6] = {0, 0, 0, 0, 0, 0};
      double lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300};
      for (int i = 0; i < 6; ++i) {
        if (!rtf::child_size_units(blob[off + rtf::IN_CHILD_INFO + i])) continue;
        const double l[3] = {ox + (double)blob[off + rtf::IN_LO_X + i] * sx, oy + (double)blob[off + rtf::IN_LO_Y + i] * sy,
                             oz + (double)blob[off + rtf::IN_LO_Z + i] * sz};
        const double h[3] = {ox + (double)blob[off + rtf::IN_HI_X + i] * sx, oy + (double)blob[off + rtf::IN_HI_Y + i] * sy,
                             oz + (double)blob[off + rtf::IN_HI_Z + i] * sz};
        const double dx = h[0] - l[0], dy = h[1] - l[1], dz = h[2] - l[2];
        area[i] = dx * dy + dy * dz + dz * dx;
        for (int a = 0; a < 3; ++a) {
          lo[a] = std::min(lo[a], l[a]);
          hi[a] = std::max(hi[a], h[a]);
        }
      }
      const double ux = hi[0] - lo[0], uy = hi[1] - lo[1], uz = hi[2] - lo[2];
      const double total = ux * uy + uy * uz + uz * ux;
      uint32_t c = (uint32_t)((int32_t)u + rd<int32_t>(blob, off + rtf::IN_CHILD_OFFSET));
      for (int i = 0; i < 6; ++i) {
        const uint8_t info = blob[off + rtf::IN_CHILD_INFO + i];
        const uint32_t size = rtf::child_size_units(info);
        if (size > 0) {
          const double pc = total > 0 ? pu * std::min(1.0, std::max(0.0, area[i] / total)) : pu;
          const bool internal = rtf::child_type(info) == rtf::CT_INTERNAL;
          add(c, internal ? lvl : (lvl == kTopInternal ? kInstance : kPrim), pc);
        }
        c += size;
      }
    }
  }
}

template <class T>
void put(std::vector<uint8_t>& b, uint64_t at, T v) {
  std::memcpy(b.data() + at, &v, sizeof(T));
}

}  // namespace

void default_pin_order(const uint8_t* blob, uint64_t n_bytes, std::vector<uint32_t>& order, const Partition& p) {
  std::vector<uint8_t> role;
  std::vector<double> prob;
  reach(blob, n_bytes, role, &prob);
  const uint32_t n = (uint32_t)p.roots.size();
  std::vector<double> score(n);
  for (uint32_t k = 0; k < n; ++k) score[k] = p.roots[k] == 0 ? 2.0 : prob[p.roots[k]];
  order.resize(n);
  for (uint32_t k = 0; k < n; ++k) order[k] = k;
  std::stable_sort(order.begin(), order.end(), [&](uint32_t a, uint32_t b) { return score[a] > score[b]; });
}

void build_pinned(const uint8_t* blob, uint64_t n_bytes, const Partition& p, const std::vector<uint16_t>& route,
                  const std::vector<uint32_t>& order, uint32_t budget, Pinned& out) {
  out = Pinned();
  budget = std::min<uint32_t>(budget, rtp::kMaxBytes) & ~127u;
  if (budget < 256) return;
  const uint64_t n_units = n_bytes / 64;
  std::vector<uint8_t> role;
  std::vector<uint32_t> parent;
  reach(blob, n_bytes, role, nullptr, &parent);
  auto rec_bytes = [&](uint8_t r) -> uint32_t {
    if (r == kTopInternal || r == kBotInternal) return rtp::kInternalBytes;
    if (r == kInstance) return rtp::kInstanceBytes;
    if (r == kPrim) return rtp::kPrimBytes;
    return 0;  // unreached, or reached in two roles: stays in global memory
  };
  // A record is only ever named by the record of its parent (or, for the
  // root, by the launch), so a node is pinned only after its parent is; a
  // treelet's members come in formation (breadth-first) order, so a treelet
  // that does not fit whole leaves its top part pinned.
  std::vector<uint32_t> soff(n_units, 0);
  std::vector<uint32_t> recs;
  std::vector<uint8_t> taken(p.roots.size(), 0);
  uint32_t used = 16;  // soff 0 is no record
  for (uint32_t k : order) {
    if (k >= p.roots.size() || taken[k]) continue;
    taken[k] = 1;
    bool any = false;
    for (uint64_t j = p.member_first[k]; j < p.member_first[k + 1]; ++j) {
      const uint32_t u = p.members[j];
      const uint32_t b = rec_bytes(role[u]);
      if (soff[u] || !b || used + b > budget) continue;
      if (parent[u] != kNoTreelet && !soff[parent[u]]) continue;
      soff[u] = used / 16;
      used += b;
      recs.push_back(u);
      any = true;
    }
    if (any) out.n_treelets++;
    if (budget - used < 64) break;
  }
  if (recs.empty()) return;
  out.bytes.assign((used + 127u) & ~127u, 0);
  out.n_records = (uint32_t)recs.size();
  auto soff_of = [&](uint32_t u) -> uint16_t {
    u &= kEntryUnitMask;
    return (uint16_t)(u < n_units ? soff[u] : 0);
  };
  for (uint32_t u : recs) {
    const uint64_t at = (uint64_t)soff[u] * 16, off = (uint64_t)u * 64;
    const uint8_t r = role[u];
    if (r == kTopInternal || r == kBotInternal) {
      std::memcpy(out.bytes.data() + at, blob + off, 64);
      put<uint16_t>(out.bytes, at + rtp::IN_ROUTE, route[u]);
      put<uint32_t>(out.bytes, at + rtp::IN_UNIT, u);
      uint32_t c = (uint32_t)((int32_t)u + rd<int32_t>(blob, off + rtf::IN_CHILD_OFFSET));
      for (int i = 0; i < 6; ++i) {
        const uint32_t size = rtf::child_size_units(blob[off + rtf::IN_CHILD_INFO + i]);
        if (size) put<uint16_t>(out.bytes, at + rtp::IN_CHILD_SOFF + 2 * i, soff_of(c));
        c += size;
      }
    } else if (r == kInstance) {
      const uint64_t hdr = off + rd<uint64_t>(blob, off + rtf::IL_BVH_ADDRESS);
      const uint64_t broot = hdr + rd<uint64_t>(blob, hdr + rtf::HDR_ROOT_OFFSET);
      const uint32_t bu = (uint32_t)(broot >> 6) & kEntryUnitMask;
      put<uint32_t>(out.bytes, at + rtp::IL_UNIT, u);
      put<uint32_t>(out.bytes, at + rtp::IL_HDR_UNIT, (uint32_t)(hdr >> 6));
      put<uint32_t>(out.bytes, at + rtp::IL_BROOT_UNIT, bu);
      put<uint16_t>(out.bytes, at + rtp::IL_ROUTE, route[u]);
      put<uint16_t>(out.bytes, at + rtp::IL_ROUTE + 2, soff_of(bu));
      for (int k = 0; k < 9; ++k)
        put<float>(out.bytes, at + rtp::IL_W2O + 4 * k, rd<float>(blob, off + rtf::IL_W2O_LINEAR + 4 * k));
      for (int k = 0; k < 3; ++k)
        put<float>(out.bytes, at + rtp::IL_W2O + 36 + 4 * k, rd<float>(blob, off + rtf::IL_W2O_TRANSLATION + 4 * k));
    } else {
      std::memcpy(out.bytes.data() + at, blob + off, 64);
      put<uint32_t>(out.bytes, at, u);
    }
  }
  const uint64_t root_off = rd<uint64_t>(blob, rtf::HDR_ROOT_OFFSET);
  const uint32_t ru = (uint32_t)(root_off >> 6) & kEntryUnitMask;
  if (root_off % 64 == 0 && ru < n_units && role[ru] == kTopInternal) out.root_soff = soff[ru];
}

bool remap_layout(const Partition& p, uint64_t n_units, uint32_t stride, std::vector<uint64_t>& new_addr,
                  std::string* err) {
  new_addr.assign(n_units, ~0ull);
  const uint64_t step = (uint64_t)p.max_bytes + stride;
  for (uint32_t k = 0; k < p.roots.size(); ++k) {
    const uint64_t base = (uint64_t)k * step;
    const uint32_t r = p.roots[k];
    if (new_addr[r] != ~0ull) {
      if (err) *err = "treelet root already placed inside an earlier treelet (the reference asserts here)";
      return false;
    }
    new_addr[r] = base;
    uint64_t next = base + p.root_bytes[k];
    for (uint64_t j = p.member_first[k]; j < p.member_first[k + 1]; ++j) {
      const uint32_t u = p.members[j];
      if (u == r) continue;
      if (new_addr[u] == ~0ull) new_addr[u] = next;
      next += p.member_bytes[j];
    }
  }
  return true;
}

}  // namespace rtt
