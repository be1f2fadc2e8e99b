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
