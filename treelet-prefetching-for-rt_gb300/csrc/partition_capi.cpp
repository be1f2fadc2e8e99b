// Host-only C ABI of the treelet partition (no device needed).
#include <algorithm>
#include <string>

#include "capi_internal.h"
#include "treelets.h"

struct rt_partition {
  rtt::Partition p;
  uint64_t n_units = 0;
};

extern "C" {

rt_status rt_partition_form(const rt_blob* blob, uint32_t max_treelet_bytes, rt_partition** out,
                            rt_treelet_info* info) {
  if (!blob || !out) return rti::fail(RT_ERR_INVALID, "rt_partition_form: NULL argument");
  *out = nullptr;
  std::string err;
  if (!rti::validate_blob(blob->bytes.data(), blob->bytes.size(), &err)) return rti::fail(RT_ERR_BLOB, err);
  auto* r = new rt_partition();
  if (!rtt::form_treelets(blob->bytes.data(), blob->bytes.size(), max_treelet_bytes, r->p, &err)) {
    delete r;
    return rti::fail(RT_ERR_INVALID, "rt_partition_form: " + err);
  }
  r->n_units = blob->bytes.size() / 64;
  if (info) {
    info->n_treelets = (uint32_t)r->p.roots.size();
    info->max_treelet_bytes = max_treelet_bytes;
    info->member_entries = r->p.members.size();
    info->image_bytes = r->p.image_bytes;
    info->largest_image = r->p.largest_image;
    info->reserved = 0;
  }
  *out = r;
  return RT_OK;
}

rt_status rt_partition_get(const rt_partition* r, uint32_t* roots, uint64_t* member_first, uint32_t* members,
                           uint16_t* member_bytes, uint32_t* node_root) {
  if (!r) return rti::fail(RT_ERR_INVALID, "rt_partition_get: NULL");
  const rtt::Partition& p = r->p;
  if (roots) std::copy(p.roots.begin(), p.roots.end(), roots);
  if (member_first) std::copy(p.member_first.begin(), p.member_first.end(), member_first);
  if (members) std::copy(p.members.begin(), p.members.end(), members);
  if (member_bytes) std::copy(p.member_bytes.begin(), p.member_bytes.end(), member_bytes);
  if (node_root) std::copy(p.node_root.begin(), p.node_root.end(), node_root);
  return RT_OK;
}

rt_status rt_partition_remap(const rt_partition* r, uint32_t stride, uint64_t* new_addr) {
  if (!r || !new_addr) return rti::fail(RT_ERR_INVALID, "rt_partition_remap: NULL");
  std::vector<uint64_t> m;
  std::string err;
  if (!rtt::remap_layout(r->p, r->n_units, stride, m, &err)) return rti::fail(RT_ERR_STATE, err);
  std::copy(m.begin(), m.end(), new_addr);
  return RT_OK;
}

void rt_partition_free(rt_partition* r) { delete r; }

rt_status rt_partition_route(const rt_partition* r, const rt_blob* blob, uint16_t* route) {
  if (!r || !blob || !route) return rti::fail(RT_ERR_INVALID, "rt_partition_route: NULL");
  if (blob->bytes.size() / 64 != r->n_units) return rti::fail(RT_ERR_INVALID, "rt_partition_route: blob size differs");
  std::vector<uint16_t> m;
  rtt::route_masks(blob->bytes.data(), blob->bytes.size(), r->p, m);
  std::copy(m.begin(), m.end(), route);
  return RT_OK;
}

rt_status rt_partition_pinned(const rt_partition* r, const rt_blob* blob, const uint32_t* order, uint32_t n_order,
                              uint32_t budget, void* out, uint64_t* n_bytes, uint32_t* root_soff) {
  if (!r || !blob || !n_bytes) return rti::fail(RT_ERR_INVALID, "rt_partition_pinned: NULL");
  if (blob->bytes.size() / 64 != r->n_units) return rti::fail(RT_ERR_INVALID, "rt_partition_pinned: blob size differs");
  const uint8_t* b = blob->bytes.data();
  std::vector<uint16_t> route;
  rtt::route_masks(b, blob->bytes.size(), r->p, route);
  std::vector<uint32_t> ord;
  if (order) ord.assign(order, order + n_order);
  else rtt::default_pin_order(b, blob->bytes.size(), ord, r->p);
  rtt::Pinned pin;
  rtt::build_pinned(b, blob->bytes.size(), r->p, route, ord, budget, pin);
  if (out) {
    if (*n_bytes < pin.bytes.size()) return rti::fail(RT_ERR_INVALID, "rt_partition_pinned: output too small");
    std::copy(pin.bytes.begin(), pin.bytes.end(), static_cast<uint8_t*>(out));
  }
  *n_bytes = pin.bytes.size();
  if (root_soff) *root_soff = pin.root_soff;
  return RT_OK;
}

}  // extern "C"
