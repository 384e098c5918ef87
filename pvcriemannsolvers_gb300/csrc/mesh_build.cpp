// Mesh ingest on the host: face connectivity from cell-node lists and the
// space-filling-curve cell order.
//
//   mcfd_build_faces   the faces of Part::BuildLocalFaces / BuildBoundaryFaces
//                      (mesh/part.hpp:932-1019, 1456-1545) from the cells
//                      alone: every (cell, local face) slot is keyed by its
//                      sorted node ids (hex faces in CGNS order, tet faces in
//                      Tetrahedron4::faces_ order), the slots are sorted by
//                      key, and equal keys pair into interior faces whose
//                      holder is the lower cell id (the shuffler writes each
//                      adjacency as [i_cell_small, i_cell_large],
//                      mesh/shuffler.hpp:399-421, so the normal points from
//                      the lower to the higher id).  Lone slots are boundary
//                      faces, grouped by the caller's boundary elements;
//                      periodic group pairs are matched by translating face
//                      centroids.
//   mcfd_hilbert_order the cells' order along a 3D Hilbert curve of their
//                      centroids (Skilling, "Programming the Hilbert curve",
//                      AIP Conf. Proc. 707, 2004: axes-to-transpose, then bit
//                      interleaving), so that cells close in space are close
//                      in memory and the face kernels' neighbour gathers
//                      coalesce.  It takes the place of the reference's METIS
//                      renumbering (mesh/shuffler.hpp) on one GPU.
#include <algorithm>
#include <climits>
#include <array>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <numeric>
#include <string>
#include <unordered_map>
#include <vector>

#include "../../include/mcfd.h"
#include "geometry.hpp"
#include "mesh_build_gpu.hpp"

namespace {

thread_local std::string g_build_error;

int build_fail(const std::string &msg) {
  g_build_error = msg;
  return MCFD_ERR_MESH;
}

using Key = std::array<int64_t, 4>;  // sorted face node ids, -1 first for triangles

Key make_key(const int64_t *ids, int n) {
  Key k{-1, -1, -1, -1};
  for (int i = 0; i < n; ++i) k[4 - n + i] = ids[i];
  std::sort(k.begin(), k.end());
  return k;
}

struct Slot {
  Key key;
  int64_t cell;
  int32_t side;
};

struct OutFace {
  int64_t holder, sharer;
  int32_t hside, sside, group;
  double shift[3];
};

int type_of(const int32_t *cell_type, int64_t c) { return cell_type ? cell_type[c] : MCFD_HEX8; }

int type_nodes(int t) { return mcfd::geo::node_count(t); }

// local faces of cell c (6 hexahedron, 4 tetrahedron, 5 wedge or pyramid)
int n_sides(const int32_t *cell_type, int64_t c) { return mcfd::geo::face_count(type_of(cell_type, c)); }

// corner ids of a local face (faces are keyed and matched by their corners)
int face_node_ids(const int64_t *cell_nodes, int64_t stride, const int32_t *cell_type, int64_t c,
                  int side, int64_t *ids) {
  int v[4];
  const int n = mcfd::geo::cell_face_corners(type_of(cell_type, c), side, v);
  for (int i = 0; i < n; ++i) ids[i] = cell_nodes[c * stride + v[i]];
  return n;
}

// Skilling's transpose form of the Hilbert index for 3 axes of b bits.
uint64_t hilbert_key(uint32_t x, uint32_t y, uint32_t z, int b) {
  uint32_t X[3] = {x, y, z};
  const uint32_t M = 1u << (b - 1);
  for (uint32_t Q = M; Q > 1; Q >>= 1) {
    const uint32_t P = Q - 1;
    for (int i = 0; i < 3; ++i) {
      if (X[i] & Q) {
        X[0] ^= P;
      } else {
        const uint32_t t = (X[0] ^ X[i]) & P;
        X[0] ^= t;
        X[i] ^= t;
      }
    }
  }
  for (int i = 1; i < 3; ++i) X[i] ^= X[i - 1];
  uint32_t t = 0;
  for (uint32_t Q = M; Q > 1; Q >>= 1)
    if (X[2] & Q) t ^= Q - 1;
  for (int i = 0; i < 3; ++i) X[i] ^= t;
  uint64_t key = 0;
  for (int bit = b - 1; bit >= 0; --bit)
    for (int i = 0; i < 3; ++i) key = (key << 1) | ((X[i] >> bit) & 1u);
  return key;
}

int finish_faces(int64_t n_nodes, const double *xyz, const int64_t *cell_nodes, int64_t stride,
                 const int32_t *cell_type, int64_t n_bfaces, const int64_t *bface_nodes,
                 const int32_t *bface_group, int32_t n_periodic, const int32_t *periodic_groups,
                 const double *periodic_shift, std::vector<OutFace> &inner, const std::vector<Slot> &lone,
                 int64_t *face_cells, int32_t *face_sides, int32_t *face_group, double *face_shift,
                 int64_t *n_faces);

}  // namespace

extern "C" {

const char *mcfd_build_error(void) { return g_build_error.c_str(); }

int64_t mcfd_face_slot_count(int64_t n_cells, const int32_t *cell_type) {
  if (n_cells < 0) return -1;
  int64_t n = 0;
  for (int64_t c = 0; c < n_cells; ++c) n += n_sides(cell_type, c);
  return n;
}

int mcfd_build_faces(int64_t n_nodes, const double *xyz, int64_t n_cells,
                     const int64_t *cell_nodes, const int32_t *cell_type,
                     int32_t cell_node_stride, int64_t n_bfaces,
                     const int64_t *bface_nodes, const int32_t *bface_group, int32_t n_periodic,
                     const int32_t *periodic_groups, const double *periodic_shift, int64_t cap,
                     int64_t *face_cells, int32_t *face_sides, int32_t *face_group,
                     double *face_shift, int64_t *n_faces) {
  g_build_error.clear();
  const int64_t stride = cell_node_stride > 0 ? cell_node_stride : 8;
  if (n_nodes <= 0 || !xyz || n_cells <= 0 || !cell_nodes || n_bfaces < 0 ||
      (n_bfaces > 0 && (!bface_nodes || !bface_group)) || n_periodic < 0 ||
      (n_periodic > 0 && (!periodic_groups || !periodic_shift)) || !face_cells || !face_sides ||
      !face_group || !face_shift || !n_faces) {
    g_build_error = "null or negative argument";
    return MCFD_ERR_ARGUMENT;
  }
  // every (cell, local face) slot keyed by its sorted node ids
  std::vector<Slot> slots;
  slots.reserve(mcfd_face_slot_count(n_cells, cell_type));
  for (int64_t c = 0; c < n_cells; ++c) {
    const int nv = type_nodes(cell_type ? cell_type[c] : MCFD_HEX8);
    if (nv == 0) return build_fail("cell " + std::to_string(c) + ": unknown cell type");
    if (nv > stride) return build_fail("cell " + std::to_string(c) + ": more nodes than cell_node_stride");
    for (int v = 0; v < nv; ++v) {
      const int64_t id = cell_nodes[c * stride + v];
      if (id < 0 || id >= n_nodes) return build_fail("cell " + std::to_string(c) + ": node index out of range");
    }
    for (int s = 0; s < n_sides(cell_type, c); ++s) {
      int64_t ids[4];
      const int n = face_node_ids(cell_nodes, stride, cell_type, c, s, ids);
      slots.push_back({make_key(ids, n), c, s});
    }
  }
  if (cap < (int64_t)slots.size()) {
    g_build_error = "output capacity below the face slot count (mcfd_face_slot_count)";
    return MCFD_ERR_ARGUMENT;
  }
  std::sort(slots.begin(), slots.end(), [](const Slot &a, const Slot &b) {
    return a.key != b.key ? a.key < b.key : (a.cell != b.cell ? a.cell < b.cell : a.side < b.side);
  });
  std::vector<OutFace> inner;
  std::vector<int64_t> lone;  // indices into slots
  for (size_t i = 0; i < slots.size();) {
    size_t j = i + 1;
    while (j < slots.size() && slots[j].key == slots[i].key) ++j;
    if (j - i > 2) return build_fail("a face is shared by more than two cells (cell " +
                                     std::to_string(slots[i].cell) + ")");
    if (j - i == 2) {
      const Slot &a = slots[i], &b = slots[i + 1];  // a.cell <= b.cell by the sort
      if (a.cell == b.cell) return build_fail("cell " + std::to_string(a.cell) + " repeats a face");
      inner.push_back({a.cell, b.cell, a.side, b.side, -1, {0, 0, 0}});
    } else {
      lone.push_back((int64_t)i);
    }
    i = j;
  }
  std::vector<Slot> lone_slots;
  lone_slots.reserve(lone.size());
  for (int64_t i : lone) lone_slots.push_back(slots[i]);
  return finish_faces(n_nodes, xyz, cell_nodes, stride, cell_type, n_bfaces, bface_nodes, bface_group,
                      n_periodic, periodic_groups, periodic_shift, inner, lone_slots, face_cells,
                      face_sides, face_group, face_shift, n_faces);
}

}  // extern "C"

namespace {

// Boundary groups, periodic pairs, order and output of the faces, given the
// interior pairs and the free slots (sorted by key): shared by the host and
// the GPU builder.
int finish_faces(int64_t n_nodes, const double *xyz, const int64_t *cell_nodes, int64_t stride,
                 const int32_t *cell_type, int64_t n_bfaces, const int64_t *bface_nodes,
                 const int32_t *bface_group, int32_t n_periodic, const int32_t *periodic_groups,
                 const double *periodic_shift, std::vector<OutFace> &inner, const std::vector<Slot> &lone,
                 int64_t *face_cells, int32_t *face_sides, int32_t *face_group, double *face_shift,
                 int64_t *n_faces) {
  // boundary elements -> groups of the lone slots
  std::vector<int32_t> lone_group(lone.size(), -1);
  for (int64_t f = 0; f < n_bfaces; ++f) {
    const int n = bface_nodes[f * 4 + 3] < 0 ? 3 : 4;
    for (int v = 0; v < n; ++v)
      if (bface_nodes[f * 4 + v] < 0 || bface_nodes[f * 4 + v] >= n_nodes)
        return build_fail("boundary face " + std::to_string(f) + ": node index out of range");
    const Key k = make_key(bface_nodes + f * 4, n);
    auto it = std::lower_bound(lone.begin(), lone.end(), k,
                               [&](const Slot &sl, const Key &key) { return sl.key < key; });
    if (it == lone.end() || it->key != k)
      return build_fail("boundary face " + std::to_string(f) + " is not a free face of any cell");
    lone_group[it - lone.begin()] = bface_group[f];
  }
  // periodic pairs: group a faces matched with group b faces translated by the shift
  std::vector<char> used(lone.size(), 0);
  auto centroid = [&](int64_t li, double *x) {
    const Slot &s = lone[li];
    int64_t ids[4];
    const int n = face_node_ids(cell_nodes, stride, cell_type, s.cell, s.side, ids);
    x[0] = x[1] = x[2] = 0;
    for (int v = 0; v < n; ++v)
      for (int e = 0; e < 3; ++e) x[e] += xyz[ids[v] * 3 + e] / n;
    double h = 0;  // face size: the longest distance from the centroid to a node
    for (int v = 0; v < n; ++v) {
      double d2 = 0;
      for (int e = 0; e < 3; ++e) d2 += (xyz[ids[v] * 3 + e] - x[e]) * (xyz[ids[v] * 3 + e] - x[e]);
      h = std::max(h, std::sqrt(d2));
    }
    return h;
  };
  for (int32_t p = 0; p < n_periodic; ++p) {
    const int32_t ga = periodic_groups[2 * p], gb = periodic_groups[2 * p + 1];
    const double *sh = periodic_shift + 3 * p;
    std::vector<int64_t> fa, fb;
    double hmin = 1e300;
    for (size_t i = 0; i < lone.size(); ++i) {
      if (used[i]) continue;
      if (lone_group[i] == ga) fa.push_back((int64_t)i);
      else if (lone_group[i] == gb) fb.push_back((int64_t)i);
    }
    if (fa.size() != fb.size())
      return build_fail("periodic groups " + std::to_string(ga) + " / " + std::to_string(gb) +
                        " have different face counts");
    std::vector<std::array<double, 3>> ca(fa.size());
    for (size_t i = 0; i < fa.size(); ++i) hmin = std::min(hmin, centroid(fa[i], ca[i].data()));
    const double tol = 1e-6 * hmin, cell = 4 * tol;
    auto qkey = [&](const double *x, int dx, int dy, int dz) {
      const int64_t qx = (int64_t)std::floor(x[0] / cell) + dx, qy = (int64_t)std::floor(x[1] / cell) + dy,
                    qz = (int64_t)std::floor(x[2] / cell) + dz;
      return (uint64_t)(qx * 73856093) ^ (uint64_t)(qy * 19349663) ^ (uint64_t)(qz * 83492791);
    };
    std::unordered_multimap<uint64_t, size_t> grid;
    grid.reserve(fa.size() * 2);
    for (size_t i = 0; i < fa.size(); ++i) grid.emplace(qkey(ca[i].data(), 0, 0, 0), i);
    std::vector<char> taken(fa.size(), 0);
    for (size_t j = 0; j < fb.size(); ++j) {
      double x[3];
      centroid(fb[j], x);
      for (int e = 0; e < 3; ++e) x[e] += sh[e];
      size_t match = (size_t)-1;
      for (int dx = -1; dx <= 1 && match == (size_t)-1; ++dx)
        for (int dy = -1; dy <= 1 && match == (size_t)-1; ++dy)
          for (int dz = -1; dz <= 1 && match == (size_t)-1; ++dz) {
            auto range = grid.equal_range(qkey(x, dx, dy, dz));
            for (auto it = range.first; it != range.second; ++it) {
              const auto &c = ca[it->second];
              if (!taken[it->second] && std::fabs(c[0] - x[0]) <= tol && std::fabs(c[1] - x[1]) <= tol &&
                  std::fabs(c[2] - x[2]) <= tol) {
                match = it->second;
                break;
              }
            }
          }
      if (match == (size_t)-1)
        return build_fail("periodic group " + std::to_string(gb) + ": a face has no partner in group " +
                          std::to_string(ga));
      taken[match] = 1;
      const Slot &sa = lone[fa[match]], &sb = lone[fb[j]];
      used[fa[match]] = used[fb[j]] = 1;
      // x(sharer) + shift = x(holder); the holder is the lower cell id
      OutFace f;
      if (sa.cell <= sb.cell) {
        f = {sa.cell, sb.cell, sa.side, sb.side, -1, {sh[0], sh[1], sh[2]}};
      } else {
        f = {sb.cell, sa.cell, sb.side, sa.side, -1, {-sh[0], -sh[1], -sh[2]}};
      }
      if (f.holder == f.sharer) return build_fail("a periodic face pairs a cell with itself");
      inner.push_back(f);
    }
  }
  // order: interior (and periodic) faces by (holder, holder side), then
  // boundary faces by (group, holder, side), faces without a group last
  std::sort(inner.begin(), inner.end(), [](const OutFace &a, const OutFace &b) {
    return a.holder != b.holder ? a.holder < b.holder : a.hside < b.hside;
  });
  std::vector<OutFace> bnd;
  for (size_t i = 0; i < lone.size(); ++i) {
    if (used[i]) continue;
    const Slot &s = lone[i];
    bnd.push_back({s.cell, -1, s.side, -1, lone_group[i], {0, 0, 0}});
  }
  std::sort(bnd.begin(), bnd.end(), [](const OutFace &a, const OutFace &b) {
    const int64_t ga = a.group < 0 ? INT64_MAX : a.group, gb = b.group < 0 ? INT64_MAX : b.group;
    if (ga != gb) return ga < gb;
    return a.holder != b.holder ? a.holder < b.holder : a.hside < b.hside;
  });
  int64_t n = 0;
  for (const auto *list : {&inner, &bnd})
    for (const OutFace &f : *list) {
      face_cells[2 * n] = f.holder;
      face_cells[2 * n + 1] = f.sharer;
      face_sides[2 * n] = f.hside;
      face_sides[2 * n + 1] = f.sside;
      face_group[n] = f.group;
      for (int e = 0; e < 3; ++e) face_shift[3 * n + e] = f.shift[e];
      ++n;
    }
  *n_faces = n;
  return MCFD_OK;
}

}  // namespace

extern "C" {

int mcfd_build_faces_gpu(int32_t device, int64_t n_nodes, const double *xyz, int64_t n_cells,
                         const int64_t *cell_nodes, const int32_t *cell_type,
                         int32_t cell_node_stride, int64_t n_bfaces, const int64_t *bface_nodes,
                         const int32_t *bface_group, int32_t n_periodic,
                         const int32_t *periodic_groups, const double *periodic_shift, int64_t cap,
                         int64_t *face_cells, int32_t *face_sides, int32_t *face_group,
                         double *face_shift, int64_t *n_faces) {
  g_build_error.clear();
  const int64_t stride = cell_node_stride > 0 ? cell_node_stride : 8;
  if (n_nodes <= 0 || !xyz || n_cells <= 0 || !cell_nodes || n_bfaces < 0 ||
      (n_bfaces > 0 && (!bface_nodes || !bface_group)) || n_periodic < 0 ||
      (n_periodic > 0 && (!periodic_groups || !periodic_shift)) || !face_cells || !face_sides ||
      !face_group || !face_shift || !n_faces) {
    g_build_error = "null or negative argument";
    return MCFD_ERR_ARGUMENT;
  }
  if (n_nodes >= (int64_t)UINT32_MAX) {
    g_build_error = "the GPU builder keys faces by 32-bit node ids";
    return MCFD_ERR_UNSUPPORTED;
  }
  std::vector<int64_t> slot_off(n_cells + 1, 0);
  for (int64_t c = 0; c < n_cells; ++c) {
    const int nv = type_nodes(cell_type ? cell_type[c] : MCFD_HEX8);
    if (nv == 0) return build_fail("cell " + std::to_string(c) + ": unknown cell type");
    if (nv > stride) return build_fail("cell " + std::to_string(c) + ": more nodes than cell_node_stride");
    for (int v = 0; v < nv; ++v) {
      const int64_t id = cell_nodes[c * stride + v];
      if (id < 0 || id >= n_nodes) return build_fail("cell " + std::to_string(c) + ": node index out of range");
    }
    slot_off[c + 1] = slot_off[c] + n_sides(cell_type, c);
  }
  if (cap < slot_off.back()) {
    g_build_error = "output capacity below the face slot count (mcfd_face_slot_count)";
    return MCFD_ERR_ARGUMENT;
  }
  if (slot_off.back() >= (int64_t)UINT32_MAX) {
    g_build_error = "more than 2^32 face slots";
    return MCFD_ERR_UNSUPPORTED;
  }
  mcfd::GpuPairs pr;
  std::string err;
  const int rc = mcfd::gpu_pair_slots(device, cell_nodes, stride, cell_type, n_cells, slot_off, &pr, &err);
  if (rc == 2) return build_fail(err);
  if (rc) {
    g_build_error = err;
    return MCFD_ERR_CUDA;
  }
  const int64_t n_inner = (int64_t)pr.inner_sides.size() / 2;
  std::vector<OutFace> inner(n_inner);
  for (int64_t f = 0; f < n_inner; ++f)
    inner[f] = {pr.inner_cells[2 * f], pr.inner_cells[2 * f + 1], pr.inner_sides[2 * f],
                pr.inner_sides[2 * f + 1], -1, {0, 0, 0}};
  std::vector<Slot> lone(pr.lone_cells.size());
  for (size_t i = 0; i < lone.size(); ++i) {
    int64_t ids[4];
    const int n = face_node_ids(cell_nodes, stride, cell_type, pr.lone_cells[i], pr.lone_sides[i], ids);
    lone[i] = {make_key(ids, n), pr.lone_cells[i], pr.lone_sides[i]};
  }
  std::sort(lone.begin(), lone.end(), [](const Slot &a, const Slot &b) {
    return a.key != b.key ? a.key < b.key : (a.cell != b.cell ? a.cell < b.cell : a.side < b.side);
  });
  return finish_faces(n_nodes, xyz, cell_nodes, stride, cell_type, n_bfaces, bface_nodes, bface_group,
                      n_periodic, periodic_groups, periodic_shift, inner, lone, face_cells, face_sides,
                      face_group, face_shift, n_faces);
}

int mcfd_hilbert_order(int64_t n, const double *points, int64_t *order) {
  if (n < 0 || (n > 0 && (!points || !order))) return MCFD_ERR_ARGUMENT;
  if (n == 0) return MCFD_OK;
  double lo[3] = {points[0], points[1], points[2]}, hi[3] = {points[0], points[1], points[2]};
  for (int64_t i = 0; i < n; ++i)
    for (int e = 0; e < 3; ++e) {
      lo[e] = std::min(lo[e], points[i * 3 + e]);
      hi[e] = std::max(hi[e], points[i * 3 + e]);
    }
  double span = 0;
  for (int e = 0; e < 3; ++e) span = std::max(span, hi[e] - lo[e]);
  if (!(span > 0)) span = 1;
  constexpr int kBits = 21;
  const double scale = (double)((1u << kBits) - 1) / span;
  std::vector<std::pair<uint64_t, int64_t>> keys(n);
  for (int64_t i = 0; i < n; ++i) {
    uint32_t q[3];
    for (int e = 0; e < 3; ++e)
      q[e] = (uint32_t)std::min<double>((points[i * 3 + e] - lo[e]) * scale, (double)((1u << kBits) - 1));
    keys[i] = {hilbert_key(q[0], q[1], q[2], kBits), i};
  }
  std::sort(keys.begin(), keys.end());
  for (int64_t i = 0; i < n; ++i) order[i] = keys[i].second;
  return MCFD_OK;
}

}  // extern "C"
