// Mesh ingest: legacy VTK unstructured grids (the reference keeps its input
// meshes as legacy .vtk files next to the gmsh scripts, input/*.vtk, and
// converts them to CGNS; CGNS needs HDF5, so this reader is the ingest path
// here).  ASCII and BINARY (big-endian) files, the classic CELLS layout and
// the OFFSETS / CONNECTIVITY layout of file version 5.  Hexahedra (VTK type
// 12) and tetrahedra (10) become cells (VTK and CGNS share their corner
// order), quadrilaterals (9) and triangles (5) boundary elements; vertices,
// lines and other types are skipped.  Boundary groups come from an integer
// (or integral-valued) CELL_DATA array, SCALARS or FIELD, by name or the first
// one.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <fstream>
#include <sstream>
#include <string>
#include <vector>

#include "geometry.hpp"

#include "../../include/mcfd.h"

struct mcfd_vtk_mesh {
  std::vector<double> xyz;
  std::vector<int64_t> cell_nodes;  // [cells][stride]
  std::vector<int32_t> cell_type;   // enum mcfd_cell_type
  int32_t stride = 8;               // slots per cell: 8, or the most nodes of a quadratic cell
  std::vector<int64_t> bface_nodes; // [bfaces][4]
  std::vector<int32_t> bface_group;
};

namespace {

// Quadratic VTK cells in CGNS node order: slot i of the CGNS cell holds VTK
// node vtk[i].  Hexahedra: VTK lists the top mid-edges (12-15) before the
// vertical ones (16-19) and its face centres as -x, +x, -y, +y, -z, +z
// (20-25); CGNS HEXA_20 / HEXA_27 the vertical mid-edges first and the
// centres bottom, -y, +x, +y, -x, top.  Quadratic wedges come in two
// layouts: VTK's own (VTK_QUADRATIC_WEDGE / VTK_BIQUADRATIC_QUADRATIC_WEDGE
// share VTK_WEDGE's corner orientation, so CGNS corners 0, 1, 2, 3, 4, 5 are
// VTK's 0, 2, 1, 3, 5, 4 as for VTK_WEDGE, mesh/vtk.hpp:236-243, with the
// mid-edge and quadrangle-centre slots permuted to match), and the order the
// reference's solution writer emits (mesh/vtk.hpp Wedge15: the CGNS corners
// unflipped, the mid-edges of the bottom and the top triangles, then the
// vertical ones, VTK 32 adding the quadrangle centres in CGNS order).  The
// reader takes the layout in which the cell's corner wedge has a positive
// volume.  Tetrahedra and pyramids: VTK_QUADRATIC_TETRA /
// VTK_QUADRATIC_PYRAMID agree with TETRA_10 / PYRA_13.
struct QuadraticVtk {
  int vtk_type, n, type;
  int vtk[27];
};
const QuadraticVtk kQuadraticVtk[] = {
    {25, 20, MCFD_HEX20, {0, 1, 2, 3, 4, 5, 6, 7, 8, 9, 10, 11, 16, 17, 18, 19, 12, 13, 14, 15}},
    {29, 27, MCFD_HEX27, {0,  1,  2,  3,  4,  5,  6,  7,  8,  9,  10, 11, 16, 17,
                          18, 19, 12, 13, 14, 15, 24, 22, 21, 23, 20, 25, 26}},
    {24, 10, MCFD_TET10, {0, 1, 2, 3, 4, 5, 6, 7, 8, 9}},
    {26, 15, MCFD_WEDGE15, {0, 1, 2, 3, 4, 5, 6, 7, 8, 12, 13, 14, 9, 10, 11}},
    {32, 18, MCFD_WEDGE18, {0, 1, 2, 3, 4, 5, 6, 7, 8, 12, 13, 14, 9, 10, 11, 15, 16, 17}},
    {27, 13, MCFD_PYRA13, {0, 1, 2, 3, 4, 5, 6, 7, 8, 9, 10, 11, 12}},
};
// VTK's own quadratic wedge layouts (corners flipped as VTK_WEDGE).
const QuadraticVtk kVtkWedge[] = {
    {26, 15, MCFD_WEDGE15, {0, 2, 1, 3, 5, 4, 8, 7, 6, 12, 14, 13, 11, 10, 9}},
    {32, 18, MCFD_WEDGE18, {0, 2, 1, 3, 5, 4, 8, 7, 6, 12, 14, 13, 11, 10, 9, 17, 16, 15}},
};
const QuadraticVtk *quadratic_vtk(int vtk_type, int64_t k) {
  for (const auto &q : kQuadraticVtk)
    if (q.vtk_type == vtk_type && q.n == k) return &q;
  return nullptr;
}

thread_local std::string g_vtk_error;

class Reader {
 public:
  explicit Reader(const std::string &path) : in_(path, std::ios::in | std::ios::binary) {}
  bool ok() const { return (bool)in_; }
  bool binary = false;

  // next whitespace-separated token (skips blank lines); the whitespace
  // after it stays in the stream, so line() then takes the rest of the line
  bool token(std::string *t) {
    t->clear();
    while (in_.peek() != EOF && std::isspace(in_.peek())) in_.get();
    while (in_.peek() != EOF && !std::isspace(in_.peek())) t->push_back((char)in_.get());
    return !t->empty();
  }
  bool line(std::string *l) { return (bool)std::getline(in_, *l); }

  // n values of the declared VTK type into doubles / int64
  template <class T>
  bool values(int64_t n, const std::string &type, std::vector<T> *out) {
    out->resize(n);
    if (!binary) {
      std::string t;
      for (int64_t i = 0; i < n; ++i) {
        if (!token(&t)) return false;
        (*out)[i] = (T)std::strtod(t.c_str(), nullptr);
      }
      return true;
    }
    // binary: skip the single newline after the header line, big-endian data
    int size = 0;
    bool real = false;
    if (type == "float") size = 4, real = true;
    else if (type == "double") size = 8, real = true;
    else if (type == "int" || type == "unsigned_int" || type == "vtktypeint32") size = 4;
    else if (type == "long" || type == "unsigned_long" || type == "vtktypeint64") size = 8;
    else if (type == "short" || type == "unsigned_short") size = 2;
    else if (type == "char" || type == "unsigned_char") size = 1;
    else return false;
    std::vector<unsigned char> raw((size_t)n * size);
    if (n > 0 && !in_.read(reinterpret_cast<char *>(raw.data()), (std::streamsize)raw.size())) return false;
    for (int64_t i = 0; i < n; ++i) {
      uint64_t v = 0;
      for (int b = 0; b < size; ++b) v = (v << 8) | raw[(size_t)i * size + b];
      if (real && size == 4) {
        float f;
        const uint32_t w = (uint32_t)v;
        std::memcpy(&f, &w, 4);
        (*out)[i] = (T)f;
      } else if (real) {
        double d;
        std::memcpy(&d, &v, 8);
        (*out)[i] = (T)d;
      } else {
        const bool is_signed = type.rfind("unsigned", 0) != 0 && type != "unsigned_char";
        int64_t s = (int64_t)v;
        if (is_signed && size < 8 && (v >> (8 * size - 1)) & 1) s = (int64_t)(v | (~0ull << (8 * size)));
        (*out)[i] = (T)s;
      }
    }
    return true;
  }
  // binary data blocks end at the next newline
  void after_binary() {
    if (binary) {
      std::string rest;
      std::getline(in_, rest);
    }
  }

 private:
  std::ifstream in_;
};

int vtk_fail(const std::string &msg) {
  g_vtk_error = msg;
  return MCFD_ERR_IO;
}

}  // namespace

extern "C" {

const char *mcfd_vtk_error(void) { return g_vtk_error.c_str(); }

int mcfd_vtk_read(const char *path, const char *group_array, mcfd_vtk_mesh **out) {
  g_vtk_error.clear();
  if (!path || !out) return MCFD_ERR_ARGUMENT;
  *out = nullptr;
  Reader r(path);
  if (!r.ok()) return vtk_fail(std::string("cannot open ") + path);
  std::string l;
  if (!r.line(&l) || l.rfind("# vtk DataFile", 0) != 0) return vtk_fail("not a legacy VTK file");
  r.line(&l);  // title
  if (!r.line(&l)) return vtk_fail("truncated header");
  while (!l.empty() && std::isspace((unsigned char)l.back())) l.pop_back();
  if (l == "BINARY") r.binary = true;
  else if (l != "ASCII") return vtk_fail("expected ASCII or BINARY");
  std::string t, type;
  if (!r.token(&t) || t != "DATASET" || !r.token(&t) || t != "UNSTRUCTURED_GRID")
    return vtk_fail("only DATASET UNSTRUCTURED_GRID is read");
  std::vector<double> xyz;
  std::vector<int64_t> conn, offsets, types;
  std::vector<double> groups;
  int64_t n_points = -1, n_cells = -1, n_attr = -1;
  bool have_groups = false, cell_data = false;
  while (r.token(&t)) {
    if (t == "POINTS") {
      r.token(&t);
      n_points = std::atoll(t.c_str());
      r.token(&type);
      r.line(&l);
      if (!r.values(3 * n_points, type, &xyz)) return vtk_fail("bad POINTS block");
      r.after_binary();
    } else if (t == "CELLS") {
      std::string a, b;
      r.token(&a);
      r.token(&b);
      r.line(&l);
      // classic layout: CELLS n size, then (npts id ...) per cell; version 5:
      // CELLS n_offsets n_conn, then OFFSETS / CONNECTIVITY blocks
      std::string next;
      const int64_t na = std::atoll(a.c_str()), nb = std::atoll(b.c_str());
      std::vector<int64_t> flat;
      // peek: version-5 files put the OFFSETS keyword next
      if (!r.token(&next)) return vtk_fail("truncated CELLS");
      if (next == "OFFSETS") {
        r.token(&type);
        r.line(&l);
        if (!r.values(na, type, &offsets)) return vtk_fail("bad OFFSETS block");
        r.after_binary();
        if (!r.token(&next) || next != "CONNECTIVITY") return vtk_fail("expected CONNECTIVITY");
        r.token(&type);
        r.line(&l);
        if (!r.values(nb, type, &conn)) return vtk_fail("bad CONNECTIVITY block");
        r.after_binary();
        n_cells = na - 1;
        if (n_cells < 0 || offsets.front() != 0 || offsets.back() != nb) return vtk_fail("bad OFFSETS");
        for (int64_t c = 0; c < n_cells; ++c)
          if (offsets[c + 1] < offsets[c]) return vtk_fail("bad OFFSETS");
      } else {
        n_cells = na;
        if (r.binary) return vtk_fail("binary classic CELLS layout: write file version 5 (OFFSETS)");
        if (na < 0 || nb < 1) return vtk_fail("bad CELLS header");
        flat.resize(nb);
        flat[0] = std::atoll(next.c_str());
        for (int64_t i = 1; i < nb; ++i) {
          if (!r.token(&t)) return vtk_fail("truncated CELLS");
          flat[i] = std::atoll(t.c_str());
        }
        offsets.assign(1, 0);
        for (int64_t i = 0, c = 0; c < n_cells; ++c) {
          const int64_t k = flat[i];
          if (k < 0 || i + 1 + k > nb) return vtk_fail("bad CELLS entry");
          conn.insert(conn.end(), flat.begin() + i + 1, flat.begin() + i + 1 + k);
          offsets.push_back((int64_t)conn.size());
          i += 1 + k;
        }
      }
    } else if (t == "CELL_TYPES") {
      r.token(&t);
      const int64_t n = std::atoll(t.c_str());
      r.line(&l);
      if (!r.values(n, "int", &types)) return vtk_fail("bad CELL_TYPES block");
      r.after_binary();
    } else if (t == "CELL_DATA" || t == "POINT_DATA") {
      cell_data = t == "CELL_DATA";
      r.token(&t);
      n_attr = std::atoll(t.c_str());
    } else if (t == "SCALARS" && n_attr >= 0) {
      std::string name;
      r.token(&name);
      r.token(&type);
      r.line(&l);  // optional component count
      const int nc = std::max(1, std::atoi(l.c_str()));
      r.token(&t);  // LOOKUP_TABLE
      r.token(&t);  // its name
      r.line(&l);
      std::vector<double> v;
      if (!r.values(n_attr * nc, type, &v)) return vtk_fail("bad SCALARS block");
      r.after_binary();
      if (cell_data && !have_groups && nc == 1 && (!group_array || name == group_array)) {
        groups = v;
        have_groups = true;
      }
    } else if (t == "FIELD" && n_attr >= 0) {
      r.token(&t);  // field name
      r.token(&t);
      const int n_arrays = std::atoi(t.c_str());
      r.line(&l);
      for (int a = 0; a < n_arrays; ++a) {
        std::string name, snc, snt;
        r.token(&name);
        r.token(&snc);
        r.token(&snt);
        r.token(&type);
        r.line(&l);
        const int64_t nc = std::atoll(snc.c_str()), nt = std::atoll(snt.c_str());
        std::vector<double> v;
        if (!r.values(nc * nt, type, &v)) return vtk_fail("bad FIELD array");
        r.after_binary();
        if (cell_data && !have_groups && nc == 1 && nt == n_attr && (!group_array || name == group_array)) {
          groups = v;
          have_groups = true;
        }
      }
    } else if ((t == "VECTORS" || t == "NORMALS" || t == "TENSORS") && n_attr >= 0) {
      std::string name;
      r.token(&name);
      r.token(&type);
      r.line(&l);
      std::vector<double> v;
      if (!r.values(n_attr * (t == "TENSORS" ? 9 : 3), type, &v)) return vtk_fail("bad attribute block");
      r.after_binary();
    } else if (t == "METADATA") {
      // skip until a blank line
      while (r.line(&l) && !l.empty()) {}
    } else {
      return vtk_fail("unexpected keyword " + t);
    }
  }
  if (n_points < 0 || n_cells < 0 || (int64_t)types.size() != n_cells ||
      (int64_t)offsets.size() != n_cells + 1)
    return vtk_fail("POINTS, CELLS and CELL_TYPES are required and must agree");
  if (have_groups && (int64_t)groups.size() != n_cells) return vtk_fail("CELL_DATA size mismatch");
  auto *m = new mcfd_vtk_mesh();
  m->xyz = std::move(xyz);
  for (int64_t c = 0; c < n_cells; ++c) {
    const int64_t b = offsets[c], k = offsets[c + 1] - b;
    auto node = [&](int i) { return conn[b + i]; };
    for (int64_t i = 0; i < k; ++i)
      if (node((int)i) < 0 || node((int)i) >= n_points) {
        delete m;
        return vtk_fail("cell " + std::to_string(c) + ": node index out of range");
      }
    const int vt = (int)types[c];
    const QuadraticVtk *qv = quadratic_vtk(vt, k);
    if (qv && (qv->type == MCFD_WEDGE15 || qv->type == MCFD_WEDGE18)) {
      // VTK's layout when its flipped corners give a positive corner wedge
      // ((x1 - x0) x (x2 - x0) . (x3 - x0) > 0 in CGNS order), else the
      // reference writer's
      const QuadraticVtk *vq = &kVtkWedge[qv->type == MCFD_WEDGE15 ? 0 : 1];
      const double *x0 = &m->xyz[3 * node(vq->vtk[0])], *x1 = &m->xyz[3 * node(vq->vtk[1])];
      const double *x2 = &m->xyz[3 * node(vq->vtk[2])], *x3 = &m->xyz[3 * node(vq->vtk[3])];
      double a[3], b[3], d[3];
      for (int i = 0; i < 3; ++i) a[i] = x1[i] - x0[i], b[i] = x2[i] - x0[i], d[i] = x3[i] - x0[i];
      const double vol = (a[1] * b[2] - a[2] * b[1]) * d[0] + (a[2] * b[0] - a[0] * b[2]) * d[1] +
                         (a[0] * b[1] - a[1] * b[0]) * d[2];
      if (vol > 0) qv = vq;
    }
    if (qv) {
      // CGNS slot i holds VTK node qv->vtk[i]
      for (int i = 0; i < qv->n; ++i) m->cell_nodes.push_back(node(qv->vtk[i]));
      for (int i = qv->n; i < 8; ++i) m->cell_nodes.push_back(-1);
      m->cell_type.push_back(qv->type);
      m->stride = std::max<int32_t>(m->stride, qv->n);
    } else if ((vt == 12 && k == 8) || (vt == 10 && k == 4) || (vt == 14 && k == 5)) {
      // hexahedron, tetrahedron and pyramid: VTK and CGNS orders agree
      for (int i = 0; i < 8; ++i) m->cell_nodes.push_back(i < k ? node(i) : -1);
      m->cell_type.push_back(vt == 10 ? MCFD_TET4 : vt == 14 ? MCFD_PYRA5 : MCFD_HEX8);
    } else if (vt == 13 && k == 6) {
      // wedge: VTK's 0, 1, 2, 3, 4, 5 are CGNS's 0, 2, 1, 3, 5, 4 (mesh/vtk.hpp:236-243)
      const int perm[6] = {0, 2, 1, 3, 5, 4};
      for (int i = 0; i < 8; ++i) m->cell_nodes.push_back(i < 6 ? node(perm[i]) : -1);
      m->cell_type.push_back(MCFD_WEDGE6);
    } else if ((vt == 9 && k == 4) || (vt == 5 && k == 3) || (vt == 22 && k == 6) ||
               (vt == 23 && k == 8) || (vt == 28 && k == 9)) {
      // boundary elements: quads and triangles, the quadratic ones (VTK 22
      // triangle, 23 / 28 quadrangles) by their corners, which VTK lists first
      const int nc = (vt == 5 || vt == 22) ? 3 : 4;
      for (int i = 0; i < 4; ++i) m->bface_nodes.push_back(i < nc ? node(i) : -1);
      const double g = have_groups ? groups[c] : 0.0;
      m->bface_group.push_back((int32_t)std::lround(g));
    } else if (vt == 1 || vt == 2 || vt == 3 || vt == 4 || vt == 21) {
      // vertices and lines (mesh generators' physical points and curves)
      // bound no volume and no face: skipped
    } else {
      delete m;
      return vtk_fail("cell " + std::to_string(c) + ": unsupported VTK cell type " + std::to_string(vt) +
                      " with " + std::to_string(k) + " nodes");
    }
  }
  if (m->stride > 8) {  // re-lay the cells at the widest cell's stride
    std::vector<int64_t> wide;
    wide.reserve(m->cell_type.size() * m->stride);
    size_t at = 0;
    for (int32_t t : m->cell_type) {
      const int n = std::max(8, mcfd::geo::node_count(t));
      for (int i = 0; i < m->stride; ++i) wide.push_back(i < n ? m->cell_nodes[at + i] : -1);
      at += n;
    }
    m->cell_nodes.swap(wide);
  }
  *out = m;
  return MCFD_OK;
}

int mcfd_vtk_mesh_stride(const mcfd_vtk_mesh *m, int32_t *stride) {
  if (!m || !stride) return MCFD_ERR_ARGUMENT;
  *stride = m->stride;
  return MCFD_OK;
}

int mcfd_vtk_mesh_sizes(const mcfd_vtk_mesh *m, int64_t *n_nodes, int64_t *n_cells,
                        int64_t *n_bfaces) {
  if (!m || !n_nodes || !n_cells || !n_bfaces) return MCFD_ERR_ARGUMENT;
  *n_nodes = (int64_t)m->xyz.size() / 3;
  *n_cells = (int64_t)m->cell_type.size();
  *n_bfaces = (int64_t)m->bface_group.size();
  return MCFD_OK;
}

int mcfd_vtk_mesh_arrays(const mcfd_vtk_mesh *m, double *xyz, int64_t *cell_nodes,
                         int32_t *cell_type, int64_t *bface_nodes, int32_t *bface_group) {
  if (!m || !xyz || !cell_nodes || !cell_type || (!m->bface_group.empty() && (!bface_nodes || !bface_group)))
    return MCFD_ERR_ARGUMENT;
  std::copy(m->xyz.begin(), m->xyz.end(), xyz);
  std::copy(m->cell_nodes.begin(), m->cell_nodes.end(), cell_nodes);
  std::copy(m->cell_type.begin(), m->cell_type.end(), cell_type);
  std::copy(m->bface_nodes.begin(), m->bface_nodes.end(), bface_nodes);
  std::copy(m->bface_group.begin(), m->bface_group.end(), bface_group);
  return MCFD_OK;
}

void mcfd_vtk_mesh_destroy(mcfd_vtk_mesh *m) { delete m; }

}  // extern "C"
