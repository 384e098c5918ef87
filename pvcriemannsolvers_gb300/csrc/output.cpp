// Solution output and restart (host side of output.cu).
//
//   mcfd_vtk_sample / mcfd_write_vtu    Writer<Part>::Prepare + WriteSolutions
//                                       (mesh/vtk.hpp:428-669): every cell is
//                                       written as a disconnected quadratic
//                                       element (Hex8 -> VTK Hexahedron27,
//                                       Tet4 -> VTK Tetrahedron10) carrying
//                                       the conservative variables at its VTK
//                                       nodes; a .pvtu index plus one .vtu
//                                       piece, in the reference's layout
//                                       (values ASCII, points base64 with a
//                                       separately encoded UInt64 byte count).
//   mcfd_gather_fields / _scatter_      Part::GatherSolutions / Scatter-
//                                       Solutions (mesh/part.hpp:380-395,
//                                       1053-1069): field i of cell c is value
//                                       i of the cell's column block.
//   mcfd_write_restart / _read_restart  Part::WriteSolutions / ReadSolutions
//                                       (mesh/part.hpp:1070-1208) with a
//                                       binary file of the DataOnCells fields
//                                       in place of CGNS (no HDF5 here).
#include <cuda_runtime.h>
#include <sys/stat.h>

#include <cerrno>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <sstream>
#include <string>
#include <vector>

#include "../../include/mcfd.h"
#include "geometry.hpp"
#include "handle.hpp"

namespace {

const char *const kFieldNames[5] = {"Density", "MomentumX", "MomentumY", "MomentumZ",
                                    "EnergyStagnationDensity"};
constexpr int kVtkHex27Type = 29, kVtkTet10Type = 24, kVtkWedge15Type = 26;
constexpr int kK5 = 5;  // conservative variables

int fail(mcfd_handle *h, int code, const std::string &msg) {
  if (h) h->err = msg;
  return code;
}

int cuda_fail(mcfd_handle *h, cudaError_t e, const char *what) {
  return fail(h, MCFD_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

#define OUT_TRY(h, call)                                   \
  do {                                                     \
    cudaError_t e_ = (call);                               \
    if (e_ != cudaSuccess) return cuda_fail(h, e_, #call); \
  } while (0)

// RFC 4648 base64 with '=' padding.
const char kBase64[] = "ABCDEFGHIJKLMNOPQRSTUVWXYZabcdefghijklmnopqrstuvwxyz0123456789+/";

std::string base64(const unsigned char *p, size_t n) {
  std::string out;
  out.reserve((n + 2) / 3 * 4);
  size_t i = 0;
  for (; i + 3 <= n; i += 3) {
    const unsigned v = (unsigned)p[i] << 16 | (unsigned)p[i + 1] << 8 | p[i + 2];
    out.push_back(kBase64[v >> 18]);
    out.push_back(kBase64[(v >> 12) & 63]);
    out.push_back(kBase64[(v >> 6) & 63]);
    out.push_back(kBase64[v & 63]);
  }
  if (i < n) {
    const unsigned v = (unsigned)p[i] << 16 | (i + 1 < n ? (unsigned)p[i + 1] << 8 : 0u);
    out.push_back(kBase64[v >> 18]);
    out.push_back(kBase64[(v >> 12) & 63]);
    out.push_back(i + 1 < n ? kBase64[(v >> 6) & 63] : '=');
    out.push_back('=');
  }
  return out;
}

// VTK inline binary: base64(UInt64 byte count) followed by base64(bytes).
std::string vtk_binary(const void *data, size_t bytes) {
  const uint64_t n = bytes;
  return base64(reinterpret_cast<const unsigned char *>(&n), sizeof(n)) +
         base64(reinterpret_cast<const unsigned char *>(data), bytes);
}

bool little_endian() {
  const uint16_t one = 1;
  unsigned char b;
  std::memcpy(&b, &one, 1);
  return b == 1;
}

// mkdir -p
bool make_dirs(const std::string &path) {
  std::string cur;
  size_t i = 0;
  while (i <= path.size()) {
    const size_t j = path.find('/', i);
    cur = path.substr(0, j == std::string::npos ? path.size() : j);
    if (!cur.empty() && mkdir(cur.c_str(), 0755) != 0 && errno != EEXIST) return false;
    if (j == std::string::npos) break;
    i = j + 1;
  }
  struct stat st;
  return stat(path.c_str(), &st) == 0 && S_ISDIR(st.st_mode);
}

template <class T, class F>
void write_list(std::ostream &os, int64_t n, F &&value, bool binary) {
  if (binary) {
    std::vector<T> v(n);
    for (int64_t i = 0; i < n; ++i) v[i] = value(i);
    os << vtk_binary(v.data(), sizeof(T) * n);
  } else {
    for (int64_t i = 0; i < n; ++i) os << +value(i) << ' ';
  }
}

// Checksum of the restart payload: 64-bit FNV-1a over 8-byte words.
uint64_t checksum(const double *p, size_t n) {
  uint64_t h = 1469598103934665603ull;
  for (size_t i = 0; i < n; ++i) {
    uint64_t w;
    std::memcpy(&w, p + i, 8);
    h = (h ^ w) * 1099511628211ull;
  }
  return h;
}

struct RestartHeader {
  char magic[8];
  uint32_t version;
  int32_t scheme, degree, n_fields;
  int64_t n_cells;
  double t;
  uint64_t checksum;
};
const char kRestartMagic[8] = {'M', 'C', 'F', 'D', 'R', 'S', 'T', '\0'};

// VTK local coordinates of the written elements (mesh/vtk.hpp:214-224,
// 310-330), for the host-side points of curved cells: Hexahedron27 in
// [-1, 1]^3 and Tetrahedron10 in units of 1/2, VTK node order.
const signed char kHostHex27[27][3] = {
    {-1, -1, -1}, {1, -1, -1}, {1, 1, -1}, {-1, 1, -1}, {-1, -1, 1}, {1, -1, 1}, {1, 1, 1},
    {-1, 1, 1},   {0, -1, -1}, {1, 0, -1}, {0, 1, -1},  {-1, 0, -1}, {0, -1, 1},  {1, 0, 1},
    {0, 1, 1},    {-1, 0, 1},  {-1, -1, 0}, {1, -1, 0}, {1, 1, 0},   {-1, 1, 0},  {-1, 0, 0},
    {1, 0, 0},    {0, -1, 0},  {0, 1, 0},  {0, 0, -1},  {0, 0, 1},   {0, 0, 0}};
const signed char kHostTet10Half[10][3] = {{2, 0, 0}, {0, 2, 0}, {0, 0, 2}, {0, 0, 0}, {1, 1, 0},
                                           {0, 1, 1}, {1, 0, 1}, {1, 0, 0}, {0, 1, 0}, {0, 0, 1}};

// Wedge15 local coordinates (a, b, z) of Writer<Part> (mesh/vtk.hpp:251-270):
// corners, bottom and top edge midpoints, vertical edge midpoints.
const double kHostWedge15[15][3] = {
    {1, 0, -1},   {0, 1, -1},   {0, 0, -1},   {1, 0, 1},     {0, 1, 1},
    {0, 0, 1},    {0.5, 0.5, -1}, {0, 0.5, -1}, {0.5, 0, -1}, {0.5, 0.5, 1},
    {0, 0.5, 1},  {0.5, 0, 1},  {1, 0, 0},    {0, 1, 0},     {0, 0, 0}};

// VTK points per cell: Hexahedron27, Tetrahedron10, Wedge15 (host_types 0, 1, 2).
int vtk_cell_points(uint8_t type) { return type == 1 ? 10 : type == 2 ? 15 : 27; }

// The VTK points of every cell through its own map (quadratic and wedge cells).
void host_vtk_points(const mcfd_handle *h, const std::vector<int64_t> &off, double *xyz) {
  const auto &m = h->mesh;
  for (int64_t c = 0; c < m.n_cells; ++c) {
    const int t = m.host_cell_type[c];
    const bool tet = mcfd::geo::is_tet(t), wedge = mcfd::geo::is_wedge(t);
    const double *xn = &m.host_nodes[(size_t)c * mcfd::geo::kMaxNodes * 3];
    for (int s = 0; s < vtk_cell_points(m.host_types[c]); ++s) {
      double loc[3], J[9];
      for (int e = 0; e < 3; ++e)
        loc[e] = tet ? 0.5 * kHostTet10Half[s][e] : wedge ? kHostWedge15[s][e] : kHostHex27[s][e];
      mcfd::geo::map_point(t, xn, loc, &xyz[(off[c] + s) * 3], J);
    }
  }
}

// VTK point offsets of the cells.
std::vector<int64_t> vtk_offsets(const mcfd_handle *h) {
  const auto &types = h->mesh.host_types;
  std::vector<int64_t> off(types.size() + 1, 0);
  for (size_t c = 0; c < types.size(); ++c) off[c + 1] = off[c] + vtk_cell_points(types[c]);
  return off;
}

// The reference's writer has no pyramid element (mesh/vtk.hpp:400-414).
bool has_pyramid(const mcfd_handle *h) {
  for (uint8_t t : h->mesh.host_types)
    if (t == 3) return true;
  return false;
}

}  // namespace

extern "C" {

int mcfd_base64_encode(const uint8_t *data, int64_t n, char *out, int64_t cap, int64_t *written) {
  if ((!data && n > 0) || n < 0 || !written) return MCFD_ERR_ARGUMENT;
  const std::string s = base64(data, (size_t)n);
  *written = (int64_t)s.size();
  if (!out) return MCFD_OK;  // size query
  if (cap < (int64_t)s.size() + 1) return MCFD_ERR_ARGUMENT;
  std::memcpy(out, s.c_str(), s.size() + 1);
  return MCFD_OK;
}

int mcfd_write_vtu_arrays(const char *directory, const char *soln_name, int64_t n_points,
                          const double *xyz, const double *values, int64_t n_cells,
                          const uint8_t *types, int32_t binary) {
  if (!directory || !soln_name || n_points < 0 || n_cells < 0 ||
      (n_points > 0 && (!xyz || !values)) || (n_cells > 0 && !types))
    return MCFD_ERR_ARGUMENT;
  int64_t total = 0;
  auto points_of = [](uint8_t t) { return t == kVtkHex27Type ? 27 : t == kVtkWedge15Type ? 15 : 10; };
  for (int64_t c = 0; c < n_cells; ++c) {
    if (types[c] != kVtkHex27Type && types[c] != kVtkTet10Type && types[c] != kVtkWedge15Type)
      return MCFD_ERR_ARGUMENT;
    total += points_of(types[c]);
  }
  if (total != n_points) return MCFD_ERR_ARGUMENT;
  const std::string dir(directory), name(soln_name);
  if (!make_dirs(dir + "/" + name)) return MCFD_ERR_IO;
  const std::string endian = little_endian() ? "\"LittleEndian\"" : "\"BigEndian\"";
  {
    std::ofstream pvtu(dir + "/" + name + ".pvtu");
    pvtu << "<VTKFile type=\"PUnstructuredGrid\" version=\"1.0\" byte_order=" << endian
         << " header_type=\"UInt64\">\n";
    pvtu << "  <PUnstructuredGrid GhostLevel=\"1\">\n";
    pvtu << "    <PPointData>\n";
    for (const char *f : kFieldNames) pvtu << "      <PDataArray type=\"Float64\" Name=\"" << f << "\"/>\n";
    pvtu << "    </PPointData>\n";
    pvtu << "    <PCellData>\n";
    pvtu << "    </PCellData>\n";
    pvtu << "    <PPoints>\n";
    pvtu << "      <PDataArray type=\"Float64\" Name=\"Points\" NumberOfComponents=\"3\"/>\n";
    pvtu << "    </PPoints>\n";
    pvtu << "    <Piece Source=\"./" << name << "/0.vtu\"/>\n";
    pvtu << "  </PUnstructuredGrid>\n";
    pvtu << "</VTKFile>\n";
    if (!pvtu) return MCFD_ERR_IO;
  }
  std::ofstream vtu(dir + "/" + name + "/0.vtu", std::ios::out | std::ios::binary);
  const char *format = binary ? "\"binary\"" : "\"ascii\"";
  vtu << "<VTKFile type=\"UnstructuredGrid\" version=\"1.0\" byte_order=" << endian
      << " header_type=\"UInt64\">\n";
  vtu << "  <UnstructuredGrid>\n";
  vtu << "    <Piece NumberOfPoints=\"" << n_points << "\" NumberOfCells=\"" << n_cells << "\">\n";
  vtu << "      <PointData>\n";
  for (int k = 0; k < kK5; ++k) {
    vtu << "        <DataArray type=\"Float64\" Name=\"" << kFieldNames[k] << "\" format=" << format
        << ">\n";
    write_list<double>(vtu, n_points, [&](int64_t i) { return values[i * kK5 + k]; }, binary);
    vtu << "\n        </DataArray>\n";
  }
  vtu << "      </PointData>\n";
  vtu << "      <CellData>\n";
  vtu << "      </CellData>\n";
  vtu << "      <Points>\n";
  vtu << "        <DataArray type=\"Float64\" Name=\"Points\" NumberOfComponents=\"3\" format="
      << "\"binary\"" << ">\n";
  vtu << vtk_binary(xyz, sizeof(double) * 3 * n_points);
  vtu << "\n        </DataArray>\n";
  vtu << "      </Points>\n";
  vtu << "      <Cells>\n";
  vtu << "        <DataArray type=\"Int32\" Name=\"connectivity\" format=\"ascii\">\n";
  for (int64_t i = 0; i < n_points; ++i) vtu << i << ' ';
  vtu << "\n        </DataArray>\n";
  vtu << "        <DataArray type=\"Int32\" Name=\"offsets\" format=" << format << ">\n";
  {
    std::vector<int32_t> off(n_cells);
    int64_t o = 0;
    for (int64_t c = 0; c < n_cells; ++c) off[c] = (int32_t)(o += points_of(types[c]));
    write_list<int32_t>(vtu, n_cells, [&](int64_t c) { return off[c]; }, binary);
  }
  vtu << "\n        </DataArray>\n";
  vtu << "        <DataArray type=\"UInt8\" Name=\"types\" format=" << format << ">\n";
  write_list<uint8_t>(vtu, n_cells, [&](int64_t c) { return types[c]; }, binary);
  vtu << "\n        </DataArray>\n";
  vtu << "      </Cells>\n";
  vtu << "    </Piece>\n";
  vtu << "  </UnstructuredGrid>\n";
  vtu << "</VTKFile>\n";
  return vtu ? MCFD_OK : MCFD_ERR_IO;
}

int mcfd_vtk_point_count(const mcfd_handle *h, int64_t *n_points) {
  if (!h || !n_points) return MCFD_ERR_ARGUMENT;
  if (has_pyramid(h)) return MCFD_ERR_UNSUPPORTED;
  *n_points = vtk_offsets(h).back();
  return MCFD_OK;
}

int mcfd_vtk_sample(mcfd_handle *h, double *xyz, double *values, uint8_t *types,
                    int64_t n_points) {
  if (!h || !xyz || !values || !types) return MCFD_ERR_ARGUMENT;
  if (has_pyramid(h)) return fail(h, MCFD_ERR_UNSUPPORTED, "the VTK writer has no pyramid cell (mesh/vtk.hpp:400-414)");
  const std::vector<int64_t> off = vtk_offsets(h);
  const int64_t np = off.back(), nc = h->mesh.n_cells;
  if (n_points != np) return fail(h, MCFD_ERR_ARGUMENT, "point count mismatch (mcfd_vtk_point_count)");
  cudaSetDevice(h->device);
  int64_t *d_off = nullptr;
  double *d_xyz = nullptr, *d_val = nullptr;
  cudaError_t e = cudaMalloc(&d_off, sizeof(int64_t) * (nc + 1));
  if (e == cudaSuccess) e = cudaMalloc(&d_xyz, sizeof(double) * 3 * np);
  if (e == cudaSuccess) e = cudaMalloc(&d_val, sizeof(double) * kK5 * np);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(d_off, off.data(), sizeof(int64_t) * (nc + 1), cudaMemcpyHostToDevice, h->stream);
  if (e == cudaSuccess && h->mesh.curved) {  // points through the quadratic maps, on the host
    host_vtk_points(h, off, xyz);
    e = cudaMemcpyAsync(d_xyz, xyz, sizeof(double) * 3 * np, cudaMemcpyHostToDevice, h->stream);
  }
  if (e == cudaSuccess) {
    h->launches += mcfd::launch_vtk_sample(h, h->buf.u, d_off, d_xyz, d_val);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(xyz, d_xyz, sizeof(double) * 3 * np, cudaMemcpyDeviceToHost, h->stream);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(values, d_val, sizeof(double) * kK5 * np, cudaMemcpyDeviceToHost, h->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
  cudaFree(d_off);
  cudaFree(d_xyz);
  cudaFree(d_val);
  if (e != cudaSuccess) return cuda_fail(h, e, "vtk sample");
  for (int64_t c = 0; c < nc; ++c) {
    const uint8_t t = h->mesh.host_types[c];
    types[c] = t == 1 ? kVtkTet10Type : t == 2 ? kVtkWedge15Type : kVtkHex27Type;
  }
  return MCFD_OK;
}

int mcfd_write_vtu(mcfd_handle *h, const char *directory, const char *soln_name, int32_t binary) {
  if (!h || !directory || !soln_name) return MCFD_ERR_ARGUMENT;
  int64_t np = 0;
  if (mcfd_vtk_point_count(h, &np))
    return fail(h, MCFD_ERR_UNSUPPORTED, "the VTK writer has no pyramid cell (mesh/vtk.hpp:400-414)");
  std::vector<double> xyz(3 * np), values(kK5 * np);
  std::vector<uint8_t> types(h->mesh.n_cells);
  int rc = mcfd_vtk_sample(h, xyz.data(), values.data(), types.data(), np);
  if (rc) return rc;
  rc = mcfd_write_vtu_arrays(directory, soln_name, np, xyz.data(), values.data(), h->mesh.n_cells,
                             types.data(), binary);
  if (rc == MCFD_ERR_IO) return fail(h, rc, std::string("cannot write ") + directory + "/" + soln_name);
  return rc;
}

int mcfd_gather_fields(mcfd_handle *h, double *d_fields, int64_t n) {
  if (!h || !d_fields) return MCFD_ERR_ARGUMENT;
  if (n != h->mesh.column) return fail(h, MCFD_ERR_ARGUMENT, "column size mismatch");
  cudaSetDevice(h->device);
  h->launches += mcfd::launch_fields_transpose(h, h->buf.u, d_fields, 1);
  OUT_TRY(h, cudaGetLastError());
  OUT_TRY(h, cudaStreamSynchronize(h->stream));
  return MCFD_OK;
}

int mcfd_scatter_fields(mcfd_handle *h, const double *d_fields, int64_t n) {
  if (!h || !d_fields) return MCFD_ERR_ARGUMENT;
  if (n != h->mesh.column) return fail(h, MCFD_ERR_ARGUMENT, "column size mismatch");
  cudaSetDevice(h->device);
  h->launches += mcfd::launch_fields_transpose(h, d_fields, h->buf.u, 0);
  mcfd::invalidate_trace(h, h->buf.u);
  OUT_TRY(h, cudaGetLastError());
  OUT_TRY(h, cudaStreamSynchronize(h->stream));
  return MCFD_OK;
}

int mcfd_write_restart(mcfd_handle *h, const char *path, double t) {
  if (!h || !path) return MCFD_ERR_ARGUMENT;
  cudaSetDevice(h->device);
  const int64_t n = h->mesh.column;
  double *d_fields = nullptr;
  OUT_TRY(h, cudaMalloc(&d_fields, sizeof(double) * n));
  std::vector<double> fields(n);
  int rc = mcfd_gather_fields(h, d_fields, n);
  cudaError_t e = rc ? cudaSuccess : cudaMemcpy(fields.data(), d_fields, sizeof(double) * n,
                                                cudaMemcpyDeviceToHost);
  cudaFree(d_fields);
  if (rc) return rc;
  if (e != cudaSuccess) return cuda_fail(h, e, "restart download");
  RestartHeader hd{};
  std::memcpy(hd.magic, kRestartMagic, 8);
  hd.version = 1;
  hd.scheme = h->opt.scheme;
  hd.degree = h->mesh.p;
  hd.n_fields = (int32_t)(n / h->mesh.n_cells);
  hd.n_cells = h->mesh.n_cells;
  hd.t = t;
  hd.checksum = checksum(fields.data(), fields.size());
  std::ofstream out(path, std::ios::out | std::ios::binary | std::ios::trunc);
  out.write(reinterpret_cast<const char *>(&hd), sizeof(hd));
  out.write(reinterpret_cast<const char *>(fields.data()), sizeof(double) * n);
  if (!out) return fail(h, MCFD_ERR_IO, std::string("cannot write ") + path);
  return MCFD_OK;
}

int mcfd_read_restart(mcfd_handle *h, const char *path, double *t) {
  if (!h || !path) return MCFD_ERR_ARGUMENT;
  std::ifstream in(path, std::ios::in | std::ios::binary);
  if (!in) return fail(h, MCFD_ERR_IO, std::string("cannot open ") + path);
  RestartHeader hd{};
  in.read(reinterpret_cast<char *>(&hd), sizeof(hd));
  if (!in || std::memcmp(hd.magic, kRestartMagic, 8) != 0 || hd.version != 1)
    return fail(h, MCFD_ERR_IO, "not a restart file of this library");
  const int64_t n = h->mesh.column;
  if (hd.scheme != h->opt.scheme || hd.degree != h->mesh.p || hd.n_cells != h->mesh.n_cells ||
      (int64_t)hd.n_fields * hd.n_cells != n)
    return fail(h, MCFD_ERR_ARGUMENT, "restart file does not match the handle's mesh and scheme");
  std::vector<double> fields(n);
  in.read(reinterpret_cast<char *>(fields.data()), sizeof(double) * n);
  if (!in) return fail(h, MCFD_ERR_IO, "restart file is truncated");
  if (checksum(fields.data(), fields.size()) != hd.checksum)
    return fail(h, MCFD_ERR_IO, "restart file checksum mismatch");
  cudaSetDevice(h->device);
  double *d_fields = nullptr;
  OUT_TRY(h, cudaMalloc(&d_fields, sizeof(double) * n));
  cudaError_t e = cudaMemcpy(d_fields, fields.data(), sizeof(double) * n, cudaMemcpyHostToDevice);
  int rc = e == cudaSuccess ? mcfd_scatter_fields(h, d_fields, n) : cuda_fail(h, e, "restart upload");
  cudaFree(d_fields);
  if (rc) return rc;
  h->t_host = hd.t;
  if (t) *t = hd.t;
  return MCFD_OK;
}

}  // extern "C"
