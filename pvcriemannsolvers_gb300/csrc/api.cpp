// C ABI of the GB300 DGSEM Euler residual + SSP-RK library (include/mcfd.h).
//
// mcfd_create ingests an unstructured Hex8 mesh and builds, on the host in
// FP64, everything the reference's FiniteElement / dg::Lobatto constructors
// build (spatial/fem.hpp:95-115, spatial/dg/lobatto.hpp:58-125,
// polynomial/hexahedron.hpp:221-239, integrator/element.hpp:102-115):
//   * per cell node: the global weight w = w_i w_j w_k det(J) and w J^-1,
//     stored together with 1/w (the lumped GLL mass);
//   * per face point: the unit normal of the holder-sorted Quad4 face
//     (coordinate/face.hpp:54-62) and the face weight w_a w_b |x_a x x_b|;
//   * face-point -> cell-node maps.  The reference searches every cell node
//     for one within 1e-12 of the face point (lobatto.hpp:58-78); here the map
//     follows from the two local face indices and the corner correspondence,
//     and every matched pair is then checked geometrically;
//   * per cell and local face the flux slots each face node lifts from.
// Everything is uploaded once; the solution column stays on the device.
#include <cuda_runtime.h>

#include <algorithm>
#include <climits>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "../../include/mcfd.h"
#include "euler.cuh"
#include "geometry.hpp"
#include "handle.hpp"

namespace {

using mcfd::BcDev;

thread_local std::string g_create_error;

// Hex8 local corner coordinates and the first four nodes of each face of
// the CGNS hexahedron (coordinate/hexahedron.hpp:353-389): the face node
// order fixes the face parametrisation and the outward normal.
const int kHexLocal[8][3] = {{-1, -1, -1}, {+1, -1, -1}, {+1, +1, -1},
                             {-1, +1, -1}, {-1, -1, +1}, {+1, -1, +1},
                             {+1, +1, +1}, {-1, +1, +1}};
const int kHexFace[6][4] = {{0, 3, 2, 1}, {0, 1, 5, 4}, {1, 2, 6, 5},
                            {2, 3, 7, 6}, {0, 4, 7, 3}, {4, 5, 6, 7}};

// Gauss-Lobatto rule (integrator/lobatto.hpp:37-83).
void gll(int q, double *x, double *w) {
  if (q == 2) {
    x[0] = -1; x[1] = 1; w[0] = 1; w[1] = 1;
  } else if (q == 3) {
    x[0] = -1; x[1] = 0; x[2] = 1;
    w[0] = 1.0 / 3; w[1] = 4.0 / 3; w[2] = 1.0 / 3;
  } else {
    x[0] = -1; x[1] = -std::sqrt(1.0 / 5); x[2] = std::sqrt(1.0 / 5); x[3] = 1;
    w[0] = 1.0 / 6; w[1] = 5.0 / 6; w[2] = 5.0 / 6; w[3] = 1.0 / 6;
  }
}

// Lagrange differentiation matrix D[a][i] = l_i'(x_a) in barycentric form.
void diff_matrix(int q, const double *x, double *d) {
  double bw[8];
  for (int i = 0; i < q; ++i) {
    double p = 1;
    for (int j = 0; j < q; ++j)
      if (j != i) p *= (x[i] - x[j]);
    bw[i] = 1.0 / p;
  }
  for (int a = 0; a < q; ++a) {
    double diag = 0;
    for (int i = 0; i < q; ++i) {
      if (i == a) continue;
      double v = (bw[i] / bw[a]) / (x[a] - x[i]);
      d[a * q + i] = v;
      diag -= v;
    }
    d[a * q + a] = diag;
  }
}

void hex8_point(const double *xn, double a, double b, double c, double *x,
                double *jac) {
  x[0] = x[1] = x[2] = 0;
  for (int e = 0; e < 9; ++e) jac[e] = 0;
  for (int v = 0; v < 8; ++v) {
    double fa = 1 + kHexLocal[v][0] * a, fb = 1 + kHexLocal[v][1] * b,
           fc = 1 + kHexLocal[v][2] * c;
    double s = fa * fb * fc / 8;
    double g[3] = {kHexLocal[v][0] * fb * fc / 8, kHexLocal[v][1] * fa * fc / 8,
                   kHexLocal[v][2] * fa * fb / 8};
    for (int d = 0; d < 3; ++d) {
      x[d] += s * xn[v * 3 + d];
      for (int r = 0; r < 3; ++r) jac[r * 3 + d] += g[r] * xn[v * 3 + d];
    }
  }
}

void quad4_point(const double *xn, double a, double b, double *x, double *ta,
                 double *tb) {
  const int loc[4][2] = {{-1, -1}, {+1, -1}, {+1, +1}, {-1, +1}};
  for (int d = 0; d < 3; ++d) x[d] = ta[d] = tb[d] = 0;
  for (int v = 0; v < 4; ++v) {
    double fa = 1 + loc[v][0] * a, fb = 1 + loc[v][1] * b;
    for (int d = 0; d < 3; ++d) {
      x[d] += fa * fb / 4 * xn[v * 3 + d];
      ta[d] += loc[v][0] * fb / 4 * xn[v * 3 + d];
      tb[d] += loc[v][1] * fa / 4 * xn[v * 3 + d];
    }
  }
}

// Slope at xi = 1 of Huynh's g2 correction function g_R = (P_p + c_prev
// P_{p-1} + c_next P_{p+1}) / 2 with c_next = p / (2p + 1)
// (basis/vincent.hpp:30-32, 57-61): P_n'(1) = n (n + 1) / 2.
double fr_correction_slope(int p) {
  double c_next = p / (2.0 * p + 1), c_prev = 1 - c_next;
  auto dp = [](int n) { return n * (n + 1) / 2.0; };
  return 0.5 * (dp(p) + c_prev * dp(p - 1) + c_next * dp(p + 1));
}

// Grid index (i, j, k) of hex corner v on a Q-point GLL grid.
void corner_grid(int v, int q, int *g) {
  for (int d = 0; d < 3; ++d) g[d] = (kHexLocal[v][d] + 1) / 2 * (q - 1);
}

int fail(mcfd_handle *h, int code, const std::string &msg) {
  if (h) h->err = msg; else g_create_error = msg;
  return code;
}

int cuda_fail(mcfd_handle *h, cudaError_t e, const char *what) {
  return fail(h, MCFD_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

#define CUDA_TRY(h, call)                                  \
  do {                                                     \
    cudaError_t e_ = (call);                               \
    if (e_ != cudaSuccess) return cuda_fail(h, e_, #call); \
  } while (0)

template <class T>
int upload(mcfd_handle *h, T **dst, const std::vector<T> &src) {
  if (src.empty()) { *dst = nullptr; return MCFD_OK; }
  CUDA_TRY(h, cudaMalloc(dst, sizeof(T) * src.size()));
  CUDA_TRY(h, cudaMemcpy(*dst, src.data(), sizeof(T) * src.size(), cudaMemcpyHostToDevice));
  return MCFD_OK;
}

// Staging buffers, copy streams and events of streamed stepping.
void stream_release(mcfd_handle *h) {
  auto &st = h->streamer;
  for (int b = 0; b < 2; ++b) {
    if (st.in[b]) cudaFree(st.in[b]);
    if (st.out[b]) cudaFree(st.out[b]);
    cudaEvent_t evs[] = {st.in_ready[b], st.in_free[b], st.out_ready[b], st.out_free[b]};
    for (cudaEvent_t e : evs)
      if (e) cudaEventDestroy(e);
    if (st.graph[b]) cudaGraphExecDestroy(st.graph[b]);
  }
  if (st.copy_in) cudaStreamDestroy(st.copy_in);
  if (st.copy_out) cudaStreamDestroy(st.copy_out);
  st = mcfd::Streamer{};
}

void release(mcfd_handle *h) {
  stream_release(h);
  auto &m = h->mesh;
  auto &b = h->buf;
  void *ptrs[] = {m.cell_geo, m.cell_geo32, m.node_w32, m.cell_rate, m.cell_rate32, m.cell_flux, m.face_cells,
                  m.face_group, m.face_geo, m.face_nh, m.face_xyz, m.face_map, m.dmat,
                  m.bcs, m.corners, m.cell_type, b.u, b.u1, b.u2, b.res, b.flux, b.trace, b.state, b.dt_hi};
  for (void *p : ptrs)
    if (p) cudaFree(p);
  auto &l = h->lim;
  void *lptrs[] = {l.psi, l.mn, l.mn32, l.proj, l.beta, l.eval, l.s00, l.divisor, l.adj,
                   l.frame, l.volume, l.modal, l.list, l.list_count, l.troubled, l.cell_hot,
                   l.cell_hot2, l.block_hot};
  for (void *p : lptrs)
    if (p) cudaFree(p);
  auto &cs = h->cases;
  void *cptrs[] = {cs.cell_case, cs.t, cs.dt, cs.rate};
  for (void *p : cptrs)
    if (p) cudaFree(p);
  auto &md = h->modal;
  void *mptrs[] = {md.center, md.s, md.vol_off, md.vol, md.cell_faces, md.face_off,
                   md.point_face, md.fpt, md.fnrm, md.fshift, md.taylor, md.values,
                   md.s32, md.vol32, md.foff32, md.taylor32};
  for (void *p : mptrs)
    if (p) cudaFree(p);
  mcfd::release_viscosity(h);
  if (h->mesh.node_w) cudaFree(h->mesh.node_w);
  if (m.bc_row) cudaFree(m.bc_row);
  for (double *t : m.bc_tables)
    if (t) cudaFree(t);
  mcfd::drop_graphs(h);
  if (h->own_stream && h->stream) cudaStreamDestroy(h->stream);
}

// Cell corners and types for output sampling (Tet4 cells: the first four
// cell_nodes entries, the rest zero).
int upload_corners(mcfd_handle *h, const mcfd_mesh_desc *d) {
  const int64_t nc = d->n_cells, S = d->cell_node_stride > 0 ? d->cell_node_stride : 8;
  std::vector<double> corners(nc * 24, 0.0);
  auto &types = h->mesh.host_types;
  auto &m = h->mesh;
  types.assign(nc, 0);
  m.host_cell_type.assign(nc, MCFD_HEX8);
  m.curved = false;
  for (int64_t c = 0; c < nc; ++c) {
    const int t = d->cell_type ? d->cell_type[c] : 0;
    m.host_cell_type[c] = (uint8_t)t;
    m.curved = m.curved || mcfd::geo::curved(t) || mcfd::geo::is_wedge(t) || mcfd::geo::is_pyramid(t);
    types[c] = (uint8_t)(mcfd::geo::is_tet(t) ? 1 : mcfd::geo::is_wedge(t) ? 2 : mcfd::geo::is_pyramid(t) ? 3 : 0);
    const int nv = mcfd::geo::corner_count(t);
    for (int v = 0; v < nv; ++v) {
      const int64_t id = d->cell_nodes[c * S + v];
      if (id < 0 || id >= d->n_nodes) return fail(h, MCFD_ERR_ARGUMENT, "cell node index out of range");
      for (int e = 0; e < 3; ++e) corners[(c * 8 + v) * 3 + e] = d->xyz[id * 3 + e];
    }
  }
  if (m.curved) {  // every node of every cell, for the output sampling points
    m.host_nodes.assign((size_t)nc * mcfd::geo::kMaxNodes * 3, 0.0);
    for (int64_t c = 0; c < nc; ++c) {
      const int nv = mcfd::geo::node_count(m.host_cell_type[c]);
      for (int v = 0; v < nv; ++v)
        for (int e = 0; e < 3; ++e)
          m.host_nodes[((size_t)c * mcfd::geo::kMaxNodes + v) * 3 + e] = d->xyz[d->cell_nodes[c * S + v] * 3 + e];
    }
  }
  int rc = upload(h, &h->mesh.corners, corners);
  if (!rc) rc = upload(h, &h->mesh.cell_type, types);
  m.host_corners = std::move(corners);
  return rc;
}

int check_status(mcfd_handle *h) {
  mcfd::DevState st;
  CUDA_TRY(h, cudaMemcpyAsync(&st, h->buf.state, sizeof(st), cudaMemcpyDeviceToHost, h->stream));
  CUDA_TRY(h, cudaStreamSynchronize(h->stream));
  CUDA_TRY(h, cudaGetLastError());
  if (st.status) {
    unsigned zero = 0;
    CUDA_TRY(h, cudaMemcpy(&h->buf.state->status, &zero, sizeof(zero), cudaMemcpyHostToDevice));
    if (st.status & mcfd::kStatusNotConverged)
      return fail(h, MCFD_ERR_NOT_CONVERGED, "Exact Riemann solver reached its iteration cap");
    return fail(h, MCFD_ERR_STATE, "a kernel produced a non-finite value");
  }
  return MCFD_OK;
}

double cfl_table(int rk_order, int p) {
  // spatial/fem.hpp:26-37
  static const double cfl[5][9] = {
      {1.000},
      {1.000, 0.333},
      {1.000, 0.333, 0.209, 0.130, 0.089, 0.066, 0.051, 0.040, 0.033},
      {1.256, 0.409, 0.209, 0.130, 0.089, 0.066, 0.051, 0.040, 0.033},
      {1.392, 0.464, 0.235, 0.145, 0.100, 0.073, 0.056, 0.045, 0.037}};
  rk_order = std::min(std::max(rk_order, 0), 4);
  return cfl[rk_order][std::min(p, 8)];
}

int build_mesh(mcfd_handle *h, const mcfd_mesh_desc *d, int degree) {
  auto &m = h->mesh;
  m.p = degree;
  m.q = degree + 1;
  m.n = m.q * m.q * m.q;
  m.qf = m.q * m.q;
  m.n_cells = d->n_cells;
  m.n_faces = d->n_faces;
  m.n_points = d->n_faces * m.qf;
  m.column = d->n_cells * mcfd::kK * m.n;
  const int Q = m.q, N = m.n, QF = m.qf;
  double xq[4], wq[4], dm[16];
  gll(Q, xq, wq);
  for (int i = 0; i < Q; ++i) h->mesh.xq[i] = xq[i];
  diff_matrix(Q, xq, dm);
  const int64_t S = d->cell_node_stride > 0 ? d->cell_node_stride : 8;
  std::vector<int> ctype(d->n_cells, MCFD_HEX8);
  for (int64_t c = 0; c < d->n_cells; ++c) {
    const int t = d->cell_type ? d->cell_type[c] : MCFD_HEX8;
    if (!mcfd::geo::is_hex(t))
      return fail(h, MCFD_ERR_UNSUPPORTED, "the nodal schemes take hexahedra (Hex8, Hex20, Hex27) only");
    if (mcfd::geo::node_count(t) > S)
      return fail(h, MCFD_ERR_MESH, "cell_node_stride is below the node count of cell " + std::to_string(c));
    ctype[c] = t;
    for (int v = 0; v < mcfd::geo::node_count(t); ++v) {
      int64_t id = d->cell_nodes[c * S + v];
      if (id < 0 || id >= d->n_nodes)
        return fail(h, MCFD_ERR_MESH, "cell node index out of range in cell " + std::to_string(c));
    }
  }
  // all nodes of cell c, [n][3]
  auto gather = [&](int64_t c, double *xn) {
    for (int v = 0; v < mcfd::geo::node_count(ctype[c]); ++v)
      for (int e = 0; e < 3; ++e) xn[v * 3 + e] = d->xyz[d->cell_nodes[c * S + v] * 3 + e];
  };
  // x and J at a local point of cell c (Hex8 through the trilinear map)
  auto cell_point = [&](int64_t c, const double *xn, double a, double b, double cc, double *x, double *J) {
    if (ctype[c] == MCFD_HEX8) {
      hex8_point(xn, a, b, cc, x, J);
    } else {
      const double loc[3] = {a, b, cc};
      mcfd::geo::map_point(ctype[c], xn, loc, x, J);
    }
  };
  // ---- per node geometry
  std::vector<double> geo((size_t)d->n_cells * N * 10);
  std::vector<double> rate(d->n_cells);
  // per cell adj(J) and det(J) at its first node, and whether every node of
  // the cell has the same ones (an affine cell: the mixed form then stores its
  // FP32 metric terms once per cell)
  std::vector<double> adj0((size_t)d->n_cells * 10);
  std::vector<uint8_t> affine(d->n_cells, 1);
  int bad_jac = 0;
#pragma omp parallel for schedule(static)
  for (int64_t c = 0; c < d->n_cells; ++c) {
    double xn[mcfd::geo::kMaxNodes * 3];
    gather(c, xn);
    double volume = 0;
    for (int i = 0; i < Q; ++i)
      for (int j = 0; j < Q; ++j)
        for (int k = 0; k < Q; ++k) {
          double x[3], J[9];
          cell_point(c, xn, xq[i], xq[j], xq[k], x, J);
          double det = J[0] * (J[4] * J[8] - J[5] * J[7]) -
                       J[1] * (J[3] * J[8] - J[5] * J[6]) +
                       J[2] * (J[3] * J[7] - J[4] * J[6]);
          if (!(det > 0)) bad_jac = 1;
          double w = wq[i] * wq[j] * wq[k] * det;
          volume += w;
          // DGSEM: w J^-1 = (w / det) adj(J) and the lumped mass 1/w.
          // FR: det(J) J^-1 = adj(J) (GetJacobianAssociated) and 1/det(J).
          const bool fr = h->opt.scheme == MCFD_FR;
          double s = fr ? 1.0 : w / det;
          double *g = &geo[((size_t)c * N + (i * Q + j) * Q + k) * 10];
          const double adj[9] = {J[4] * J[8] - J[5] * J[7], J[2] * J[7] - J[1] * J[8],
                                 J[1] * J[5] - J[2] * J[4], J[5] * J[6] - J[3] * J[8],
                                 J[0] * J[8] - J[2] * J[6], J[2] * J[3] - J[0] * J[5],
                                 J[3] * J[7] - J[4] * J[6], J[1] * J[6] - J[0] * J[7],
                                 J[0] * J[4] - J[1] * J[3]};
          for (int e = 0; e < 9; ++e) g[e] = s * adj[e];
          g[9] = fr ? 1.0 / det : 1.0 / w;
          double *a0 = &adj0[(size_t)c * 10];
          if (i == 0 && j == 0 && k == 0) {
            for (int e = 0; e < 9; ++e) a0[e] = adj[e];
            a0[9] = det;
          } else {
            double scale = 0;
            for (int e = 0; e < 9; ++e) scale = std::max(scale, std::fabs(a0[e]));
            for (int e = 0; e < 9; ++e)
              if (std::fabs(adj[e] - a0[e]) > 1e-13 * scale) affine[c] = 0;
            if (std::fabs(det - a0[9]) > 1e-13 * std::fabs(a0[9])) affine[c] = 0;
          }
        }
    rate[c] = 1.0 / (std::cbrt(volume) * 0.5);
  }
  if (bad_jac) return fail(h, MCFD_ERR_MESH, "non-positive Jacobian determinant at a cell node");
  // ---- faces
  std::vector<int2> fcells(d->n_faces);
  std::vector<int32_t> fgroup(d->n_faces);
  std::vector<double4> fgeo(m.n_points);
  std::vector<double> fxyz(m.n_points * 3);
  std::vector<short2> fmap(m.n_points);
  m.map_h.assign(m.n_points, -1);
  m.map_s.assign(m.n_points, -1);
  std::vector<int32_t> cflux((size_t)d->n_cells * 6 * QF, INT32_MIN);
  int max_group = -1;
  std::string mesh_error;
  m.host_face_sides.assign((size_t)d->n_faces * 2, -1);
  if (d->face_shift) m.host_shift.assign(d->face_shift, d->face_shift + d->n_faces * 3);
  else m.host_shift.clear();
  for (int64_t f = 0; f < d->n_faces; ++f) {
    int64_t hc = d->face_cells[f * 2], sc = d->face_cells[f * 2 + 1];
    int sh = d->face_sides[f * 2], ss = d->face_sides[f * 2 + 1];
    if (hc < 0 || hc >= d->n_cells || sh < 0 || sh > 5 || sc >= d->n_cells ||
        (sc >= 0 && (ss < 0 || ss > 5)) || hc > INT32_MAX) {
      return fail(h, MCFD_ERR_MESH, "bad face record " + std::to_string(f));
    }
    fcells[f] = make_int2((int)hc, (int)sc);
    fgroup[f] = d->face_group ? d->face_group[f] : -1;
    m.host_face_sides[f * 2] = (int8_t)sh;
    m.host_face_sides[f * 2 + 1] = (int8_t)(sc >= 0 ? ss : -1);
    if (sc < 0) max_group = std::max(max_group, fgroup[f]);
  }
  m.n_groups = max_group + 1;
#pragma omp parallel for schedule(static)
  for (int64_t f = 0; f < d->n_faces; ++f) {
    int64_t hc = d->face_cells[f * 2], sc = d->face_cells[f * 2 + 1];
    int sh = d->face_sides[f * 2], ss = d->face_sides[f * 2 + 1];
    double xn[12];
    int hg[4][3];
    for (int v = 0; v < 4; ++v) {
      int hv = kHexFace[sh][v];
      corner_grid(hv, Q, hg[v]);
      for (int e = 0; e < 3; ++e) xn[v * 3 + e] = d->xyz[d->cell_nodes[hc * S + hv] * 3 + e];
    }
    // curved holder: face points from the cell map at the face's local
    // points, tangents J^T dloc/da and J^T dloc/db (the face is a square of
    // the local cube, corner 0 -> 1 along a, corner 0 -> 3 along b)
    const bool curved_face = ctype[hc] != MCFD_HEX8;
    double xc[mcfd::geo::kMaxNodes * 3], l0[3], da[3], db[3];
    if (curved_face) {
      gather(hc, xc);
      double l1[3], l3[3];
      for (int e = 0; e < 3; ++e) {
        l0[e] = kHexLocal[kHexFace[sh][0]][e];
        l1[e] = kHexLocal[kHexFace[sh][1]][e];
        l3[e] = kHexLocal[kHexFace[sh][3]][e];
        da[e] = (l1[e] - l0[e]) / 2;
        db[e] = (l3[e] - l0[e]) / 2;
      }
    }
    double shift[3] = {0, 0, 0};
    if (d->face_shift)
      for (int e = 0; e < 3; ++e) shift[e] = d->face_shift[f * 3 + e];
    // sharer corner matched to each holder face corner
    int sg[4][3];
    if (sc >= 0) {
      for (int v = 0; v < 4; ++v) {
        int64_t hid = d->cell_nodes[hc * S + kHexFace[sh][v]];
        int best = -1;
        double best_d = 1e300;
        for (int w = 0; w < 4; ++w) {
          int sv = kHexFace[ss][w];
          int64_t sid = d->cell_nodes[sc * S + sv];
          double dd = 0;
          for (int e = 0; e < 3; ++e) {
            double diff = d->xyz[sid * 3 + e] + shift[e] - d->xyz[hid * 3 + e];
            dd += diff * diff;
          }
          if (sid == hid && !d->face_shift) dd = -1;
          if (dd < best_d) { best_d = dd; best = sv; }
        }
        corner_grid(best, Q, sg[v]);
      }
    }
    double scale = 0;
    for (int e = 0; e < 12; ++e) scale = std::max(scale, std::fabs(xn[e]));
    double tol = 1e-10 * (1 + scale);
    for (int a = 0; a < Q; ++a)
      for (int b = 0; b < Q; ++b) {
        int fp = a * Q + b;
        int64_t pt = f * QF + fp;
        double x[3], ta[3], tb[3];
        if (curved_face) {
          double loc[3], J[9];
          for (int e = 0; e < 3; ++e) loc[e] = l0[e] + (xq[a] + 1) * da[e] + (xq[b] + 1) * db[e];
          mcfd::geo::map_point(ctype[hc], xc, loc, x, J);
          mcfd::geo::tangent(J, da, ta);
          mcfd::geo::tangent(J, db, tb);
        } else {
          quad4_point(xn, xq[a], xq[b], x, ta, tb);
        }
        double nrm[3] = {ta[1] * tb[2] - ta[2] * tb[1], ta[2] * tb[0] - ta[0] * tb[2],
                         ta[0] * tb[1] - ta[1] * tb[0]};
        double area = std::sqrt(nrm[0] * nrm[0] + nrm[1] * nrm[1] + nrm[2] * nrm[2]);
        // DGSEM lifts the flux with the face quadrature weight; FR scales it
        // by the area element |det(J) J^-1 e_dir| of the flux point.
        fgeo[pt] = make_double4(nrm[0] / area, nrm[1] / area, nrm[2] / area,
                                h->opt.scheme == MCFD_FR ? area : wq[a] * wq[b] * area);
        for (int e = 0; e < 3; ++e) fxyz[pt * 3 + e] = x[e];
        int gi[3], node_h, node_s = -1;
        for (int e = 0; e < 3; ++e)
          gi[e] = hg[0][e] + a * (hg[1][e] - hg[0][e]) / (Q - 1) + b * (hg[3][e] - hg[0][e]) / (Q - 1);
        node_h = (gi[0] * Q + gi[1]) * Q + gi[2];
        if (sc >= 0) {
          for (int e = 0; e < 3; ++e)
            gi[e] = sg[0][e] + a * (sg[1][e] - sg[0][e]) / (Q - 1) + b * (sg[3][e] - sg[0][e]) / (Q - 1);
          node_s = (gi[0] * Q + gi[1]) * Q + gi[2];
        }
        m.map_h[pt] = (int16_t)node_h;
        m.map_s[pt] = (int16_t)node_s;
        fmap[pt] = make_short2((short)node_h, (short)node_s);
      }
  }
  // geometric check of every matched pair and flux-slot table
  for (int64_t f = 0; f < d->n_faces && mesh_error.empty(); ++f) {
    int64_t hc = d->face_cells[f * 2], sc = d->face_cells[f * 2 + 1];
    int sh = d->face_sides[f * 2], ss = d->face_sides[f * 2 + 1];
    for (int fp = 0; fp < QF; ++fp) {
      int64_t pt = f * QF + fp;
      int sides[2] = {sh, ss};
      int64_t cells[2] = {hc, sc};
      int nodes[2] = {m.map_h[pt], m.map_s[pt]};
      for (int s = 0; s < 2; ++s) {
        if (cells[s] < 0) continue;
        int node = nodes[s];
        int i = node / QF, j = (node / Q) % Q, k = node % Q;
        int t;
        switch (sides[s]) {
          case 0: t = (k == 0) ? i * Q + j : -1; break;
          case 5: t = (k == Q - 1) ? i * Q + j : -1; break;
          case 1: t = (j == 0) ? i * Q + k : -1; break;
          case 3: t = (j == Q - 1) ? i * Q + k : -1; break;
          case 4: t = (i == 0) ? j * Q + k : -1; break;
          default: t = (i == Q - 1) ? j * Q + k : -1; break;
        }
        if (t < 0) { mesh_error = "face node off its local face at face " + std::to_string(f); break; }
        int32_t &slot = cflux[((size_t)cells[s] * 6 + sides[s]) * QF + t];
        if (slot != INT32_MIN) { mesh_error = "cell face used twice at face " + std::to_string(f); break; }
        if (pt > INT32_MAX) { mesh_error = "too many face points"; break; }
        slot = s == 0 ? (int32_t)pt : ~(int32_t)pt;
      }
      if (!mesh_error.empty()) break;
    }
  }
  if (!mesh_error.empty()) return fail(h, MCFD_ERR_MESH, mesh_error);
  // verify matched positions: face point == holder node == sharer node (+shift)
  int bad_match = 0;
#pragma omp parallel for schedule(static)
  for (int64_t f = 0; f < d->n_faces; ++f) {
    int64_t hc = d->face_cells[f * 2], sc = d->face_cells[f * 2 + 1];
    double xh[mcfd::geo::kMaxNodes * 3], xs[mcfd::geo::kMaxNodes * 3];
    gather(hc, xh);
    if (sc >= 0) gather(sc, xs);
    double shift[3] = {0, 0, 0};
    if (d->face_shift)
      for (int e = 0; e < 3; ++e) shift[e] = d->face_shift[f * 3 + e];
    for (int fp = 0; fp < QF; ++fp) {
      int64_t pt = f * QF + fp;
      const double *x = &fxyz[pt * 3];
      double scale = 1 + std::fabs(x[0]) + std::fabs(x[1]) + std::fabs(x[2]);
      double p[3], J[9];
      int node = m.map_h[pt];
      cell_point(hc, xh, xq[node / QF], xq[(node / Q) % Q], xq[node % Q], p, J);
      double e2 = 0;
      for (int e = 0; e < 3; ++e) e2 += (p[e] - x[e]) * (p[e] - x[e]);
      if (std::sqrt(e2) > 1e-10 * scale) bad_match = 1;
      if (sc >= 0) {
        node = m.map_s[pt];
        cell_point(sc, xs, xq[node / QF], xq[(node / Q) % Q], xq[node % Q], p, J);
        e2 = 0;
        for (int e = 0; e < 3; ++e) e2 += (p[e] + shift[e] - x[e]) * (p[e] + shift[e] - x[e]);
        if (std::sqrt(e2) > 1e-10 * scale) bad_match = 1;
      }
    }
  }
  if (bad_match) return fail(h, MCFD_ERR_MESH, "a face point matches no node of its cells");
  // ---- upload
  int rc;
  if (h->opt.precision == MCFD_MIXED) {
    m.geo32_affine = d->n_cells > 0;
    for (int64_t c = 0; c < d->n_cells && m.geo32_affine; ++c) m.geo32_affine = affine[c] != 0;
    if (m.geo32_affine) {
      // per cell adj(J) and 1/det(J); per node w_q and 1/w_q (DGSEM: the
      // node's metric terms are w_q adj(J) and 1/(w_q det(J))) or 1 (FR)
      std::vector<float> geo32((size_t)d->n_cells * 10);
#pragma omp parallel for schedule(static)
      for (int64_t c = 0; c < d->n_cells; ++c) {
        for (int e = 0; e < 9; ++e) geo32[(size_t)c * 10 + e] = (float)adj0[(size_t)c * 10 + e];
        geo32[(size_t)c * 10 + 9] = (float)(1.0 / adj0[(size_t)c * 10 + 9]);
      }
      if ((rc = upload(h, &m.cell_geo32, geo32))) return rc;
      std::vector<float> w32(2 * (size_t)N);
      const bool fr = h->opt.scheme == MCFD_FR;
      for (int i = 0; i < Q; ++i)
        for (int j = 0; j < Q; ++j)
          for (int k = 0; k < Q; ++k) {
            const double w = wq[i] * wq[j] * wq[k];
            w32[(i * Q + j) * Q + k] = fr ? 1.f : (float)w;
            w32[N + (i * Q + j) * Q + k] = fr ? 1.f : (float)(1.0 / w);
          }
      if ((rc = upload(h, &m.node_w32, w32))) return rc;
    } else {
      std::vector<float> geo32((size_t)d->n_cells * N * 10);
#pragma omp parallel for schedule(static)
      for (int64_t i = 0; i < d->n_cells * N; ++i)
        for (int e = 0; e < 10; ++e) geo32[(size_t)i * 10 + e] = (float)geo[(size_t)i * 10 + e];
      if ((rc = upload(h, &m.cell_geo32, geo32))) return rc;
    }
    std::vector<float> rate32(rate.begin(), rate.end());
    if ((rc = upload(h, &m.cell_rate32, rate32))) return rc;
  }
  if ((rc = upload(h, &m.cell_geo, geo))) return rc;
  if ((rc = upload(h, &m.cell_rate, rate))) return rc;
  if ((rc = upload(h, &m.cell_flux, cflux))) return rc;
  if ((rc = upload(h, &m.face_cells, fcells))) return rc;
  if ((rc = upload(h, &m.face_group, fgroup))) return rc;
  if ((rc = upload(h, &m.face_geo, fgeo))) return rc;
  if (h->opt.riemann == MCFD_RUSANOV) {
    // the half-weighted normals of the traced Rusanov flux, formed as the
    // face kernel formed them: (0.5 w) n_i
    std::vector<double4> fnh(m.n_points);
    for (int64_t i = 0; i < m.n_points; ++i) {
      const double hw = 0.5 * fgeo[i].w;
      fnh[i] = make_double4(hw * fgeo[i].x, hw * fgeo[i].y, hw * fgeo[i].z, hw);
    }
    if ((rc = upload(h, &m.face_nh, fnh))) return rc;
  }
  if ((rc = upload(h, &m.face_xyz, fxyz))) return rc;
  if ((rc = upload(h, &m.face_map, fmap))) return rc;
  std::vector<double> dvec(dm, dm + Q * Q);
  if ((rc = upload(h, &m.dmat, dvec))) return rc;
  m.host_bcs.assign(std::max(m.n_groups, 1), BcDev{});
  if ((rc = upload(h, &m.bcs, m.host_bcs))) return rc;
  return MCFD_OK;
}

// ---------------------------------------------------------------------------
// WENO limiter tables.  The modal basis of a cell (polynomial::Projection in
// polynomial::Extrapolation) is the set of Taylor monomials of total degree
// <= p about the cell centre, orthonormalised under the cell's own quadrature
// (the GLL nodes with weights w = w_i w_j w_k det J).  With A the Gram matrix
// of the monomials and A = L L^T its Cholesky factorisation, the basis is
// psi = L^-1 T: the unique lower-triangular orthonormalisation, i.e. the one
// the reference's Gram-Schmidt produces (integrator/function.hpp:139-172).

// exponents (x, y, z) of the Taylor monomials in the reference's order
// (basis/taylor.hpp:40-55, 200-218)
const int kTaylorExp[20][3] = {
    {0, 0, 0}, {1, 0, 0}, {0, 1, 0}, {0, 0, 1}, {2, 0, 0}, {1, 1, 0}, {1, 0, 1},
    {0, 2, 0}, {0, 1, 1}, {0, 0, 2}, {3, 0, 0}, {2, 1, 0}, {2, 0, 1}, {1, 2, 0},
    {1, 1, 1}, {1, 0, 2}, {0, 3, 0}, {0, 2, 1}, {0, 1, 2}, {0, 0, 3}};

double ipow(double x, int e) {
  double r = 1;
  for (int i = 0; i < e; ++i) r *= x;
  return r;
}

// d^alpha T_j at offset d, alpha = exponents of monomial a
double taylor_derivative(int j, int a, const double *d) {
  double f = 1;
  for (int e = 0; e < 3; ++e) {
    int ej = kTaylorExp[j][e], ea = kTaylorExp[a][e];
    if (ej < ea) return 0;
    double fall = 1;
    for (int i = 0; i < ea; ++i) fall *= (ej - i);
    f *= fall * ipow(d[e], ej - ea);
  }
  return f;
}

struct CellBasis {
  double center[3];
  double s[20 * 20];  // psi_m = sum_j s[m][j] T_j(x - center), lower triangular
};

void basis_values(const CellBasis &b, int M, const double *x, double *psi) {
  double d[3] = {x[0] - b.center[0], x[1] - b.center[1], x[2] - b.center[2]};
  double t[20];
  for (int j = 0; j < M; ++j) t[j] = taylor_derivative(j, 0, d);
  for (int m = 0; m < M; ++m) {
    double s = 0;
    for (int j = 0; j <= m; ++j) s += b.s[m * M + j] * t[j];
    psi[m] = s;
  }
}

int build_limiter(mcfd_handle *h, const mcfd_mesh_desc *d, int kind, double w0,
                  double eps) {
  auto &m = h->mesh;
  auto &l = h->lim;
  const int Q = m.q, N = m.n, p = m.p;
  const int M = (p + 1) * (p + 2) * (p + 3) / 6;
  const int64_t S = d->cell_node_stride > 0 ? d->cell_node_stride : 8;
  if (d->cell_type)
    for (int64_t c = 0; c < d->n_cells; ++c)
      if (d->cell_type[c] != MCFD_HEX8)
        return fail(h, MCFD_ERR_UNSUPPORTED, "the WENO limiter takes Hex8 cells only");
  l.kind = kind;
  l.m = M;
  l.w0 = w0 > 0 ? w0 : 0.001;
  l.eps = eps > 0 ? eps : 1e-6;
  const int64_t C = d->n_cells;
  double xq[4], wq[4];
  gll(Q, xq, wq);
  // adjacency in face order with periodic shifts (a point x of the cell is
  // x - shift in the neighbour's frame)
  std::vector<int32_t> adj((size_t)C * 6, -1);
  std::vector<double> adj_shift((size_t)C * 6 * 3, 0.0);
  std::vector<double> adj_frame((size_t)C * 6 * 9, 0.0);
  std::vector<int> n_adj(C, 0);
  for (int64_t f = 0; f < d->n_faces; ++f) {
    int64_t hc = d->face_cells[f * 2], sc = d->face_cells[f * 2 + 1];
    if (sc < 0) continue;
    double sh[3] = {0, 0, 0};
    if (d->face_shift)
      for (int e = 0; e < 3; ++e) sh[e] = d->face_shift[f * 3 + e];
    // frame of the face at its first GLL point, local (-1, -1) on the
    // holder's face (coordinate/face.hpp:54-62): normal, tangent, bitangent
    double xn[12], x[3], ta[3], tb[3], fr[9];
    const int side = d->face_sides[f * 2];
    for (int v = 0; v < 4; ++v)
      for (int e = 0; e < 3; ++e) xn[v * 3 + e] = d->xyz[d->cell_nodes[hc * S + kHexFace[side][v]] * 3 + e];
    quad4_point(xn, -1.0, -1.0, x, ta, tb);
    fr[0] = ta[1] * tb[2] - ta[2] * tb[1];
    fr[1] = ta[2] * tb[0] - ta[0] * tb[2];
    fr[2] = ta[0] * tb[1] - ta[1] * tb[0];
    const double nn = std::sqrt(fr[0] * fr[0] + fr[1] * fr[1] + fr[2] * fr[2]);
    const double tn = std::sqrt(ta[0] * ta[0] + ta[1] * ta[1] + ta[2] * ta[2]);
    for (int e = 0; e < 3; ++e) { fr[e] /= nn; fr[3 + e] = ta[e] / tn; }
    fr[6] = fr[1] * fr[5] - fr[2] * fr[4];
    fr[7] = fr[2] * fr[3] - fr[0] * fr[5];
    fr[8] = fr[0] * fr[4] - fr[1] * fr[3];
    if (n_adj[hc] < 6) {
      for (int e = 0; e < 3; ++e) adj_shift[((size_t)hc * 6 + n_adj[hc]) * 3 + e] = sh[e];
      for (int e = 0; e < 9; ++e) adj_frame[((size_t)hc * 6 + n_adj[hc]) * 9 + e] = fr[e];
      adj[(size_t)hc * 6 + n_adj[hc]++] = (int32_t)sc;
    }
    if (n_adj[sc] < 6) {
      for (int e = 0; e < 3; ++e) adj_shift[((size_t)sc * 6 + n_adj[sc]) * 3 + e] = -sh[e];
      for (int e = 0; e < 9; ++e) adj_frame[((size_t)sc * 6 + n_adj[sc]) * 9 + e] = fr[e];
      adj[(size_t)sc * 6 + n_adj[sc]++] = (int32_t)hc;
    }
  }
  std::vector<CellBasis> basis(C);
  std::vector<double> node_x((size_t)C * N * 3), node_w((size_t)C * N), volume(C);
  std::vector<double> psi((size_t)C * N * M), mn((size_t)C * N * M);
  std::vector<double> beta((size_t)C * M * M), s00(C), divisor(C);
  int bad = 0;
#pragma omp parallel for schedule(static)
  for (int64_t c = 0; c < C; ++c) {
    double xn[24], J[9];
    for (int v = 0; v < 8; ++v)
      for (int e = 0; e < 3; ++e) xn[v * 3 + e] = d->xyz[d->cell_nodes[c * S + v] * 3 + e];
    CellBasis &b = basis[c];
    hex8_point(xn, 0, 0, 0, b.center, J);
    double vol = 0;
    for (int i = 0; i < Q; ++i)
      for (int j = 0; j < Q; ++j)
        for (int k = 0; k < Q; ++k) {
          int q = (i * Q + j) * Q + k;
          double *x = &node_x[((size_t)c * N + q) * 3];
          hex8_point(xn, xq[i], xq[j], xq[k], x, J);
          double det = J[0] * (J[4] * J[8] - J[5] * J[7]) - J[1] * (J[3] * J[8] - J[5] * J[6]) +
                       J[2] * (J[3] * J[7] - J[4] * J[6]);
          node_w[(size_t)c * N + q] = wq[i] * wq[j] * wq[k] * det;
          vol += node_w[(size_t)c * N + q];
        }
    volume[c] = vol;
    // Gram matrix of the monomials and its Cholesky factor L (A = L L^T)
    std::vector<double> T((size_t)N * M), A((size_t)M * M, 0.0), L((size_t)M * M, 0.0);
    for (int q = 0; q < N; ++q) {
      const double *x = &node_x[((size_t)c * N + q) * 3];
      double dd[3] = {x[0] - b.center[0], x[1] - b.center[1], x[2] - b.center[2]};
      for (int j = 0; j < M; ++j) T[q * M + j] = taylor_derivative(j, 0, dd);
    }
    for (int i = 0; i < M; ++i)
      for (int j = 0; j < M; ++j) {
        double s = 0;
        for (int q = 0; q < N; ++q) s += node_w[(size_t)c * N + q] * T[q * M + i] * T[q * M + j];
        A[i * M + j] = s;
      }
    for (int i = 0; i < M; ++i) {
      for (int j = 0; j <= i; ++j) {
        double s = A[i * M + j];
        for (int k = 0; k < j; ++k) s -= L[i * M + k] * L[j * M + k];
        if (i == j) {
          if (!(s > 0)) { bad = 1; s = 1; }
          L[i * M + i] = std::sqrt(s);
        } else {
          L[i * M + j] = s / L[j * M + j];
        }
      }
    }
    // S = L^-1 (lower triangular, forward substitution per column)
    for (int i = 0; i < M * M; ++i) b.s[i] = 0;
    for (int col = 0; col < M; ++col) {
      for (int i = col; i < M; ++i) {
        double s = (i == col) ? 1.0 : 0.0;
        for (int k = col; k < i; ++k) s -= L[i * M + k] * b.s[k * M + col];
        b.s[i * M + col] = s / L[i * M + i];
      }
    }
    s00[c] = b.s[0];
    for (int q = 0; q < N; ++q) {
      double *pq = &psi[((size_t)c * N + q) * M];
      basis_values(b, M, &node_x[((size_t)c * N + q) * 3], pq);
      for (int mm = 0; mm < M; ++mm) mn[((size_t)c * N + q) * M + mm] = node_w[(size_t)c * N + q] * pq[mm];
    }
    // smoothness quadratic form: sum over derivative multi-indices a (|a| >= 1)
    // of weight(|a|) * integral of d^a psi_m d^a psi_m' (limiter/weno.hpp:25-95)
    double measure = 1 / (b.s[0] * b.s[0]);
    double weight[4] = {0, 0, 0, 0};
    for (int deg = 1; deg <= p; ++deg) {
      double kf = std::tgamma(deg + 1);
      weight[deg] = std::pow(measure, deg * 2. / 3 - 1) / (kf * kf);
    }
    double *B = &beta[(size_t)c * M * M];
    for (int i = 0; i < M * M; ++i) B[i] = 0;
    std::vector<double> dpsi(M);
    for (int q = 0; q < N; ++q) {
      const double *x = &node_x[((size_t)c * N + q) * 3];
      double dd[3] = {x[0] - b.center[0], x[1] - b.center[1], x[2] - b.center[2]};
      double wgt = node_w[(size_t)c * N + q];
      for (int a = 1; a < M; ++a) {
        int deg = kTaylorExp[a][0] + kTaylorExp[a][1] + kTaylorExp[a][2];
        for (int mm = 0; mm < M; ++mm) {
          double s = 0;
          for (int j = 0; j <= mm; ++j) s += b.s[mm * M + j] * taylor_derivative(j, a, dd);
          dpsi[mm] = s;
        }
        for (int i = 0; i < M; ++i)
          for (int j = 0; j < M; ++j) B[i * M + j] += wgt * weight[deg] * dpsi[i] * dpsi[j];
      }
    }
    divisor[c] = std::pow(vol, (p + 1.0) / 2.0 / 3) * n_adj[c];
  }
  if (bad) return fail(h, MCFD_ERR_MESH, "degenerate cell: modal basis Gram matrix not positive definite");
  // neighbour projections and basis values at the cell centre
  std::vector<double> proj((size_t)C * 6 * M * M, 0.0), eval((size_t)C * 7 * M, 0.0);
#pragma omp parallel for schedule(static)
  for (int64_t c = 0; c < C; ++c) {
    std::vector<double> pb(M);
    for (int s = 0; s < 6; ++s) {
      int32_t nb = adj[(size_t)c * 6 + s];
      if (nb < 0) continue;
      const double *sh = &adj_shift[((size_t)c * 6 + s) * 3];
      double *P = &proj[(((size_t)c * 6 + s) * M) * M];
      for (int q = 0; q < N; ++q) {
        const double *x = &node_x[((size_t)c * N + q) * 3];
        double xs[3] = {x[0] - sh[0], x[1] - sh[1], x[2] - sh[2]};
        basis_values(basis[nb], M, xs, pb.data());
        const double *mq = &mn[((size_t)c * N + q) * M];
        for (int i = 0; i < M; ++i)
          for (int j = 0; j < M; ++j) P[i * M + j] += pb[i] * mq[j];
      }
      double xc[3] = {basis[c].center[0] - sh[0], basis[c].center[1] - sh[1], basis[c].center[2] - sh[2]};
      basis_values(basis[nb], M, xc, &eval[((size_t)c * 7 + s) * M]);
    }
    basis_values(basis[c], M, basis[c].center, &eval[((size_t)c * 7 + 6) * M]);
  }
  int rc;
  if ((rc = upload(h, &l.psi, psi))) return rc;
  if ((rc = upload(h, &l.mn, mn))) return rc;
  if (h->opt.precision == MCFD_MIXED) {  // the mixed form's nodal -> modal map in FP32
    std::vector<float> mn32(mn.size());
    for (size_t i = 0; i < mn.size(); ++i) mn32[i] = (float)mn[i];
    if ((rc = upload(h, &l.mn32, mn32))) return rc;
  }
  if ((rc = upload(h, &l.proj, proj))) return rc;
  if ((rc = upload(h, &l.beta, beta))) return rc;
  if ((rc = upload(h, &l.eval, eval))) return rc;
  if ((rc = upload(h, &l.s00, s00))) return rc;
  if ((rc = upload(h, &l.divisor, divisor))) return rc;
  if ((rc = upload(h, &l.adj, adj))) return rc;
  if ((rc = upload(h, &l.frame, adj_frame))) return rc;
  if ((rc = upload(h, &l.volume, volume))) return rc;
  CUDA_TRY(h, cudaMalloc(&l.modal, sizeof(double) * C * mcfd::kK * M));
  CUDA_TRY(h, cudaMalloc(&l.list, sizeof(int32_t) * C));
  if (h->opt.shock_fp64) {
    const int cpb = Q == 4 ? 4 : (Q == 3 ? 9 : 32);  // CellCfg<Q>::kCells of the cell kernels
    l.n_blocks = (C + cpb - 1) / cpb;
    CUDA_TRY(h, cudaMalloc(&l.cell_hot, C));
    CUDA_TRY(h, cudaMalloc(&l.cell_hot2, C));
    CUDA_TRY(h, cudaMalloc(&l.block_hot, l.n_blocks));
    CUDA_TRY(h, cudaMemset(l.cell_hot, 0, C));
    CUDA_TRY(h, cudaMemset(l.block_hot, 0, l.n_blocks));
  }
  CUDA_TRY(h, cudaMalloc(&l.list_count, sizeof(unsigned)));
  CUDA_TRY(h, cudaMalloc(&l.troubled, sizeof(unsigned long long)));
  CUDA_TRY(h, cudaMemset(l.troubled, 0, sizeof(unsigned long long)));
  return MCFD_OK;
}

}  // namespace

extern "C" {

int mcfd_abi_version(void) { return MCFD_ABI_VERSION; }

const char *mcfd_last_error(const mcfd_handle *h) {
  return h ? h->err.c_str() : g_create_error.c_str();
}

int mcfd_create(const mcfd_mesh_desc *mesh, const mcfd_options *options,
                mcfd_handle **out) {
  mcfd::NvtxRange nvtx_range("mcfd_create");
  g_create_error.clear();
  if (!mesh || !options || !out) return fail(nullptr, MCFD_ERR_ARGUMENT, "null argument");
  *out = nullptr;
  if (mesh->n_cells <= 0 || mesh->n_nodes <= 0 || !mesh->xyz || !mesh->cell_nodes ||
      (mesh->n_faces > 0 && (!mesh->face_cells || !mesh->face_sides)))
    return fail(nullptr, MCFD_ERR_ARGUMENT, "incomplete mesh description");
  if (options->degree < 1 || options->degree > 3)
    return fail(nullptr, MCFD_ERR_UNSUPPORTED, "degree must be 1, 2 or 3");
  if (options->scheme != MCFD_DGSEM && options->scheme != MCFD_FR && options->scheme != MCFD_MODAL)
    return fail(nullptr, MCFD_ERR_UNSUPPORTED, "unknown scheme");
  if (options->riemann < MCFD_EXACT || options->riemann > MCFD_RUSANOV)
    return fail(nullptr, MCFD_ERR_ARGUMENT, "unknown Riemann solver");
  if (options->precision != MCFD_FP64 && options->precision != MCFD_MIXED)
    return fail(nullptr, MCFD_ERR_UNSUPPORTED, "unknown precision form");
  if (options->shock_cells_fp64 &&
      (options->precision != MCFD_MIXED || options->scheme == MCFD_MODAL ||
       options->limiter == MCFD_LIMITER_NONE))
    return fail(nullptr, MCFD_ERR_UNSUPPORTED,
                "FP64 shock cells need the mixed form, a nodal scheme and a WENO limiter");
  if (options->contraction != MCFD_CONTRACTION_SIMT &&
      (options->contraction != MCFD_CONTRACTION_TENSOR || options->precision != MCFD_MIXED ||
       options->scheme != MCFD_DGSEM || options->degree != 3))
    return fail(nullptr, MCFD_ERR_UNSUPPORTED,
                "the tensor-core contraction is built for the mixed DGSEM form at p = 3");
  int n_dev = 0;
  if (cudaGetDeviceCount(&n_dev) != cudaSuccess || n_dev <= options->device || options->device < 0)
    return fail(nullptr, MCFD_ERR_NO_DEVICE, "no CUDA device available");
  cudaDeviceProp prop;
  if (cudaGetDeviceProperties(&prop, options->device) != cudaSuccess || prop.major < 10)
    return fail(nullptr, MCFD_ERR_NO_DEVICE, "device is not a Blackwell-class GPU");
  mcfd_handle *h = new (std::nothrow) mcfd_handle();
  if (!h) return fail(nullptr, MCFD_ERR_ARGUMENT, "out of host memory");
  h->device = options->device;
  h->opt.riemann = options->riemann;
  h->opt.precision = options->precision;
  h->opt.cfl = options->cfl;
  h->opt.scheme = options->scheme;
  h->opt.fr_g1 = fr_correction_slope(options->degree);
  h->opt.tensor_contraction = options->contraction == MCFD_CONTRACTION_TENSOR;
  h->opt.shock_fp64 = options->shock_cells_fp64 > 0 ? std::min(options->shock_cells_fp64, 2) : 0;
  int rc = MCFD_OK;
  if (cudaSetDevice(h->device) != cudaSuccess) rc = fail(h, MCFD_ERR_CUDA, "cudaSetDevice failed");
  if (!rc && cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking) != cudaSuccess)
    rc = fail(h, MCFD_ERR_CUDA, "cudaStreamCreate failed");
  h->own_stream = true;
  h->modal.keep_host = options->scheme == MCFD_MODAL && options->limiter != MCFD_LIMITER_NONE;
  if (!rc)
    rc = options->scheme == MCFD_MODAL ? mcfd::build_modal_mesh(h, mesh, options->degree)
                                       : build_mesh(h, mesh, options->degree);
  if (!rc) rc = upload_corners(h, mesh);
  if (!rc && options->limiter != MCFD_LIMITER_NONE) {
    if (options->limiter != MCFD_LIMITER_LAZY && options->limiter != MCFD_LIMITER_DETECT_LAZY &&
        options->limiter != MCFD_LIMITER_EIGEN)
      rc = fail(h, MCFD_ERR_ARGUMENT, "unknown limiter");
    else if (options->scheme == MCFD_MODAL)
      rc = mcfd::build_modal_limiter(h, mesh, options->limiter, options->weno_w0, options->weno_eps);
    else
      rc = build_limiter(h, mesh, options->limiter, options->weno_w0, options->weno_eps);
  }
  if (!rc) {
    size_t col = sizeof(double) * h->mesh.column;
    cudaError_t e = cudaMalloc(&h->buf.u, col);
    if (e == cudaSuccess) e = cudaMalloc(&h->buf.u1, col);
    if (e == cudaSuccess) e = cudaMalloc(&h->buf.u2, col);
    if (e == cudaSuccess) e = cudaMalloc(&h->buf.res, col);
    if (e == cudaSuccess) e = cudaMalloc(&h->buf.flux, sizeof(double) * mcfd::kK * std::max<int64_t>(h->mesh.n_points, 1));
    if (e == cudaSuccess) e = cudaMalloc(&h->buf.state, sizeof(mcfd::DevState));
    if (e == cudaSuccess) e = cudaMemset(h->buf.u, 0, col);
    if (e == cudaSuccess) e = cudaMemset(h->buf.state, 0, sizeof(mcfd::DevState));
    // node traces for the Rusanov, Roe and HLLC face fluxes of the nodal
    // schemes (the limiter rewrites the traces of the cells it reconstructs)
    h->use_trace = options->scheme != MCFD_MODAL &&
                   (options->riemann == MCFD_RUSANOV || options->riemann == MCFD_ROE ||
                    options->riemann == MCFD_HLLC);
    if (e == cudaSuccess && h->use_trace)
      e = cudaMalloc(&h->buf.trace, sizeof(double) * 3 * h->mesh.n_cells * h->mesh.n);
    if (e == cudaSuccess && options->scheme != MCFD_MODAL && options->precision != MCFD_MIXED)
      e = cudaMalloc(&h->buf.dt_hi, sizeof(unsigned) * ((h->mesh.n_cells * h->mesh.n + 127) / 128));
    if (e != cudaSuccess) rc = cuda_fail(h, e, "device allocation");
  }
  if (rc) {
    g_create_error = h->err;
    release(h);
    delete h;
    return rc;
  }
  *out = h;
  return MCFD_OK;
}

int mcfd_destroy(mcfd_handle *h) {
  if (!h) return MCFD_ERR_ARGUMENT;
  cudaSetDevice(h->device);
  if (h->stream) cudaStreamSynchronize(h->stream);
  release(h);
  delete h;
  return MCFD_OK;
}

int64_t mcfd_column_size(const mcfd_handle *h) { return h ? h->mesh.column : -1; }

int mcfd_set_bc(mcfd_handle *h, int32_t group, const mcfd_bc_state *s) {
  if (!h || !s) return MCFD_ERR_ARGUMENT;
  if (group < 0 || group >= h->mesh.n_groups)
    return fail(h, MCFD_ERR_ARGUMENT, "boundary group out of range");
  if (s->kind == MCFD_BC_NO_SLIP_WALL && h->opt.scheme != MCFD_FR)
    return fail(h, MCFD_ERR_UNSUPPORTED, "no-slip walls run on the fr::Lobatto scheme only");
  if (s->kind < MCFD_BC_NONE || s->kind > MCFD_BC_NO_SLIP_WALL ||
      s->program < MCFD_STATE_CONSTANT || s->program > MCFD_STATE_TABLE || s->axis < 0 || s->axis > 2)
    return fail(h, MCFD_ERR_ARGUMENT, "bad boundary description");
  BcDev bc{};
  bc.kind = s->kind;
  bc.program = s->program;
  bc.axis = s->axis;
  bc.position = s->position;
  bc.speed = s->speed;
  for (int k = 0; k < 5; ++k) { bc.a[k] = s->a[k]; bc.b[k] = s->b[k]; }
  for (int e = 0; e < 3; ++e) bc.normal[e] = s->normal[e];
  // a table registered earlier for this group stays until replaced
  if (s->program == MCFD_STATE_TABLE && (size_t)group < h->mesh.bc_tables.size())
    bc.table = h->mesh.bc_tables[group];
  h->mesh.host_bcs[group] = bc;
  cudaSetDevice(h->device);
  CUDA_TRY(h, cudaMemcpyAsync(h->mesh.bcs + group, &h->mesh.host_bcs[group], sizeof(BcDev),
                              cudaMemcpyHostToDevice, h->stream));
  CUDA_TRY(h, cudaStreamSynchronize(h->stream));
  return MCFD_OK;
}

// The face points of boundary group `group` (global point ids, in order).
static int group_points(const mcfd_handle *h, int32_t group, std::vector<int64_t> *gids,
                        std::vector<double> *xyz) {
  const auto &m = h->mesh;
  std::vector<int32_t> fg(m.n_faces);
  cudaSetDevice(h->device);
  if (m.n_faces && cudaMemcpy(fg.data(), m.face_group, sizeof(int32_t) * m.n_faces,
                              cudaMemcpyDeviceToHost) != cudaSuccess)
    return MCFD_ERR_CUDA;
  std::vector<int32_t> off(m.n_faces + 1);
  const bool modal = h->opt.scheme == MCFD_MODAL;
  if (modal) {
    if (cudaMemcpy(off.data(), h->modal.face_off, sizeof(int32_t) * (m.n_faces + 1), cudaMemcpyDeviceToHost) !=
        cudaSuccess)
      return MCFD_ERR_CUDA;
  } else {
    for (int64_t f = 0; f <= m.n_faces; ++f) off[f] = (int32_t)(f * m.qf);
  }
  gids->clear();
  for (int64_t f = 0; f < m.n_faces; ++f)
    if (fg[f] == group)
      for (int32_t q = off[f]; q < off[f + 1]; ++q) gids->push_back(q);
  if (!xyz) return MCFD_OK;
  xyz->assign(gids->size() * 3, 0.0);
  if (modal) {
    std::vector<double4> fpt(m.n_points);
    if (m.n_points && cudaMemcpy(fpt.data(), h->modal.fpt, sizeof(double4) * m.n_points,
                                 cudaMemcpyDeviceToHost) != cudaSuccess)
      return MCFD_ERR_CUDA;
    for (size_t i = 0; i < gids->size(); ++i) {
      const double4 x = fpt[(*gids)[i]];
      (*xyz)[i * 3] = x.x; (*xyz)[i * 3 + 1] = x.y; (*xyz)[i * 3 + 2] = x.z;
    }
  } else {
    std::vector<double> fx(m.n_points * 3);
    if (m.n_points && cudaMemcpy(fx.data(), m.face_xyz, sizeof(double) * 3 * m.n_points,
                                 cudaMemcpyDeviceToHost) != cudaSuccess)
      return MCFD_ERR_CUDA;
    for (size_t i = 0; i < gids->size(); ++i)
      for (int e = 0; e < 3; ++e) (*xyz)[i * 3 + e] = fx[(*gids)[i] * 3 + e];
  }
  return MCFD_OK;
}

int mcfd_bc_point_count(const mcfd_handle *h, int32_t group, int64_t *n) {
  if (!h || !n || group < 0 || group >= h->mesh.n_groups) return MCFD_ERR_ARGUMENT;
  std::vector<int64_t> gids;
  int rc = group_points(h, group, &gids, nullptr);
  if (rc) return rc;
  *n = (int64_t)gids.size();
  return MCFD_OK;
}

int mcfd_bc_points(const mcfd_handle *h, int32_t group, double *xyz, int64_t n) {
  if (!h || !xyz || group < 0 || group >= h->mesh.n_groups) return MCFD_ERR_ARGUMENT;
  std::vector<int64_t> gids;
  std::vector<double> pts;
  int rc = group_points(h, group, &gids, &pts);
  if (rc) return rc;
  if ((int64_t)gids.size() != n) return MCFD_ERR_ARGUMENT;
  std::copy(pts.begin(), pts.end(), xyz);
  return MCFD_OK;
}

int mcfd_set_bc_table(mcfd_handle *h, int32_t group, const double *values, int64_t n) {
  if (!h || !values) return MCFD_ERR_ARGUMENT;
  if (group < 0 || group >= h->mesh.n_groups) return fail(h, MCFD_ERR_ARGUMENT, "boundary group out of range");
  auto &m = h->mesh;
  if (m.host_bcs[group].program != MCFD_STATE_TABLE)
    return fail(h, MCFD_ERR_ARGUMENT, "the group's state program is not MCFD_STATE_TABLE");
  std::vector<int64_t> gids;
  int rc = group_points(h, group, &gids, nullptr);
  if (rc) return fail(h, rc, "reading the face table");
  if ((int64_t)gids.size() != n) return fail(h, MCFD_ERR_ARGUMENT, "table size != the group's face points");
  for (int64_t i = 0; i < n * mcfd::kK; ++i)
    if (!std::isfinite(values[i])) return fail(h, MCFD_ERR_ARGUMENT, "non-finite boundary table value");
  cudaSetDevice(h->device);
  if (m.bc_tables.size() < (size_t)m.n_groups) m.bc_tables.resize(m.n_groups, nullptr);
  if (!m.bc_row) {
    CUDA_TRY(h, cudaMalloc(&m.bc_row, sizeof(int32_t) * std::max<int64_t>(m.n_points, 1)));
    m.host_bc_row.assign(std::max<int64_t>(m.n_points, 1), -1);
  }
  for (int64_t i = 0; i < n; ++i) m.host_bc_row[gids[i]] = (int32_t)i;
  CUDA_TRY(h, cudaMemcpy(m.bc_row, m.host_bc_row.data(), sizeof(int32_t) * m.host_bc_row.size(),
                         cudaMemcpyHostToDevice));
  if (m.bc_tables[group]) {
    cudaFree(m.bc_tables[group]);
    m.bc_tables[group] = nullptr;
  }
  CUDA_TRY(h, cudaMalloc(&m.bc_tables[group], sizeof(double) * mcfd::kK * std::max<int64_t>(n, 1)));
  CUDA_TRY(h, cudaMemcpy(m.bc_tables[group], values, sizeof(double) * mcfd::kK * n, cudaMemcpyHostToDevice));
  m.host_bcs[group].table = m.bc_tables[group];
  CUDA_TRY(h, cudaMemcpy(m.bcs + group, &m.host_bcs[group], sizeof(BcDev), cudaMemcpyHostToDevice));
  // captured step graphs hold the old bc_row pointer only if it changed: recapture
  mcfd::drop_graphs(h);
  return MCFD_OK;
}

int mcfd_set_time(mcfd_handle *h, double t) {
  if (!h) return MCFD_ERR_ARGUMENT;
  h->t_host = t;
  return MCFD_OK;
}

static int copy_column(mcfd_handle *h, void *dst, const void *src, int64_t n,
                       cudaMemcpyKind kind) {
  if (!h || !dst || !src) return MCFD_ERR_ARGUMENT;
  if (n != h->mesh.column) return fail(h, MCFD_ERR_ARGUMENT, "column size mismatch");
  mcfd::invalidate_trace(h, (const double *)dst);
  cudaSetDevice(h->device);
  CUDA_TRY(h, cudaMemcpyAsync(dst, src, sizeof(double) * n, kind, h->stream));
  CUDA_TRY(h, cudaStreamSynchronize(h->stream));
  return MCFD_OK;
}

// WithLimiter::SetSolutionColumn runs the limiter after setting the column
// (spatial/with_limiter.hpp:56-59).
static int limit_current(mcfd_handle *h) {
  if (h->lim.kind == MCFD_LIMITER_NONE) return MCFD_OK;
  h->launches += mcfd::launch_limiter(h, h->buf.u);
  CUDA_TRY(h, cudaGetLastError());
  CUDA_TRY(h, cudaStreamSynchronize(h->stream));
  return MCFD_OK;
}

int mcfd_set_solution(mcfd_handle *h, const double *column, int64_t n) {
  mcfd::NvtxRange nvtx_range("mcfd_set_solution");
  if (!h) return MCFD_ERR_ARGUMENT;
  int rc = copy_column(h, h->buf.u, column, n, cudaMemcpyHostToDevice);
  return rc ? rc : limit_current(h);
}

int mcfd_limit(mcfd_handle *h, int64_t *troubled) {
  mcfd::NvtxRange nvtx_range("mcfd_limit");
  if (!h) return MCFD_ERR_ARGUMENT;
  cudaSetDevice(h->device);
  int64_t before = 0, after = 0;
  if (h->lim.kind != MCFD_LIMITER_NONE) {
    CUDA_TRY(h, cudaMemcpy(&before, h->lim.troubled, sizeof(before), cudaMemcpyDeviceToHost));
    int rc = limit_current(h);
    if (rc) return rc;
    CUDA_TRY(h, cudaMemcpy(&after, h->lim.troubled, sizeof(after), cudaMemcpyDeviceToHost));
  }
  if (troubled) *troubled = after - before;
  return MCFD_OK;
}

int mcfd_set_viscosity(mcfd_handle *h, double ddg_beta0, double ddg_beta1, double time_scale) {
  if (!h) return MCFD_ERR_ARGUMENT;
  if (!std::isfinite(ddg_beta0) || !std::isfinite(ddg_beta1) || !std::isfinite(time_scale))
    return fail(h, MCFD_ERR_ARGUMENT, "viscosity parameters must be finite");
  if (h->opt.scheme != MCFD_FR)
    return fail(h, MCFD_ERR_UNSUPPORTED, "the artificial viscosity runs on the fr::Lobatto scheme (MCFD_FR)");
  if (h->opt.precision != MCFD_FP64)
    return fail(h, MCFD_ERR_UNSUPPORTED, "the artificial viscosity runs in the plain FP64 form");
  if (h->lim.kind != MCFD_LIMITER_NONE)
    return fail(h, MCFD_ERR_UNSUPPORTED, "a handle has either a limiter or the artificial viscosity");
  if (h->cases.n)
    return fail(h, MCFD_ERR_UNSUPPORTED, "the artificial viscosity takes a handle without cases");
  for (uint8_t t : h->mesh.host_cell_type)
    if (t != MCFD_HEX8) return fail(h, MCFD_ERR_UNSUPPORTED, "the artificial viscosity takes Hex8 cells");
  cudaSetDevice(h->device);
  CUDA_TRY(h, cudaStreamSynchronize(h->stream));
  const int rc = mcfd::build_viscosity(h, ddg_beta0, ddg_beta1, time_scale);
  if (rc) return fail(h, rc, h->err);
  // the viscous face kernel evaluates its own states: no Rusanov node traces
  h->use_trace = false;
  h->trace_for = nullptr;
  mcfd::drop_graphs(h);
  return MCFD_OK;
}

int mcfd_get_viscosity(mcfd_handle *h, double *nu, int64_t n) {
  if (!h || !nu) return MCFD_ERR_ARGUMENT;
  if (!h->visc.on) return fail(h, MCFD_ERR_ARGUMENT, "no artificial viscosity on this handle");
  if (n != h->mesh.n_cells * mcfd::kK) return fail(h, MCFD_ERR_ARGUMENT, "viscosity array length mismatch");
  cudaSetDevice(h->device);
  h->launches += mcfd::launch_visc_properties(h, h->buf.u, 0);
  CUDA_TRY(h, cudaMemcpyAsync(nu, h->visc.nu, sizeof(double) * n, cudaMemcpyDeviceToHost, h->stream));
  return check_status(h);
}

int mcfd_initial_limiter(mcfd_handle *h, int32_t kind) {
  if (!h) return MCFD_ERR_ARGUMENT;
  if (kind != MCFD_INIT_AVERAGE && kind != MCFD_INIT_MAJORITY)
    return fail(h, MCFD_ERR_ARGUMENT, "unknown initial limiter");
  if (h->opt.scheme == mcfd::kSchemeModal)
    return fail(h, MCFD_ERR_UNSUPPORTED, "the initial limiters take the nodal schemes");
  cudaSetDevice(h->device);
  auto &m = h->mesh;
  if (kind == MCFD_INIT_MAJORITY && m.p < 2) return MCFD_OK;
  if (kind == MCFD_INIT_AVERAGE && !m.node_w) {
    // global weights w_i w_j w_k det(J) of every node (integrator/element.hpp:102-115)
    const int Q = m.q, N = m.n;
    double xq[4], wq[4];
    gll(Q, xq, wq);
    std::vector<double> w((size_t)m.n_cells * N);
    for (int64_t c = 0; c < m.n_cells; ++c) {
      const int t = m.host_cell_type[c];
      for (int i = 0; i < Q; ++i)
        for (int j = 0; j < Q; ++j)
          for (int k = 0; k < Q; ++k) {
            double x[3], J[9];
            if (t == MCFD_HEX8) {
              hex8_point(&m.host_corners[c * 24], xq[i], xq[j], xq[k], x, J);
            } else {
              const double loc[3] = {xq[i], xq[j], xq[k]};
              mcfd::geo::map_point(t, &m.host_nodes[(size_t)c * mcfd::geo::kMaxNodes * 3], loc, x, J);
            }
            const double det = J[0] * (J[4] * J[8] - J[5] * J[7]) - J[1] * (J[3] * J[8] - J[5] * J[6]) +
                               J[2] * (J[3] * J[7] - J[4] * J[6]);
            w[(size_t)c * N + (i * Q + j) * Q + k] = wq[i] * wq[j] * wq[k] * det;
          }
    }
    int rc = upload(h, &m.node_w, w);
    if (rc) return rc;
  }
  unsigned long long *missing = nullptr, count = 0;
  CUDA_TRY(h, cudaMalloc(&missing, sizeof(unsigned long long)));
  cudaMemsetAsync(missing, 0, sizeof(unsigned long long), h->stream);
  h->launches += mcfd::launch_initial_limiter(h, kind, h->buf.u, missing);
  mcfd::invalidate_trace(h, h->buf.u);
  cudaMemcpyAsync(&count, missing, sizeof(count), cudaMemcpyDeviceToHost, h->stream);
  cudaError_t e = cudaStreamSynchronize(h->stream);
  cudaFree(missing);
  if (e != cudaSuccess) return cuda_fail(h, e, "initial limiter");
  if (count)
    return fail(h, MCFD_ERR_STATE, std::to_string(count) +
                " cells have a component without a strict majority value (left unchanged)");
  return check_status(h);
}

int mcfd_troubled_cells(mcfd_handle *h, int64_t *count) {
  if (!h || !count) return MCFD_ERR_ARGUMENT;
  *count = 0;
  if (h->lim.kind == MCFD_LIMITER_NONE) return MCFD_OK;
  cudaSetDevice(h->device);
  CUDA_TRY(h, cudaStreamSynchronize(h->stream));
  CUDA_TRY(h, cudaMemcpy(count, h->lim.troubled, sizeof(*count), cudaMemcpyDeviceToHost));
  CUDA_TRY(h, cudaMemset(h->lim.troubled, 0, sizeof(unsigned long long)));
  return MCFD_OK;
}

int mcfd_get_solution(mcfd_handle *h, double *column, int64_t n) {
  mcfd::NvtxRange nvtx_range("mcfd_get_solution");
  if (!h) return MCFD_ERR_ARGUMENT;
  return copy_column(h, column, h->buf.u, n, cudaMemcpyDeviceToHost);
}

int mcfd_set_solution_device(mcfd_handle *h, const double *d_column, int64_t n) {
  if (!h) return MCFD_ERR_ARGUMENT;
  int rc = copy_column(h, h->buf.u, d_column, n, cudaMemcpyDeviceToDevice);
  return rc ? rc : limit_current(h);
}

int mcfd_get_solution_device(mcfd_handle *h, double *d_column, int64_t n) {
  if (!h) return MCFD_ERR_ARGUMENT;
  return copy_column(h, d_column, h->buf.u, n, cudaMemcpyDeviceToDevice);
}

static int residual_into(mcfd_handle *h, double *dst, int64_t n, cudaMemcpyKind kind) {
  if (!h || !dst) return MCFD_ERR_ARGUMENT;
  if (n != h->mesh.column) return fail(h, MCFD_ERR_ARGUMENT, "column size mismatch");
  cudaSetDevice(h->device);
  h->launches += mcfd::launch_set_state(h, h->t_host, 0.0, 0.0, 0.0, 1);
  h->launches += mcfd::launch_face_flux(h, h->buf.u, 0.0);
  h->launches += mcfd::launch_cell_update(h, mcfd::kStageResidual, h->buf.u, nullptr, h->buf.res, 0);
  CUDA_TRY(h, cudaGetLastError());
  CUDA_TRY(h, cudaMemcpyAsync(dst, h->buf.res, sizeof(double) * n, kind, h->stream));
  return check_status(h);
}

int mcfd_residual(mcfd_handle *h, double *residual, int64_t n) {
  mcfd::NvtxRange nvtx_range("mcfd_residual");
  return residual_into(h, residual, n, cudaMemcpyDeviceToHost);
}

int mcfd_residual_device(mcfd_handle *h, double *d_residual, int64_t n) {
  mcfd::NvtxRange nvtx_range("mcfd_residual_device");
  return residual_into(h, d_residual, n, cudaMemcpyDeviceToDevice);
}

int mcfd_residual_device_noalloc(mcfd_handle *h, const double *d_u,
                                 double *d_residual, int64_t n) {
  if (!h || !d_u || !d_residual) return MCFD_ERR_ARGUMENT;
  if (n != h->mesh.column) return fail(h, MCFD_ERR_ARGUMENT, "column size mismatch");
  if (h->opt.scheme == MCFD_MODAL)
    return fail(h, MCFD_ERR_UNSUPPORTED, "the no-allocation residual covers the nodal schemes");
  if (h->visc.on)
    return fail(h, MCFD_ERR_UNSUPPORTED, "the no-allocation residual does not cover the artificial viscosity");
  if (h->mesh.n_points * mcfd::kK > mcfd::kStaticFluxCapacity)
    return fail(h, MCFD_ERR_ARGUMENT,
                "mesh too large for the no-allocation residual: " +
                    std::to_string(h->mesh.n_points) + " face points need " +
                    std::to_string(h->mesh.n_points * mcfd::kK) +
                    " scratch doubles, the static capacity is " +
                    std::to_string(mcfd::kStaticFluxCapacity) + " (16 MiB)");
  // the caller's current device is restored on return
  mcfd::DeviceGuard guard(h->device);
  CUDA_TRY(h, cudaGetLastError());
  double *scratch = nullptr;
  std::string why;
  if (mcfd::static_flux_scratch(h->device, &scratch, &why))
    return fail(h, MCFD_ERR_CUDA, why);
  h->launches += mcfd::launch_set_state(h, h->t_host, 0.0, 0.0, 0.0, 1);
  h->launches += mcfd::launch_residual_static_scratch(h, d_u, d_residual, scratch);
  CUDA_TRY(h, cudaGetLastError());
  return check_status(h);
}

int mcfd_time_step(mcfd_handle *h, double dt_guess, int32_t rk_order, double *dt) {
  mcfd::NvtxRange nvtx_range("mcfd_time_step");
  if (!h || !dt) return MCFD_ERR_ARGUMENT;
  cudaSetDevice(h->device);
  double cfl = h->opt.cfl > 0 ? h->opt.cfl : cfl_table(rk_order, h->mesh.p);
  h->launches += mcfd::launch_set_state(h, h->t_host, 0.0, dt_guess, cfl, 1);
  h->launches += mcfd::launch_dt(h, h->buf.u);
  CUDA_TRY(h, cudaGetLastError());
  mcfd::DevState st;
  CUDA_TRY(h, cudaMemcpyAsync(&st, h->buf.state, sizeof(st), cudaMemcpyDeviceToHost, h->stream));
  CUDA_TRY(h, cudaStreamSynchronize(h->stream));
  *dt = st.dt;
  return MCFD_OK;
}

int mcfd_rk_step(mcfd_handle *h, double t, double dt, int32_t order) {
  mcfd::NvtxRange nvtx_range("mcfd_rk_step");
  if (!h || order < 1 || order > 3) return h ? fail(h, MCFD_ERR_ARGUMENT, "order must be 1, 2 or 3") : MCFD_ERR_ARGUMENT;
  cudaSetDevice(h->device);
  h->launches += mcfd::launch_set_state(h, t, dt, dt, 0.0, 0);
  h->launches += mcfd::launch_set_cases(h, t, dt);
  h->launches += mcfd::launch_rk_stage_sequence(h, order);
  CUDA_TRY(h, cudaGetLastError());
  h->t_host = t + dt;
  return check_status(h);
}

// Capture (once per RK order) the CUDA graph of one step: dt + RK stages.
// The captured step reads the trace of u in its first stage and leaves the
// trace of the new u behind, so the trace is made current first.
static int ensure_step_graph(mcfd_handle *h, int32_t rk_order) {
  if (h->use_trace && h->trace_for != h->buf.u) h->launches += mcfd::launch_trace(h, h->buf.u);
  CUDA_TRY(h, cudaGetLastError());
  if (!h->step_graph || h->step_graph_order != rk_order) {
    if (h->step_graph) { cudaGraphExecDestroy(h->step_graph); h->step_graph = nullptr; }
    cudaGraph_t graph;
    CUDA_TRY(h, cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal));
    int n = mcfd::launch_dt(h, h->buf.u);
    n += mcfd::launch_rk_stage_sequence(h, rk_order, nullptr, nullptr, true);
    cudaError_t e = cudaStreamEndCapture(h->stream, &graph);
    if (e != cudaSuccess) return cuda_fail(h, e, "cudaStreamEndCapture");
    e = cudaGraphInstantiate(&h->step_graph, graph, 0);
    cudaGraphDestroy(graph);
    if (e != cudaSuccess) return cuda_fail(h, e, "cudaGraphInstantiate");
    h->step_graph_order = rk_order;
    h->step_graph_kernels = n;
  }
  return MCFD_OK;
}

// Capture the graph of one streamed job on staging slot b: the limiter on
// the loaded column (as mcfd_set_solution), its trace, then n_steps x (dt +
// RK stages), the first step reading in[b] and every step writing out[b].
static int ensure_job_graph(mcfd_handle *h, int b, int32_t n_steps, int32_t rk_order) {
  auto &st = h->streamer;
  if (st.graph[b] && st.graph_order[b] == rk_order && st.graph_steps[b] == n_steps) return MCFD_OK;
  if (st.graph[b]) { cudaGraphExecDestroy(st.graph[b]); st.graph[b] = nullptr; }
  cudaGraph_t graph;
  CUDA_TRY(h, cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal));
  int n = mcfd::launch_limiter(h, st.in[b]);
  n += mcfd::launch_trace(h, st.in[b]);
  for (int s = 0; s < n_steps; ++s) {
    const double *src = s == 0 ? st.in[b] : st.out[b];
    n += mcfd::launch_dt(h, src);
    n += mcfd::launch_rk_stage_sequence(h, rk_order, src, st.out[b], true);
  }
  cudaError_t e = cudaStreamEndCapture(h->stream, &graph);
  if (e != cudaSuccess) return cuda_fail(h, e, "cudaStreamEndCapture");
  e = cudaGraphInstantiate(&st.graph[b], graph, 0);
  cudaGraphDestroy(graph);
  if (e != cudaSuccess) return cuda_fail(h, e, "cudaGraphInstantiate");
  st.graph_order[b] = rk_order;
  st.graph_steps[b] = n_steps;
  st.graph_kernels[b] = n;
  return MCFD_OK;
}

int mcfd_advance(mcfd_handle *h, int32_t n_steps, double dt_guess, int32_t rk_order, double *t) {
  mcfd::NvtxRange nvtx_range("mcfd_advance");
  if (!h || !t || n_steps < 0 || rk_order < 1 || rk_order > 3) return MCFD_ERR_ARGUMENT;
  cudaSetDevice(h->device);
  double cfl = h->opt.cfl > 0 ? h->opt.cfl : cfl_table(rk_order, h->mesh.p);
  h->launches += mcfd::launch_set_state(h, *t, 0.0, dt_guess, cfl, 1);
  int grc = ensure_step_graph(h, rk_order);
  if (grc) return grc;
  for (int s = 0; s < n_steps; ++s) {
    CUDA_TRY(h, cudaGraphLaunch(h->step_graph, h->stream));
    h->launches += h->step_graph_kernels;
  }
  mcfd::DevState st;
  CUDA_TRY(h, cudaMemcpyAsync(&st, h->buf.state, sizeof(st), cudaMemcpyDeviceToHost, h->stream));
  int rc = check_status(h);
  *t = st.t;
  h->t_host = st.t;
  return rc;
}

int mcfd_stream_begin(mcfd_handle *h) {
  if (!h) return MCFD_ERR_ARGUMENT;
  if (h->streamer.on) return MCFD_OK;
  cudaSetDevice(h->device);
  auto &st = h->streamer;
  if (st.copy_out) {  // staging kept from an earlier stream
    st.on = true;
    st.k = 0;
    return MCFD_OK;
  }
  const size_t bytes = sizeof(double) * h->mesh.column;
  cudaError_t e = cudaSuccess;
  for (int b = 0; b < 2 && e == cudaSuccess; ++b) {
    e = cudaMalloc(&st.in[b], bytes);
    if (e == cudaSuccess) e = cudaMalloc(&st.out[b], bytes);
    cudaEvent_t *evs[] = {&st.in_ready[b], &st.in_free[b], &st.out_ready[b], &st.out_free[b]};
    for (cudaEvent_t *ev : evs)
      if (e == cudaSuccess) e = cudaEventCreateWithFlags(ev, cudaEventDisableTiming);
  }
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&st.copy_in, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&st.copy_out, cudaStreamNonBlocking);
  if (e != cudaSuccess) {
    stream_release(h);
    return cuda_fail(h, e, "stream set-up");
  }
  st.on = true;
  st.k = 0;
  return MCFD_OK;
}

int mcfd_stream_step(mcfd_handle *h, const double *host_in, double *host_out, int64_t n,
                     double t, int32_t n_steps, double dt_guess, int32_t rk_order) {
  mcfd::NvtxRange nvtx_range("mcfd_stream_step");
  if (!h || !host_in || !host_out || n_steps < 1 || rk_order < 1 || rk_order > 3)
    return MCFD_ERR_ARGUMENT;
  if (!h->streamer.on) return fail(h, MCFD_ERR_STATE, "mcfd_stream_begin first");
  if (n != h->mesh.column) return fail(h, MCFD_ERR_ARGUMENT, "column size mismatch");
  cudaSetDevice(h->device);
  auto &st = h->streamer;
  const int b = (int)(st.k & 1);
  const size_t bytes = sizeof(double) * n;
  // upload into in[b] once job k-2 has finished reading it
  CUDA_TRY(h, cudaStreamWaitEvent(st.copy_in, st.in_free[b], 0));
  CUDA_TRY(h, cudaMemcpyAsync(st.in[b], host_in, bytes, cudaMemcpyHostToDevice, st.copy_in));
  CUDA_TRY(h, cudaEventRecord(st.in_ready[b], st.copy_in));
  // compute in[b] -> out[b] once the upload has landed and the download of
  // job k-2 has left out[b]
  CUDA_TRY(h, cudaStreamWaitEvent(h->stream, st.in_ready[b], 0));
  CUDA_TRY(h, cudaStreamWaitEvent(h->stream, st.out_free[b], 0));
  double cfl = h->opt.cfl > 0 ? h->opt.cfl : cfl_table(rk_order, h->mesh.p);
  h->launches += mcfd::launch_set_state(h, t, 0.0, dt_guess, cfl, 1);
  int grc = ensure_job_graph(h, b, n_steps, rk_order);
  if (grc) return grc;
  CUDA_TRY(h, cudaGraphLaunch(st.graph[b], h->stream));
  h->launches += st.graph_kernels[b];
  h->trace_for = nullptr;  // the job overwrote the trace buffer
  CUDA_TRY(h, cudaEventRecord(st.in_free[b], h->stream));
  CUDA_TRY(h, cudaEventRecord(st.out_ready[b], h->stream));
  // download once the result is complete
  CUDA_TRY(h, cudaStreamWaitEvent(st.copy_out, st.out_ready[b], 0));
  CUDA_TRY(h, cudaMemcpyAsync(host_out, st.out[b], bytes, cudaMemcpyDeviceToHost, st.copy_out));
  CUDA_TRY(h, cudaEventRecord(st.out_free[b], st.copy_out));
  ++st.k;
  return MCFD_OK;
}

int mcfd_stream_end(mcfd_handle *h) {
  if (!h) return MCFD_ERR_ARGUMENT;
  if (!h->streamer.on) return MCFD_OK;
  cudaSetDevice(h->device);
  cudaError_t e = cudaStreamSynchronize(h->streamer.copy_in);
  if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(h->streamer.copy_out);
  h->streamer.on = false;  // staging buffers, streams and graphs stay for the next stream
  if (e != cudaSuccess) return cuda_fail(h, e, "stream end");
  return check_status(h);
}

}  // extern "C"

// Ensemble: several handles stepped by one CUDA graph per step.  The graph
// forks from the ensemble's stream to every member's stream, captures the
// member's dt reduction and RK stages there, and joins back, so members with
// different schemes or degrees run concurrently inside one replay.
struct mcfd_ensemble {
  std::vector<mcfd_handle *> members;
  int device = 0;
  cudaStream_t stream = nullptr;
  bool own_stream = true;
  cudaEvent_t fork = nullptr;
  std::vector<cudaEvent_t> join;
  cudaGraphExec_t graph = nullptr;
  int order = 0;
  std::vector<int> kernels;
  std::string err;
  // streamed stepping (mcfd_ensemble_stream_*): per member and slot b the
  // staged input / output columns; one copy stream per direction
  bool streaming = false;
  std::vector<double *> in[2], out[2];
  cudaStream_t copy_in = nullptr, copy_out = nullptr;
  cudaEvent_t in_ready[2] = {nullptr, nullptr}, in_free[2] = {nullptr, nullptr};
  cudaEvent_t out_ready[2] = {nullptr, nullptr}, out_free[2] = {nullptr, nullptr};
  int64_t k = 0;
};

namespace {

int ens_fail(mcfd_ensemble *e, int code, const std::string &msg) {
  if (e) e->err = msg; else g_create_error = msg;
  return code;
}

void ens_stream_release(mcfd_ensemble *e) {
  for (int b = 0; b < 2; ++b) {
    for (double *p : e->in[b]) if (p) cudaFree(p);
    for (double *p : e->out[b]) if (p) cudaFree(p);
    e->in[b].clear();
    e->out[b].clear();
    cudaEvent_t evs[] = {e->in_ready[b], e->in_free[b], e->out_ready[b], e->out_free[b]};
    for (cudaEvent_t ev : evs) if (ev) cudaEventDestroy(ev);
    e->in_ready[b] = e->in_free[b] = e->out_ready[b] = e->out_free[b] = nullptr;
  }
  if (e->copy_in) cudaStreamDestroy(e->copy_in);
  if (e->copy_out) cudaStreamDestroy(e->copy_out);
  e->copy_in = e->copy_out = nullptr;
  e->streaming = false;
}

// Capture (once per RK order) the fork/join graph of one ensemble step.
int ens_ensure_graph(mcfd_ensemble *e, int32_t rk_order) {
  if (e->graph && e->order == rk_order) return MCFD_OK;
  if (e->graph) { cudaGraphExecDestroy(e->graph); e->graph = nullptr; }
  e->kernels.assign(e->members.size(), 0);
  cudaGraph_t graph;
  cudaError_t err = cudaStreamBeginCapture(e->stream, cudaStreamCaptureModeThreadLocal);
  if (err == cudaSuccess) err = cudaEventRecord(e->fork, e->stream);
  for (size_t i = 0; i < e->members.size() && err == cudaSuccess; ++i) {
    mcfd_handle *h = e->members[i];
    err = cudaStreamWaitEvent(h->stream, e->fork, 0);
    if (err != cudaSuccess) break;
    int k = mcfd::launch_dt(h, h->buf.u);
    k += mcfd::launch_rk_stage_sequence(h, rk_order, nullptr, nullptr, true);
    e->kernels[i] = k;
    err = cudaEventRecord(e->join[i], h->stream);
    if (err == cudaSuccess) err = cudaStreamWaitEvent(e->stream, e->join[i], 0);
  }
  cudaError_t end = cudaStreamEndCapture(e->stream, &graph);
  if (err == cudaSuccess) err = end;
  if (err != cudaSuccess) return ens_fail(e, MCFD_ERR_CUDA, std::string("ensemble capture: ") + cudaGetErrorString(err));
  err = cudaGraphInstantiate(&e->graph, graph, 0);
  cudaGraphDestroy(graph);
  if (err != cudaSuccess) return ens_fail(e, MCFD_ERR_CUDA, std::string("ensemble graph: ") + cudaGetErrorString(err));
  e->order = rk_order;
  return MCFD_OK;
}

void ens_release(mcfd_ensemble *e) {
  ens_stream_release(e);
  if (e->graph) cudaGraphExecDestroy(e->graph);
  for (cudaEvent_t ev : e->join)
    if (ev) cudaEventDestroy(ev);
  if (e->fork) cudaEventDestroy(e->fork);
  if (e->stream && e->own_stream) cudaStreamDestroy(e->stream);
}

}  // namespace

extern "C" {

int mcfd_ensemble_create(mcfd_handle *const *handles, int32_t n, mcfd_ensemble **out) {
  g_create_error.clear();
  if (!handles || !out || n < 1) return ens_fail(nullptr, MCFD_ERR_ARGUMENT, "null or empty member list");
  *out = nullptr;
  for (int32_t i = 0; i < n; ++i) {
    if (!handles[i]) return ens_fail(nullptr, MCFD_ERR_ARGUMENT, "null member");
    if (handles[i]->device != handles[0]->device)
      return ens_fail(nullptr, MCFD_ERR_ARGUMENT, "ensemble members must share one device");
    for (int32_t j = 0; j < i; ++j)
      if (handles[j] == handles[i]) return ens_fail(nullptr, MCFD_ERR_ARGUMENT, "a handle appears twice");
  }
  mcfd_ensemble *e = new (std::nothrow) mcfd_ensemble();
  if (!e) return ens_fail(nullptr, MCFD_ERR_ARGUMENT, "out of host memory");
  e->members.assign(handles, handles + n);
  e->device = handles[0]->device;
  e->join.assign(n, nullptr);
  cudaError_t err = cudaSetDevice(e->device);
  if (err == cudaSuccess) err = cudaStreamCreateWithFlags(&e->stream, cudaStreamNonBlocking);
  if (err == cudaSuccess) err = cudaEventCreateWithFlags(&e->fork, cudaEventDisableTiming);
  for (int32_t i = 0; i < n && err == cudaSuccess; ++i)
    err = cudaEventCreateWithFlags(&e->join[i], cudaEventDisableTiming);
  if (err != cudaSuccess) {
    g_create_error = std::string("ensemble set-up: ") + cudaGetErrorString(err);
    ens_release(e);
    delete e;
    return MCFD_ERR_CUDA;
  }
  *out = e;
  return MCFD_OK;
}

int mcfd_ensemble_destroy(mcfd_ensemble *e) {
  if (!e) return MCFD_ERR_ARGUMENT;
  cudaSetDevice(e->device);
  if (e->stream) cudaStreamSynchronize(e->stream);
  ens_release(e);
  delete e;
  return MCFD_OK;
}

int mcfd_ensemble_set_stream(mcfd_ensemble *e, void *cuda_stream) {
  if (!e || !cuda_stream) return MCFD_ERR_ARGUMENT;
  cudaSetDevice(e->device);
  cudaError_t err = cudaStreamSynchronize(e->stream);
  if (err != cudaSuccess) return ens_fail(e, MCFD_ERR_CUDA, cudaGetErrorString(err));
  cudaStreamDestroy(e->stream);
  e->stream = (cudaStream_t)cuda_stream;
  e->own_stream = false;
  return MCFD_OK;
}

const char *mcfd_ensemble_last_error(const mcfd_ensemble *e) {
  return e ? e->err.c_str() : g_create_error.c_str();
}

int mcfd_ensemble_advance(mcfd_ensemble *e, int32_t n_steps, double dt_guess, int32_t rk_order) {
  mcfd::NvtxRange nvtx_range("mcfd_ensemble_advance");
  if (!e || n_steps < 0 || rk_order < 1 || rk_order > 3) return MCFD_ERR_ARGUMENT;
  cudaSetDevice(e->device);
  // per-member step bounds, ordered before the replays
  for (mcfd_handle *h : e->members) {
    double cfl = h->opt.cfl > 0 ? h->opt.cfl : cfl_table(rk_order, h->mesh.p);
    h->launches += mcfd::launch_set_state(h, h->t_host, 0.0, dt_guess, cfl, 1);
    if (h->use_trace && h->trace_for != h->buf.u) h->launches += mcfd::launch_trace(h, h->buf.u);
    cudaError_t err = cudaGetLastError();
    if (err == cudaSuccess) err = cudaStreamSynchronize(h->stream);
    if (err != cudaSuccess) return ens_fail(e, MCFD_ERR_CUDA, std::string("member set-up: ") + cudaGetErrorString(err));
  }
  {
    const int grc = ens_ensure_graph(e, rk_order);
    if (grc) return grc;
  }
  for (int s = 0; s < n_steps; ++s) {
    cudaError_t err = cudaGraphLaunch(e->graph, e->stream);
    if (err != cudaSuccess) return ens_fail(e, MCFD_ERR_CUDA, std::string("cudaGraphLaunch: ") + cudaGetErrorString(err));
  }
  cudaError_t err = cudaStreamSynchronize(e->stream);
  if (err != cudaSuccess) return ens_fail(e, MCFD_ERR_CUDA, std::string("ensemble replay: ") + cudaGetErrorString(err));
  int rc = MCFD_OK;
  for (size_t i = 0; i < e->members.size(); ++i) {
    mcfd_handle *h = e->members[i];
    h->launches += (int64_t)e->kernels[i] * n_steps;
    mcfd::DevState st;
    if (cudaMemcpy(&st, h->buf.state, sizeof(st), cudaMemcpyDeviceToHost) == cudaSuccess) h->t_host = st.t;
    int r = check_status(h);
    if (r && !rc) {
      rc = r;
      e->err = "member " + std::to_string(i) + ": " + h->err;
    }
  }
  return rc;
}

int mcfd_ensemble_stream_begin(mcfd_ensemble *e) {
  if (!e) return MCFD_ERR_ARGUMENT;
  if (e->streaming) return MCFD_OK;
  cudaSetDevice(e->device);
  cudaError_t err = cudaSuccess;
  if (!e->copy_out) {
    for (int b = 0; b < 2 && err == cudaSuccess; ++b) {
      for (mcfd_handle *h : e->members) {
        double *pi = nullptr, *po = nullptr;
        if (err == cudaSuccess) err = cudaMalloc(&pi, sizeof(double) * h->mesh.column);
        if (err == cudaSuccess) e->in[b].push_back(pi);
        if (err == cudaSuccess) err = cudaMalloc(&po, sizeof(double) * h->mesh.column);
        if (err == cudaSuccess) e->out[b].push_back(po);
      }
      cudaEvent_t *evs[] = {&e->in_ready[b], &e->in_free[b], &e->out_ready[b], &e->out_free[b]};
      for (cudaEvent_t *ev : evs)
        if (err == cudaSuccess) err = cudaEventCreateWithFlags(ev, cudaEventDisableTiming);
    }
    if (err == cudaSuccess) err = cudaStreamCreateWithFlags(&e->copy_in, cudaStreamNonBlocking);
    if (err == cudaSuccess) err = cudaStreamCreateWithFlags(&e->copy_out, cudaStreamNonBlocking);
    if (err != cudaSuccess) {
      ens_stream_release(e);
      return ens_fail(e, MCFD_ERR_CUDA, std::string("ensemble stream set-up: ") + cudaGetErrorString(err));
    }
  }
  e->streaming = true;
  e->k = 0;
  return MCFD_OK;
}

int mcfd_ensemble_stream_step(mcfd_ensemble *e, const double *const *host_in, double *const *host_out,
                              int32_t n_steps, double dt_guess, int32_t rk_order) {
  mcfd::NvtxRange nvtx_range("mcfd_ensemble_stream_step");
  if (!e || !host_in || !host_out || n_steps < 1 || rk_order < 1 || rk_order > 3) return MCFD_ERR_ARGUMENT;
  if (!e->streaming) return ens_fail(e, MCFD_ERR_STATE, "mcfd_ensemble_stream_begin first");
  cudaSetDevice(e->device);
  const int b = (int)(e->k & 1);
  const size_t nm = e->members.size();
  cudaError_t err = cudaStreamWaitEvent(e->copy_in, e->in_free[b], 0);
  for (size_t i = 0; i < nm && err == cudaSuccess; ++i)
    err = cudaMemcpyAsync(e->in[b][i], host_in[i], sizeof(double) * e->members[i]->mesh.column,
                          cudaMemcpyHostToDevice, e->copy_in);
  if (err == cudaSuccess) err = cudaEventRecord(e->in_ready[b], e->copy_in);
  if (err == cudaSuccess) err = cudaStreamWaitEvent(e->stream, e->in_ready[b], 0);
  if (err == cudaSuccess) err = cudaStreamWaitEvent(e->stream, e->out_free[b], 0);
  // load every member's column and set its step bounds, ordered on the
  // ensemble stream ahead of the replays that fork from it
  for (size_t i = 0; i < nm && err == cudaSuccess; ++i) {
    mcfd_handle *h = e->members[i];
    err = cudaMemcpyAsync(h->buf.u, e->in[b][i], sizeof(double) * h->mesh.column, cudaMemcpyDeviceToDevice,
                          e->stream);
    if (err != cudaSuccess) break;
    mcfd::invalidate_trace(h, h->buf.u);
    const cudaStream_t own = h->stream;
    h->stream = e->stream;
    const double cfl = h->opt.cfl > 0 ? h->opt.cfl : cfl_table(rk_order, h->mesh.p);
    h->launches += mcfd::launch_set_bounds(h, dt_guess, cfl);  // times continue on the device
    h->launches += mcfd::launch_trace(h, h->buf.u);
    h->stream = own;
    err = cudaGetLastError();
  }
  if (err == cudaSuccess) err = cudaEventRecord(e->in_free[b], e->stream);
  if (err != cudaSuccess) return ens_fail(e, MCFD_ERR_CUDA, std::string("ensemble stream load: ") + cudaGetErrorString(err));
  const int grc = ens_ensure_graph(e, rk_order);
  if (grc) return grc;
  for (int s = 0; s < n_steps && err == cudaSuccess; ++s) err = cudaGraphLaunch(e->graph, e->stream);
  for (size_t i = 0; i < nm; ++i) e->members[i]->launches += (int64_t)e->kernels[i] * n_steps;
  for (size_t i = 0; i < nm && err == cudaSuccess; ++i)
    err = cudaMemcpyAsync(e->out[b][i], e->members[i]->buf.u, sizeof(double) * e->members[i]->mesh.column,
                          cudaMemcpyDeviceToDevice, e->stream);
  if (err == cudaSuccess) err = cudaEventRecord(e->out_ready[b], e->stream);
  if (err == cudaSuccess) err = cudaStreamWaitEvent(e->copy_out, e->out_ready[b], 0);
  for (size_t i = 0; i < nm && err == cudaSuccess; ++i)
    err = cudaMemcpyAsync(host_out[i], e->out[b][i], sizeof(double) * e->members[i]->mesh.column,
                          cudaMemcpyDeviceToHost, e->copy_out);
  if (err == cudaSuccess) err = cudaEventRecord(e->out_free[b], e->copy_out);
  if (err != cudaSuccess) return ens_fail(e, MCFD_ERR_CUDA, std::string("ensemble stream step: ") + cudaGetErrorString(err));
  ++e->k;
  return MCFD_OK;
}

int mcfd_ensemble_stream_end(mcfd_ensemble *e) {
  if (!e) return MCFD_ERR_ARGUMENT;
  if (!e->streaming) return MCFD_OK;
  cudaSetDevice(e->device);
  cudaError_t err = cudaStreamSynchronize(e->copy_in);
  if (err == cudaSuccess) err = cudaStreamSynchronize(e->stream);
  if (err == cudaSuccess) err = cudaStreamSynchronize(e->copy_out);
  e->streaming = false;
  if (err != cudaSuccess) return ens_fail(e, MCFD_ERR_CUDA, std::string("ensemble stream end: ") + cudaGetErrorString(err));
  int rc = MCFD_OK;
  for (size_t i = 0; i < e->members.size(); ++i) {
    mcfd_handle *h = e->members[i];
    mcfd::DevState st;
    if (cudaMemcpy(&st, h->buf.state, sizeof(st), cudaMemcpyDeviceToHost) == cudaSuccess) h->t_host = st.t;
    const int r = check_status(h);
    if (r && !rc) {
      rc = r;
      e->err = "member " + std::to_string(i) + ": " + h->err;
    }
  }
  return rc;
}

int mcfd_set_stream(mcfd_handle *h, void *cuda_stream) {
  if (!h) return MCFD_ERR_ARGUMENT;
  cudaSetDevice(h->device);
  CUDA_TRY(h, cudaStreamSynchronize(h->stream));
  if (cuda_stream) {
    if (h->own_stream) cudaStreamDestroy(h->stream);
    h->stream = (cudaStream_t)cuda_stream;
    h->own_stream = false;
  } else if (!h->own_stream) {
    CUDA_TRY(h, cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking));
    h->own_stream = true;
  }
  return MCFD_OK;
}

int mcfd_synchronize(mcfd_handle *h) {
  if (!h) return MCFD_ERR_ARGUMENT;
  cudaSetDevice(h->device);
  return check_status(h);
}

int mcfd_face_node_maps(const mcfd_handle *h, int16_t *holder, int16_t *sharer) {
  if (!h || !holder || !sharer) return MCFD_ERR_ARGUMENT;
  if (h->opt.scheme == MCFD_MODAL) return MCFD_ERR_UNSUPPORTED;
  std::memcpy(holder, h->mesh.map_h.data(), sizeof(int16_t) * h->mesh.map_h.size());
  std::memcpy(sharer, h->mesh.map_s.data(), sizeof(int16_t) * h->mesh.map_s.size());
  return MCFD_OK;
}

int64_t mcfd_launch_count(const mcfd_handle *h) { return h ? h->launches : -1; }

int mcfd_set_cases(mcfd_handle *h, int32_t n_cases, const int64_t *case_offsets) {
  if (!h || n_cases < 1 || !case_offsets) return MCFD_ERR_ARGUMENT;
  if (h->visc.on) return fail(h, MCFD_ERR_UNSUPPORTED, "cases take a handle without the artificial viscosity");
  const int64_t C = h->mesh.n_cells;
  if (n_cases > 1024) return fail(h, MCFD_ERR_UNSUPPORTED, "at most 1024 cases per handle");
  if (case_offsets[0] != 0 || case_offsets[n_cases] != C)
    return fail(h, MCFD_ERR_ARGUMENT, "case offsets must run from 0 to the cell count");
  std::vector<int32_t> cell_case(C);
  for (int32_t k = 0; k < n_cases; ++k) {
    if (case_offsets[k + 1] <= case_offsets[k])
      return fail(h, MCFD_ERR_ARGUMENT, "case offsets must increase strictly");
    for (int64_t c = case_offsets[k]; c < case_offsets[k + 1]; ++c) cell_case[c] = k;
  }
  cudaSetDevice(h->device);
  CUDA_TRY(h, cudaStreamSynchronize(h->stream));
  // no face may join two cases
  if (h->mesh.n_faces > 0) {
    std::vector<int2> fc(h->mesh.n_faces);
    CUDA_TRY(h, cudaMemcpy(fc.data(), h->mesh.face_cells, sizeof(int2) * fc.size(), cudaMemcpyDeviceToHost));
    for (const int2 &f : fc)
      if (f.y >= 0 && cell_case[f.x] != cell_case[f.y])
        return fail(h, MCFD_ERR_MESH, "a face joins two cases");
  }
  auto &cs = h->cases;
  void *old[] = {cs.cell_case, cs.t, cs.dt, cs.rate};
  for (void *p : old)
    if (p) cudaFree(p);
  cs = mcfd::Cases{};
  int rc;
  if ((rc = upload(h, &cs.cell_case, cell_case))) return rc;
  std::vector<double> zeros(n_cases, 0.0);
  if ((rc = upload(h, &cs.t, zeros))) return rc;
  if ((rc = upload(h, &cs.dt, zeros))) return rc;
  std::vector<unsigned long long> zr(n_cases, 0ull);
  if ((rc = upload(h, &cs.rate, zr))) return rc;
  cs.offsets.assign(case_offsets, case_offsets + n_cases + 1);
  cs.n = n_cases;
  mcfd::drop_graphs(h);
  return MCFD_OK;
}

int mcfd_case_times(mcfd_handle *h, double *t, double *dt, int32_t n) {
  if (!h || !t || n != h->cases.n || n < 1) return MCFD_ERR_ARGUMENT;
  cudaSetDevice(h->device);
  CUDA_TRY(h, cudaMemcpyAsync(t, h->cases.t, sizeof(double) * n, cudaMemcpyDeviceToHost, h->stream));
  if (dt)
    CUDA_TRY(h, cudaMemcpyAsync(dt, h->cases.dt, sizeof(double) * n, cudaMemcpyDeviceToHost, h->stream));
  CUDA_TRY(h, cudaStreamSynchronize(h->stream));
  return MCFD_OK;
}

int64_t mcfd_point_count(const mcfd_handle *h) {
  if (!h) return -1;
  return h->opt.scheme == MCFD_MODAL ? h->modal.n_vol : 0;
}

int mcfd_points(const mcfd_handle *h, double *xyz, int64_t n) {
  if (!h || !xyz) return MCFD_ERR_ARGUMENT;
  if (h->opt.scheme != MCFD_MODAL) return MCFD_ERR_UNSUPPORTED;
  if (n != h->modal.n_vol) return MCFD_ERR_ARGUMENT;
  std::memcpy(xyz, h->modal.host_points.data(), sizeof(double) * 3 * n);
  return MCFD_OK;
}

int mcfd_project(mcfd_handle *h, const double *values, int64_t n) {
  mcfd::NvtxRange nvtx_range("mcfd_project");
  if (!h || !values) return MCFD_ERR_ARGUMENT;
  if (h->opt.scheme != MCFD_MODAL)
    return fail(h, MCFD_ERR_UNSUPPORTED, "mcfd_project belongs to the modal scheme");
  if (n != h->modal.n_vol) return fail(h, MCFD_ERR_ARGUMENT, "point count mismatch");
  cudaSetDevice(h->device);
  if (!h->modal.values)
    CUDA_TRY(h, cudaMalloc(&h->modal.values, sizeof(double) * mcfd::kK * n));
  CUDA_TRY(h, cudaMemcpyAsync(h->modal.values, values, sizeof(double) * mcfd::kK * n,
                              cudaMemcpyHostToDevice, h->stream));
  h->launches += mcfd::launch_modal_project(h, h->buf.u);
  CUDA_TRY(h, cudaGetLastError());
  CUDA_TRY(h, cudaStreamSynchronize(h->stream));
  // WithLimiter::Approximate reconstructs after projecting (with_limiter.hpp:61-65)
  return limit_current(h);
}

int mcfd_kernel_times(mcfd_handle *h, int32_t reps, double *out_ms) {
  if (!h || !out_ms || reps < 1) return MCFD_ERR_ARGUMENT;
  cudaSetDevice(h->device);
  cudaEvent_t e0, e1;
  CUDA_TRY(h, cudaEventCreate(&e0));
  CUDA_TRY(h, cudaEventCreate(&e1));
  auto &b = h->buf;
  double cfl = h->opt.cfl > 0 ? h->opt.cfl : cfl_table(3, h->mesh.p);
  h->launches += mcfd::launch_set_state(h, h->t_host, 0.0, 1e300, cfl, 1);
  if (h->use_trace && h->trace_for != b.u) h->launches += mcfd::launch_trace(h, b.u);
  float ms = 0;
  // dt reduction (reads u)
  CUDA_TRY(h, cudaEventRecord(e0, h->stream));
  for (int r = 0; r < reps; ++r) h->launches += mcfd::launch_dt(h, b.u);
  CUDA_TRY(h, cudaEventRecord(e1, h->stream));
  CUDA_TRY(h, cudaEventSynchronize(e1));
  CUDA_TRY(h, cudaEventElapsedTime(&ms, e0, e1));
  out_ms[0] = ms / reps;
  // face fluxes of the current solution
  CUDA_TRY(h, cudaEventRecord(e0, h->stream));
  for (int r = 0; r < reps; ++r) h->launches += mcfd::launch_face_flux(h, b.u, 0.0);
  CUDA_TRY(h, cudaEventRecord(e1, h->stream));
  CUDA_TRY(h, cudaEventSynchronize(e1));
  CUDA_TRY(h, cudaEventElapsedTime(&ms, e0, e1));
  out_ms[1] = ms / reps;
  // cell update in the middle-stage form (reads u_in and u0, writes u_out)
  CUDA_TRY(h, cudaEventRecord(e0, h->stream));
  for (int r = 0; r < reps; ++r)
    h->launches += mcfd::launch_cell_update(h, mcfd::kStageRk3Mid, b.u, b.u, b.u2, 0);
  CUDA_TRY(h, cudaEventRecord(e1, h->stream));
  CUDA_TRY(h, cudaEventSynchronize(e1));
  CUDA_TRY(h, cudaEventElapsedTime(&ms, e0, e1));
  out_ms[2] = ms / reps;
  // one whole step on a copy of the solution (u is restored afterwards)
  CUDA_TRY(h, cudaMemcpyAsync(b.res, b.u, sizeof(double) * h->mesh.column, cudaMemcpyDeviceToDevice, h->stream));
  if (h->use_trace && h->trace_for != b.u) h->launches += mcfd::launch_trace(h, b.u);
  CUDA_TRY(h, cudaEventRecord(e0, h->stream));
  for (int r = 0; r < reps; ++r) {
    h->launches += mcfd::launch_dt(h, b.u);
    h->launches += mcfd::launch_rk_stage_sequence(h, 3);
  }
  CUDA_TRY(h, cudaEventRecord(e1, h->stream));
  CUDA_TRY(h, cudaEventSynchronize(e1));
  CUDA_TRY(h, cudaEventElapsedTime(&ms, e0, e1));
  out_ms[3] = ms / reps;
  CUDA_TRY(h, cudaMemcpyAsync(b.u, b.res, sizeof(double) * h->mesh.column, cudaMemcpyDeviceToDevice, h->stream));
  mcfd::invalidate_trace(h, b.u);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  return check_status(h);
}

}  // extern "C"
