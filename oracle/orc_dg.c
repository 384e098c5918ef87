/*
 * ORACLE (test infrastructure only): geometry, DGSEM residual, time step and
 * SSP-RK steppers restated from the reference project.  It is the parity
 * checker and the timed CPU baseline ("reference algorithm, restated"); the
 * product library never calls it.
 *
 * It follows the reference's data structures where they decide the numbers:
 *   - GLL rule and tensor-product point order (i outer, k inner):
 *       include/mini/integrator/lobatto.hpp:37-83, integrator/hexahedron.hpp:66-93
 *   - Lagrange derivatives from the inverted Vandermonde matrix:
 *       include/mini/basis/lagrange.hpp:53-85, 131-134
 *   - Hex8 shape functions and J = d(x,y,z)/d(xi,eta,zeta) with rows per
 *     local direction:  coordinate/hexahedron.hpp:426-464, coordinate/cell.hpp:82-90
 *   - global weights w*det(J):  integrator/element.hpp:102-115
 *   - cached basis global gradients J^-1 * grad_local, dense 3 x N per node:
 *       polynomial/hexahedron.hpp:221-239 (kLocal = false, the demo setting)
 *   - face nodes sorted by the holder's face table (hexahedron.hpp:378-389),
 *     Quad4 map, weight w*sqrt(det(J J^T)), frame (n, t, n x t):
 *       coordinate/face.hpp:54-62, coordinate/quadrangle.hpp:77-105
 *   - face point to cell node matching by |x_f - x_h| < 1e-12:
 *       spatial/dg/lobatto.hpp:58-78, spatial/fem.hpp:43-45
 *   - residual: zero, volume (dense F * G per node), local faces, boundaries
 *     (supersonic in, supersonic out, subsonic in, subsonic out, inviscid
 *     wall, smart), then residual *= 1/w per node:
 *       spatial/fem.hpp:248-307, spatial/dg/lobatto.hpp:143-302
 *   - time step: spatial/fem.hpp:26-37, 417-435; part.hpp:213 (cbrt(V)/2)
 *   - RK1/2/3: temporal/rk.hpp:16-49, temporal/ode.hpp:121-133
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "orc.h"
#include "orc_internal.h"

#define K ORC_K
#define MAXQ ORC_MAXQ
#define MAXN (MAXQ * MAXQ * MAXQ)

static int g_threads = 0;
void orc_set_threads(int n) { g_threads = n; }
int orc_get_threads(void) {
#ifdef _OPENMP
  return g_threads > 0 ? g_threads : omp_get_max_threads();
#else
  return 1;
#endif
}

/* ---------------- 1D rules and Lagrange basis ---------------- */

static void gll_rule(int q, double *x, double *w) {
  switch (q) {
    case 2:
      x[0] = -1.0; x[1] = +1.0;
      w[0] = 1.0; w[1] = 1.0;
      break;
    case 3:
      x[0] = -1.0; x[1] = 0.0; x[2] = +1.0;
      w[0] = 1.0 / 3; w[1] = 4.0 / 3; w[2] = 1.0 / 3;
      break;
    case 4:
      x[0] = -1.0; x[1] = -sqrt(1.0 / 5); x[2] = +sqrt(1.0 / 5); x[3] = +1.0;
      w[0] = 1.0 / 6; w[1] = 5.0 / 6; w[2] = 5.0 / 6; w[3] = 1.0 / 6;
      break;
    case 5:
      x[0] = -1.0; x[1] = -sqrt(21.0) / 7; x[2] = 0.0; x[3] = +sqrt(21.0) / 7;
      x[4] = +1.0;
      w[0] = 0.1; w[1] = 49.0 / 90; w[2] = 32.0 / 45; w[3] = 49.0 / 90;
      w[4] = 0.1;
      break;
    default: {  /* 6 */
      double s7 = sqrt(7.0);
      x[0] = -1.0;
      x[1] = -sqrt((7 + 2 * s7) / 21);
      x[2] = -sqrt((7 - 2 * s7) / 21);
      x[3] = +sqrt((7 - 2 * s7) / 21);
      x[4] = +sqrt((7 + 2 * s7) / 21);
      x[5] = +1.0;
      w[0] = 1.0 / 15; w[1] = (14.0 - s7) / 30; w[2] = (14.0 + s7) / 30;
      w[3] = (14.0 + s7) / 30; w[4] = (14.0 - s7) / 30; w[5] = 1.0 / 15;
    }
  }
}

/* In-place inverse of an n x n row-major matrix (Gauss-Jordan, partial
 * pivoting).  Returns 0 on success. */
static int invert(int n, double *a) {
  double inv[MAXQ * MAXQ];
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < n; ++j) inv[i * n + j] = (i == j);
  for (int c = 0; c < n; ++c) {
    int piv = c;
    for (int r = c + 1; r < n; ++r)
      if (fabs(a[r * n + c]) > fabs(a[piv * n + c])) piv = r;
    if (a[piv * n + c] == 0) return -1;
    if (piv != c) {
      for (int j = 0; j < n; ++j) {
        double t = a[c * n + j]; a[c * n + j] = a[piv * n + j]; a[piv * n + j] = t;
        t = inv[c * n + j]; inv[c * n + j] = inv[piv * n + j]; inv[piv * n + j] = t;
      }
    }
    double d = a[c * n + c];
    for (int j = 0; j < n; ++j) { a[c * n + j] /= d; inv[c * n + j] /= d; }
    for (int r = 0; r < n; ++r) {
      if (r == c) continue;
      double f = a[r * n + c];
      if (f == 0) continue;
      for (int j = 0; j < n; ++j) {
        a[r * n + j] -= f * a[c * n + j];
        inv[r * n + j] -= f * inv[c * n + j];
      }
    }
  }
  memcpy(a, inv, sizeof(double) * n * n);
  return 0;
}

/* D[a][i] = l_i'(x_a): Taylor derivative row times the inverse Vandermonde
 * matrix (lagrange.hpp:73-85, 131-134). */
static void lagrange_derivatives(int q, const double *x, double *d) {
  double v[MAXQ * MAXQ];
  for (int j = 0; j < q; ++j) {
    double p = 1;
    for (int m = 0; m < q; ++m) { v[j * q + m] = p; p *= x[j]; }
  }
  invert(q, v);  /* v = lagrange_to_taylor */
  for (int a = 0; a < q; ++a) {
    double trow[MAXQ];
    trow[0] = 0;
    double p = 1;
    for (int m = 1; m < q; ++m) { trow[m] = m * p; p *= x[a]; }
    for (int i = 0; i < q; ++i) {
      double s = 0;
      for (int m = 0; m < q; ++m) s += trow[m] * v[m * q + i];
      d[a * q + i] = s;
    }
  }
}

/* Second derivatives D2[a][i] = l_i''(x_a) the same way: the Taylor second
 * derivative row times the inverse Vandermonde matrix (lagrange.hpp:130-133,
 * polynomial/hexahedron.hpp:155-170). */
void orc_lagrange_second(int q, const double *x, double *d2) {
  double v[MAXQ * MAXQ];
  for (int j = 0; j < q; ++j) {
    double p = 1;
    for (int m = 0; m < q; ++m) { v[j * q + m] = p; p *= x[j]; }
  }
  invert(q, v);
  for (int a = 0; a < q; ++a) {
    double trow[MAXQ];
    trow[0] = 0;
    if (q > 1) trow[1] = 0;
    double p = 1;
    for (int m = 2; m < q; ++m) { trow[m] = m * (m - 1) * p; p *= x[a]; }
    for (int i = 0; i < q; ++i) {
      double s = 0;
      for (int m = 0; m < q; ++m) s += trow[m] * v[m * q + i];
      d2[a * q + i] = s;
    }
  }
}

/* ---------------- Hex8 / Quad4 maps ---------------- */

static const int kHexLocal[8][3] = {
    {-1, -1, -1}, {+1, -1, -1}, {+1, +1, -1}, {-1, +1, -1},
    {-1, -1, +1}, {+1, -1, +1}, {+1, +1, +1}, {-1, +1, +1}};
/* The first 4 entries of Hexahedron27::faces_ (coordinate/hexahedron.hpp:378-389). */
static const int kHexFace[6][4] = {
    {0, 3, 2, 1}, {0, 1, 5, 4}, {1, 2, 6, 5},
    {2, 3, 7, 6}, {0, 4, 7, 3}, {4, 5, 6, 7}};
static const int kQuadLocal[4][2] = {{-1, -1}, {+1, -1}, {+1, +1}, {-1, +1}};

static void hex8_global(const double *xn, const double *loc, double *g) {
  g[0] = g[1] = g[2] = 0;
  for (int n = 0; n < 8; ++n) {
    double v = (1 + kHexLocal[n][0] * loc[0]);
    v *= (1 + kHexLocal[n][1] * loc[1]);
    v *= (1 + kHexLocal[n][2] * loc[2]);
    v /= 8;
    for (int d = 0; d < 3; ++d) g[d] += xn[n * 3 + d] * v;
  }
}

/* J[i][j] = d x_j / d xi_i */
static void hex8_jacobian(const double *xn, const double *loc, double *jac) {
  memset(jac, 0, sizeof(double) * 9);
  for (int n = 0; n < 8; ++n) {
    double fx = (1 + kHexLocal[n][0] * loc[0]);
    double fy = (1 + kHexLocal[n][1] * loc[1]);
    double fz = (1 + kHexLocal[n][2] * loc[2]);
    double g[3] = {kHexLocal[n][0] * (fy * fz / 8), kHexLocal[n][1] * (fz * fx / 8),
                   kHexLocal[n][2] * (fx * fy / 8)};
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) jac[i * 3 + j] += g[i] * xn[n * 3 + j];
  }
}

static double det3(const double *m) {
  return m[0] * (m[4] * m[8] - m[5] * m[7]) - m[1] * (m[3] * m[8] - m[5] * m[6]) +
         m[2] * (m[3] * m[7] - m[4] * m[6]);
}

static void inv3(const double *m, double *inv) {
  double det = det3(m);
  inv[0] = (m[4] * m[8] - m[5] * m[7]) / det;
  inv[1] = (m[2] * m[7] - m[1] * m[8]) / det;
  inv[2] = (m[1] * m[5] - m[2] * m[4]) / det;
  inv[3] = (m[5] * m[6] - m[3] * m[8]) / det;
  inv[4] = (m[0] * m[8] - m[2] * m[6]) / det;
  inv[5] = (m[2] * m[3] - m[0] * m[5]) / det;
  inv[6] = (m[3] * m[7] - m[4] * m[6]) / det;
  inv[7] = (m[1] * m[6] - m[0] * m[7]) / det;
  inv[8] = (m[0] * m[4] - m[1] * m[3]) / det;
}

static void quad4_global(const double *xn, double x, double y, double *g) {
  g[0] = g[1] = g[2] = 0;
  for (int n = 0; n < 4; ++n) {
    double v = (1 + kQuadLocal[n][0] * x) * (1 + kQuadLocal[n][1] * y) / 4;
    for (int d = 0; d < 3; ++d) g[d] += xn[n * 3 + d] * v;
  }
}

static void quad4_jacobian(const double *xn, double x, double y, double *j) {
  memset(j, 0, sizeof(double) * 6);
  for (int n = 0; n < 4; ++n) {
    double fx = (1 + kQuadLocal[n][0] * x) / 4;
    double fy = (1 + kQuadLocal[n][1] * y) / 4;
    double gx = kQuadLocal[n][0] * fy, gy = kQuadLocal[n][1] * fx;
    for (int d = 0; d < 3; ++d) {
      j[d] += gx * xn[n * 3 + d];
      j[3 + d] += gy * xn[n * 3 + d];
    }
  }
}

static void cross(const double *a, const double *b, double *c) {
  c[0] = a[1] * b[2] - a[2] * b[1];
  c[1] = a[2] * b[0] - a[0] * b[2];
  c[2] = a[0] * b[1] - a[1] * b[0];
}

static void normalize(double *a) {
  double n = sqrt(a[0] * a[0] + a[1] * a[1] + a[2] * a[2]);
  a[0] /= n; a[1] /= n; a[2] /= n;
}

/* ---------------- mesh ---------------- */

/* struct orc_mesh: orc_internal.h */

int64_t orc_column_size(const orc_mesh *m) { return m->n_cells * m->n * K; }
int orc_mesh_degree(const orc_mesh *m) { return m->p; }
int64_t orc_mesh_cells(const orc_mesh *m) { return m->n_cells; }
int64_t orc_mesh_faces(const orc_mesh *m) { return m->n_faces; }
const int64_t *orc_mesh_face_cells(const orc_mesh *m) { return m->face_cells; }
const double *orc_mesh_face_shift(const orc_mesh *m) { return m->face_shift; }
void orc_cell_centers(const orc_mesh *m, double *center) {
  for (int64_t c = 0; c < m->n_cells; ++c)
    for (int d = 0; d < 3; ++d) center[c * 3 + d] = m->cell_center[c * 3 + d];
}
int orc_nodes_per_cell(const orc_mesh *m) { return m->n; }
double orc_cell_length(const orc_mesh *m, int64_t c) { return m->length[c]; }

void orc_mesh_destroy(orc_mesh *m) {
  if (!m) return;
  free(m->node_xyz); free(m->node_w); free(m->grad); free(m->length); free(m->cell_center);
  free(m->corners); free(m->type);
  free(m->face_shift); free(m->jdi); free(m->detj); free(m->face_sides);
  free(m->face_cells); free(m->face_group); free(m->face_xyz); free(m->face_w);
  free(m->face_frame); free(m->map_h); free(m->map_s);
  free(m);
}

static int near12(const double *a, const double *b) {
  double dx = a[0] - b[0], dy = a[1] - b[1], dz = a[2] - b[2];
  return sqrt(dx * dx + dy * dy + dz * dz) < 1e-12;
}

orc_mesh *orc_mesh_create(int64_t n_nodes, const double *xyz, int64_t n_cells,
                          const int64_t *cell_nodes, const int32_t *cell_type,
                          int32_t stride, int64_t n_faces,
                          const int64_t *face_cells, const int32_t *face_sides,
                          const int32_t *face_group, const double *face_shift,
                          int degree) {
  if (degree < 1 || degree > 5 || n_cells <= 0) return NULL;
  orc_mesh *m = (orc_mesh *)calloc(1, sizeof(orc_mesh));
  m->p = degree;
  m->q = degree + 1;
  m->n = m->q * m->q * m->q;
  m->qf = m->q * m->q;
  m->n_cells = n_cells;
  m->n_faces = n_faces;
  gll_rule(m->q, m->xq, m->wq);
  lagrange_derivatives(m->q, m->xq, m->d);
  int Q = m->q, N = m->n, QF = m->qf;
  m->node_xyz = (double *)malloc(sizeof(double) * n_cells * N * 3);
  m->node_w = (double *)malloc(sizeof(double) * n_cells * N);
  m->grad = (double *)malloc(sizeof(double) * n_cells * N * 3 * N);
  m->length = (double *)malloc(sizeof(double) * n_cells);
  m->cell_center = (double *)malloc(sizeof(double) * n_cells * 3);
  m->corners = (double *)calloc(n_cells * 81, sizeof(double));
  m->type = (int32_t *)malloc(sizeof(int32_t) * n_cells);
  const int64_t S = stride > 0 ? stride : 8;
  for (int64_t c = 0; c < n_cells; ++c) {
    int t = cell_type ? cell_type[c] : ORC_CELL_HEX8;
    if (orc_type_is_tet(t) || orc_type_nodes(t) == 0 || orc_type_nodes(t) > S) {
      orc_mesh_destroy(m);
      return NULL;
    }
    m->type[c] = t;
  }
  m->jdi = (double *)malloc(sizeof(double) * n_cells * N * 9);
  m->detj = (double *)malloc(sizeof(double) * n_cells * N);
  m->face_sides = (int32_t *)malloc(sizeof(int32_t) * (n_faces * 2 + 1));
  if (n_faces) memcpy(m->face_sides, face_sides, sizeof(int32_t) * n_faces * 2);
  m->scheme = ORC_SCHEME_DGSEM;
  int bad = 0;
#pragma omp parallel for schedule(static) num_threads(orc_get_threads())
  for (int64_t c = 0; c < n_cells; ++c) {
    const int type = m->type[c], nv = orc_type_nodes(type);
    double xn[81];
    for (int v = 0; v < nv; ++v) {
      int64_t id = cell_nodes[c * S + v];
      if (id < 0 || id >= n_nodes) { bad = 1; id = 0; }
      for (int d = 0; d < 3; ++d) xn[v * 3 + d] = xyz[id * 3 + d];
    }
    double volume = 0;
    const double zero[3] = {0, 0, 0};
    memcpy(&m->corners[c * 81], xn, sizeof(double) * 3 * nv);
    if (type == ORC_CELL_HEX8) {
      hex8_global(xn, zero, &m->cell_center[c * 3]);
    } else {
      double jz[9];
      orc_map_point(type, xn, zero, &m->cell_center[c * 3], jz);
    }
    for (int i = 0; i < Q; ++i)
      for (int j = 0; j < Q; ++j)
        for (int k = 0; k < Q; ++k) {
          int qn = (i * Q + j) * Q + k;
          double loc[3] = {m->xq[i], m->xq[j], m->xq[k]};
          double jac[9], inv[9];
          if (type == ORC_CELL_HEX8) {
            hex8_global(xn, loc, &m->node_xyz[(c * N + qn) * 3]);
            hex8_jacobian(xn, loc, jac);
          } else {
            orc_map_point(type, xn, loc, &m->node_xyz[(c * N + qn) * 3], jac);
          }
          double det = det3(jac);
          double w = m->wq[i] * m->wq[j] * m->wq[k] * det;
          m->node_w[c * N + qn] = w;
          volume += w;
          inv3(jac, inv);
          m->detj[c * N + qn] = det;
          for (int e = 0; e < 9; ++e) m->jdi[(c * N + qn) * 9 + e] = det * inv[e];
          /* local gradients of every basis function at node (i,j,k) */
          double *g = &m->grad[((c * N + qn) * 3) * N];
          for (int r = 0; r < 3; ++r)
            for (int nb = 0; nb < N; ++nb) {
              int bi = nb / (Q * Q), bj = (nb / Q) % Q, bk = nb % Q;
              double l0 = (bj == j && bk == k) ? m->d[i * Q + bi] : 0;
              double l1 = (bi == i && bk == k) ? m->d[j * Q + bj] : 0;
              double l2 = (bi == i && bj == j) ? m->d[k * Q + bk] : 0;
              g[r * N + nb] = inv[r * 3 + 0] * l0 + inv[r * 3 + 1] * l1 +
                              inv[r * 3 + 2] * l2;
            }
        }
    m->length[c] = cbrt(volume) * 0.5;
  }
  m->face_cells = (int64_t *)malloc(sizeof(int64_t) * n_faces * 2);
  m->face_group = (int32_t *)malloc(sizeof(int32_t) * n_faces);
  m->face_xyz = (double *)malloc(sizeof(double) * n_faces * QF * 3);
  m->face_w = (double *)malloc(sizeof(double) * n_faces * QF);
  m->face_frame = (double *)malloc(sizeof(double) * n_faces * QF * 9);
  m->map_h = (int16_t *)malloc(sizeof(int16_t) * n_faces * QF);
  m->map_s = (int16_t *)malloc(sizeof(int16_t) * n_faces * QF);
  memcpy(m->face_cells, face_cells, sizeof(int64_t) * n_faces * 2);
  memcpy(m->face_group, face_group, sizeof(int32_t) * n_faces);
  m->face_shift = (double *)calloc(n_faces * 3 + 1, sizeof(double));
  if (face_shift) memcpy(m->face_shift, face_shift, sizeof(double) * n_faces * 3);
#pragma omp parallel for schedule(static) num_threads(orc_get_threads())
  for (int64_t f = 0; f < n_faces; ++f) {
    int64_t h = face_cells[f * 2], s = face_cells[f * 2 + 1];
    int side = face_sides[f * 2];
    if (h < 0 || h >= n_cells || side < 0 || side > 5) { bad = 1; continue; }
    double xn[12];
    for (int v = 0; v < 4; ++v) {
      int64_t id = cell_nodes[h * S + kHexFace[side][v]];
      for (int d = 0; d < 3; ++d) xn[v * 3 + d] = xyz[id * 3 + d];
    }
    /* curved holder: the face's points from the cell map at the face's local
     * points; tangents J^T dloc/da (corner 0 -> 1) and J^T dloc/db (0 -> 3) */
    const int htype = m->type[h];
    double l0[3], da[3], db[3];
    for (int d = 0; d < 3; ++d) {
      l0[d] = kHexLocal[kHexFace[side][0]][d];
      da[d] = (kHexLocal[kHexFace[side][1]][d] - l0[d]) / 2;
      db[d] = (kHexLocal[kHexFace[side][3]][d] - l0[d]) / 2;
    }
    double shift[3] = {0, 0, 0};
    if (face_shift) for (int d = 0; d < 3; ++d) shift[d] = face_shift[f * 3 + d];
    for (int i = 0; i < Q; ++i)
      for (int j = 0; j < Q; ++j) {
        int fp = i * Q + j;
        double *gx = &m->face_xyz[(f * QF + fp) * 3];
        double jac[6];
        if (htype == ORC_CELL_HEX8) {
          quad4_global(xn, m->xq[i], m->xq[j], gx);
          quad4_jacobian(xn, m->xq[i], m->xq[j], jac);
        } else {
          double loc[3], J[9];
          for (int d = 0; d < 3; ++d) loc[d] = l0[d] + (m->xq[i] + 1) * da[d] + (m->xq[j] + 1) * db[d];
          orc_map_point(htype, &m->corners[h * 81], loc, gx, J);
          for (int d = 0; d < 3; ++d) {
            jac[d] = J[0 * 3 + d] * da[0] + J[1 * 3 + d] * da[1] + J[2 * 3 + d] * da[2];
            jac[3 + d] = J[0 * 3 + d] * db[0] + J[1 * 3 + d] * db[1] + J[2 * 3 + d] * db[2];
          }
        }
        double a = jac[0] * jac[0] + jac[1] * jac[1] + jac[2] * jac[2];
        double b = jac[0] * jac[3] + jac[1] * jac[4] + jac[2] * jac[5];
        double cc = jac[3] * jac[3] + jac[4] * jac[4] + jac[5] * jac[5];
        m->face_w[f * QF + fp] = m->wq[i] * m->wq[j] * sqrt(a * cc - b * b);
        double *fr = &m->face_frame[(f * QF + fp) * 9];
        cross(&jac[0], &jac[3], &fr[0]);
        normalize(&fr[0]);
        fr[3] = jac[0]; fr[4] = jac[1]; fr[5] = jac[2];
        normalize(&fr[3]);
        cross(&fr[0], &fr[3], &fr[6]);
        /* Near matching over every node of the holder and the sharer */
        int16_t mh = -1, ms = -1;
        for (int nb = 0; nb < N; ++nb)
          if (near12(gx, &m->node_xyz[(h * N + nb) * 3])) { mh = (int16_t)nb; break; }
        if (s >= 0) {
          for (int nb = 0; nb < N; ++nb) {
            const double *xs = &m->node_xyz[(s * N + nb) * 3];
            double sh[3] = {xs[0] + shift[0], xs[1] + shift[1], xs[2] + shift[2]};
            if (near12(gx, sh)) { ms = (int16_t)nb; break; }
          }
          if (ms < 0) bad = 1;
        }
        if (mh < 0) bad = 1;
        m->map_h[f * QF + fp] = mh;
        m->map_s[f * QF + fp] = ms;
      }
  }
  if (bad) {
    orc_mesh_destroy(m);
    return NULL;
  }
  return m;
}

int orc_face_node_maps(const orc_mesh *m, int16_t *holder, int16_t *sharer) {
  memcpy(holder, m->map_h, sizeof(int16_t) * m->n_faces * m->qf);
  memcpy(sharer, m->map_s, sizeof(int16_t) * m->n_faces * m->qf);
  return 0;
}

int orc_node_geometry(const orc_mesh *m, double *xyz, double *weights) {
  if (xyz) memcpy(xyz, m->node_xyz, sizeof(double) * m->n_cells * m->n * 3);
  if (weights) memcpy(weights, m->node_w, sizeof(double) * m->n_cells * m->n);
  return 0;
}

int orc_face_geometry(const orc_mesh *m, double *xyz, double *weights,
                      double *frames) {
  int64_t n = m->n_faces * m->qf;
  if (xyz) memcpy(xyz, m->face_xyz, sizeof(double) * n * 3);
  if (weights) memcpy(weights, m->face_w, sizeof(double) * n);
  if (frames) memcpy(frames, m->face_frame, sizeof(double) * n * 9);
  return 0;
}

/* ---------------- residual ---------------- */

static void given_value(const orc_bc *bc, const double *x, double t, int64_t point,
                        double *v) {
  const double *src = bc->a;
  if (bc->program == ORC_STATE_MOVING_SPLIT) {
    src = (x[bc->axis] - bc->speed * t) < bc->position ? bc->a : bc->b;
  } else if (bc->program == ORC_STATE_OBLIQUE_SPLIT) {
    src = (bc->normal[0] * x[0] + bc->normal[1] * x[1] + bc->normal[2] * x[2] - bc->speed * t) < bc->position
              ? bc->a : bc->b;
  } else if (bc->program == ORC_STATE_TABLE && bc->table) {
    src = &bc->table[point * K];
  }
  memcpy(v, src, sizeof(double) * K);
}

void orc_mesh_set_scheme(orc_mesh *m, int scheme) { m->scheme = scheme; }

/* Vincent::LocalToRightDerivative(1) with c_next = HuynhLumpingLobatto(p)
 * (basis/vincent.hpp:30-32, 73-89): Legendre derivatives by the recurrence
 * P'_{k+1}(x) = (k+1) P_k(x) + x P'_k(x) at x = 1, where P_k(1) = 1. */
double orc_fr_g_prime(int p) {
  double c_next = p / (2.0 * p + 1), c_prev = 1 - c_next;
  double prev = 0, curr = 0, next = 0;
  for (int k = 0; k <= p; ++k) {
    if (k > 0) { prev = curr; curr = next; }
    next = (k + 1) * 1.0 + 1.0 * curr;
  }
  return 0.5 * (curr + c_prev * prev + c_next * next);
}

/* fr::Lobatto residual (spatial/fr/general.hpp:249-288, fr/lobatto.hpp:66-433):
 * residual[q] -= div of the interpolated contravariant flux at node q; at
 * every flux point the holder (sharer) node gets
 *   -= g'(+-1) (F_upwind * scale - F_contravariant[:, dir])
 * with scale = +-|det(J) J^-1 e_dir|; finally residual /= det(J). */
static int fr_residual(const orc_mesh *m, int riemann, int n_bc,
                       const orc_bc *bcs, double t, const double *u,
                       double *r) {
  const int Q = m->q, N = m->n, QF = m->qf, KN = K * m->n;
  int64_t L = orc_column_size(m);
  memset(r, 0, sizeof(double) * L);
  const double g1 = orc_fr_g_prime(m->p);
  double *cflux = (double *)malloc(sizeof(double) * m->n_cells * N * 15);
  /* AddFluxDivergence */
#pragma omp parallel for schedule(static) num_threads(orc_get_threads())
  for (int64_t c = 0; c < m->n_cells; ++c) {
    const double *uc = u + c * KN;
    double *fc = cflux + c * N * 15;
    for (int q = 0; q < N; ++q) {
      double f[15];
      orc_flux_matrix(uc + q * K, f);
      const double *jd = &m->jdi[(c * N + q) * 9];
      for (int k = 0; k < K; ++k)
        for (int e = 0; e < 3; ++e)
          fc[q * 15 + k * 3 + e] = f[k * 3 + 0] * jd[0 * 3 + e] + f[k * 3 + 1] * jd[1 * 3 + e] +
                                   f[k * 3 + 2] * jd[2 * 3 + e];
    }
    for (int q = 0; q < N; ++q) {
      int i = q / QF, j = (q / Q) % Q, l = q % Q;
      double value[K] = {0, 0, 0, 0, 0};
      for (int kb = 0; kb < N; ++kb) {
        int a = kb / QF, b = (kb / Q) % Q, cc = kb % Q;
        double g0 = (b == j && cc == l) ? m->d[i * Q + a] : 0;
        double gy = (a == i && cc == l) ? m->d[j * Q + b] : 0;
        double gz = (a == i && b == j) ? m->d[l * Q + cc] : 0;
        for (int k = 0; k < K; ++k)
          value[k] += fc[kb * 15 + k * 3 + 0] * g0 + fc[kb * 15 + k * 3 + 1] * gy +
                      fc[kb * 15 + k * 3 + 2] * gz;
      }
      for (int k = 0; k < K; ++k) r[c * KN + q * K + k] -= value[k];
    }
  }
  /* face corrections; dir and sign of each local face (fr/lobatto.hpp:81-152) */
  static const int kDir[6] = {2, 1, 0, 1, 0, 2};
  static const double kSign[6] = {-1, -1, +1, +1, -1, +1};
  for (int64_t f = 0; f < m->n_faces; ++f) {
    int64_t h = m->face_cells[f * 2], s = m->face_cells[f * 2 + 1];
    int g = m->face_group[f];
    if (s < 0 && !(g >= 0 && g < n_bc && bcs[g].kind != ORC_BC_NONE)) continue;
    /* a no-slip wall without viscosity: zero correction (fr/general.hpp:455-459) */
    if (s < 0 && bcs[g].kind == ORC_BC_NO_SLIP_WALL) continue;
    int sh = m->face_sides[f * 2], ss = s >= 0 ? m->face_sides[f * 2 + 1] : 0;
    for (int fp = 0; fp < QF; ++fp) {
      const double *fr = &m->face_frame[(f * QF + fp) * 9];
      int nh = m->map_h[f * QF + fp];
      const double *uh = u + h * KN + nh * K;
      double flux[K];
      if (s >= 0) {
        const double *us = u + s * KN + m->map_s[f * QF + fp] * K;
        orc_flux_rotated(riemann, fr, uh, us, flux);
      } else {
        double given[K];
        given_value(&bcs[g], &m->face_xyz[(f * QF + fp) * 3], t, f * QF + fp, given);
        orc_flux_boundary(riemann, bcs[g].kind, fr, uh, given, flux);
      }
      {
        const double *jd = &m->jdi[(h * N + nh) * 9];
        int dir = kDir[sh];
        double nrm = sqrt(jd[0 * 3 + dir] * jd[0 * 3 + dir] + jd[1 * 3 + dir] * jd[1 * 3 + dir] +
                          jd[2 * 3 + dir] * jd[2 * 3 + dir]);
        double scale = kSign[sh] * nrm, gp = kSign[sh] * g1;
        for (int k = 0; k < K; ++k) {
          double fh = flux[k] * scale - cflux[(h * N + nh) * 15 + k * 3 + dir];
          r[h * KN + nh * K + k] -= fh * gp;
        }
      }
      if (s >= 0) {
        int ns = m->map_s[f * QF + fp];
        const double *jd = &m->jdi[(s * N + ns) * 9];
        int dir = kDir[ss];
        double nrm = sqrt(jd[0 * 3 + dir] * jd[0 * 3 + dir] + jd[1 * 3 + dir] * jd[1 * 3 + dir] +
                          jd[2 * 3 + dir] * jd[2 * 3 + dir]);
        double scale = kSign[ss] * nrm, gp = kSign[ss] * g1;
        for (int k = 0; k < K; ++k) {
          double fs = flux[k] * (-scale) - cflux[(s * N + ns) * 15 + k * 3 + dir];
          r[s * KN + ns * K + k] -= fs * gp;
        }
      }
    }
  }
  free(cflux);
  /* divide by det(J) (fr/general.hpp:249-268) */
#pragma omp parallel for schedule(static) num_threads(orc_get_threads())
  for (int64_t c = 0; c < m->n_cells; ++c)
    for (int q = 0; q < N; ++q) {
      double scale = 1.0 / m->detj[c * N + q];
      for (int k = 0; k < K; ++k) r[c * KN + q * K + k] *= scale;
    }
  return 0;
}

int orc_dgsem_residual(const orc_mesh *m, int riemann, int n_bc,
                       const orc_bc *bcs, double t, const double *u,
                       double *r) {
  if (m->scheme == ORC_SCHEME_FR) return fr_residual(m, riemann, n_bc, bcs, t, u, r);
  const int N = m->n, QF = m->qf, KN = K * m->n;
  int64_t L = orc_column_size(m);
  memset(r, 0, sizeof(double) * L);
  /* volume: AddFluxDivergence (dg/lobatto.hpp:161-170) */
#pragma omp parallel for schedule(static) num_threads(orc_get_threads())
  for (int64_t c = 0; c < m->n_cells; ++c) {
    const double *uc = u + c * KN;
    double *rc = r + c * KN;
    for (int q = 0; q < N; ++q) {
      double f[15];
      orc_flux_matrix(uc + q * K, f);
      double w = m->node_w[c * N + q];
      for (int i = 0; i < 15; ++i) f[i] *= w;
      const double *g = &m->grad[((c * N + q) * 3) * N];
      for (int nb = 0; nb < N; ++nb) {
        for (int k = 0; k < K; ++k) {
          double s = f[k * 3 + 0] * g[0 * N + nb] + f[k * 3 + 1] * g[1 * N + nb] +
                     f[k * 3 + 2] * g[2 * N + nb];
          rc[nb * K + k] += s;
        }
      }
    }
  }
  /* face fluxes (evaluated in parallel, scattered in face order) */
  double *flux = (double *)malloc(sizeof(double) * m->n_faces * QF * K);
#pragma omp parallel for schedule(static) num_threads(orc_get_threads())
  for (int64_t f = 0; f < m->n_faces; ++f) {
    int64_t h = m->face_cells[f * 2], s = m->face_cells[f * 2 + 1];
    int g = m->face_group[f];
    for (int fp = 0; fp < QF; ++fp) {
      double *out = &flux[(f * QF + fp) * K];
      const double *fr = &m->face_frame[(f * QF + fp) * 9];
      const double *uh = u + h * KN + m->map_h[f * QF + fp] * K;
      if (s >= 0) {
        const double *us = u + s * KN + m->map_s[f * QF + fp] * K;
        orc_flux_rotated(riemann, fr, uh, us, out);
      } else if (g >= 0 && g < n_bc && bcs[g].kind != ORC_BC_NONE) {
        double given[K];
        given_value(&bcs[g], &m->face_xyz[(f * QF + fp) * 3], t, f * QF + fp, given);
        orc_flux_boundary(riemann, bcs[g].kind, fr, uh, given, out);
      } else {
        memset(out, 0, sizeof(double) * K);
      }
      double w = m->face_w[f * QF + fp];
      for (int k = 0; k < K; ++k) out[k] *= w;
    }
  }
  /* interior faces: holder -= flux, sharer += flux (dg/lobatto.hpp:171-191) */
  for (int64_t f = 0; f < m->n_faces; ++f) {
    int64_t h = m->face_cells[f * 2], s = m->face_cells[f * 2 + 1];
    if (s < 0) continue;
    for (int fp = 0; fp < QF; ++fp) {
      const double *fl = &flux[(f * QF + fp) * K];
      double *rh = r + h * KN + m->map_h[f * QF + fp] * K;
      double *rs = r + s * KN + m->map_s[f * QF + fp] * K;
      for (int k = 0; k < K; ++k) rh[k] -= fl[k];
      for (int k = 0; k < K; ++k) rs[k] += fl[k];
    }
  }
  /* boundaries in the order of fem.hpp:260-307 */
  static const int order[6] = {ORC_BC_SUPERSONIC_INLET, ORC_BC_SUPERSONIC_OUTLET,
                               ORC_BC_SUBSONIC_INLET, ORC_BC_SUBSONIC_OUTLET,
                               ORC_BC_INVISCID_WALL, ORC_BC_SMART};
  for (int o = 0; o < 6; ++o) {
    for (int g = 0; g < n_bc; ++g) {
      if (bcs[g].kind != order[o]) continue;
      for (int64_t f = 0; f < m->n_faces; ++f) {
        if (m->face_cells[f * 2 + 1] >= 0 || m->face_group[f] != g) continue;
        int64_t h = m->face_cells[f * 2];
        for (int fp = 0; fp < QF; ++fp) {
          const double *fl = &flux[(f * QF + fp) * K];
          double *rh = r + h * KN + m->map_h[f * QF + fp] * K;
          for (int k = 0; k < K; ++k) rh[k] -= fl[k];
        }
      }
    }
  }
  free(flux);
  /* lumped mass (dg/lobatto.hpp:143-158) */
#pragma omp parallel for schedule(static) num_threads(orc_get_threads())
  for (int64_t c = 0; c < m->n_cells; ++c) {
    for (int q = 0; q < N; ++q) {
      double scale = 1.0 / m->node_w[c * N + q];
      double *rq = r + c * KN + q * K;
      for (int k = 0; k < K; ++k) rq[k] *= scale;
    }
  }
  return 0;
}

/* ---------------- time step ---------------- */

static const double kCfl[5][9] = {
    {1.000},
    {1.000, 0.333},
    {1.000, 0.333, 0.209, 0.130, 0.089, 0.066, 0.051, 0.040, 0.033},
    {1.256, 0.409, 0.209, 0.130, 0.089, 0.066, 0.051, 0.040, 0.033},
    {1.392, 0.464, 0.235, 0.145, 0.100, 0.073, 0.056, 0.045, 0.037},
};

double orc_time_step(const orc_mesh *m, const double *u, double dt_guess,
                     int rk_order, double cfl) {
  const int N = m->n, KN = K * m->n;
  double min_dt = 1.e+100;
#pragma omp parallel for reduction(min : min_dt) schedule(static) num_threads(orc_get_threads())
  for (int64_t c = 0; c < m->n_cells; ++c) {
    double max_speed = 1e-5;
    for (int i = 0; i < N; ++i) {
      double speed = orc_max_speed(u + c * KN + i * K);
      max_speed = fmax(max_speed, speed);
    }
    double dt_c = m->length[c] / max_speed;
    if (dt_c < min_dt) min_dt = dt_c;
  }
  if (cfl <= 0) {
    int ro = rk_order < 0 ? 0 : (rk_order > 4 ? 4 : rk_order);
    int pp = m->p > 8 ? 8 : m->p;
    cfl = kCfl[ro][pp];
  }
  double dt = cfl * min_dt;
  dt = fmin(dt, dt_guess);
  /* fr::Lobatto::GetTimeStep doubles the base step (fr/lobatto.hpp:220-222) */
  if (m->scheme == ORC_SCHEME_FR) dt = fmin(dt_guess, 2.0 * dt);
  return dt;
}

/* ---------------- Runge-Kutta over a generic residual ---------------- */


/* Euler::NextSolution: u_next = u + (R(u) * dt)   (ode.hpp:121-128) */
static void next_solution(orc_residual_fn fn, void *ctx, int64_t L, double t,
                          double dt, const double *u, double *u_next,
                          double *r) {
  fn(ctx, t, u, r);
#pragma omp parallel for schedule(static) num_threads(orc_get_threads())
  for (int64_t i = 0; i < L; ++i) u_next[i] = u[i] + r[i] * dt;
}

int orc_rk_generic(orc_residual_fn fn, void *ctx, int64_t L, int order, double t,
                     double dt, double *u, orc_set_hook hook, void *hook_ctx) {
  double *u_curr = (double *)malloc(sizeof(double) * L);
  double *u_tmp = (double *)malloc(sizeof(double) * L);
  double *r = (double *)malloc(sizeof(double) * L);
  memcpy(u_curr, u, sizeof(double) * L);
  if (order == 1) {
    next_solution(fn, ctx, L, t, dt, u_curr, u, r);
    if (hook) hook(hook_ctx, u);
  } else if (order == 2) {  /* rk.hpp:21-29 */
    next_solution(fn, ctx, L, t, dt, u_curr, u, r);
    if (hook) hook(hook_ctx, u);
    next_solution(fn, ctx, L, t + dt, dt, u, u_tmp, r);
    for (int64_t i = 0; i < L; ++i) {
      double v = u_tmp[i];
      v += u_curr[i];
      v *= 0.5;
      u[i] = v;
    }
    if (hook) hook(hook_ctx, u);
  } else {  /* rk.hpp:31-49 */
    next_solution(fn, ctx, L, t, dt, u_curr, u, r);
    if (hook) hook(hook_ctx, u);
    next_solution(fn, ctx, L, t + dt, dt, u, u_tmp, r);
    for (int64_t i = 0; i < L; ++i) {
      double v = u_curr[i];
      v *= 3;
      v += u_tmp[i];
      v /= 4;
      u[i] = v;
    }
    if (hook) hook(hook_ctx, u);
    next_solution(fn, ctx, L, t + dt / 2, dt, u, u_tmp, r);
    for (int64_t i = 0; i < L; ++i) {
      double v = u_tmp[i];
      v *= 2;
      v += u_curr[i];
      v /= 3;
      u[i] = v;
    }
    if (hook) hook(hook_ctx, u);
  }
  free(u_curr); free(u_tmp); free(r);
  return 0;
}

typedef struct {
  const orc_limiter *l;
  int mode;
  double w0, eps;
} limit_ctx;

static void limit_hook(void *ctx, double *u) {
  limit_ctx *c = (limit_ctx *)ctx;
  orc_limit(c->l, c->mode, c->w0, c->eps, u);
}

typedef struct {
  const orc_mesh *m;
  int riemann, n_bc;
  const orc_bc *bcs;
} dg_ctx;

static int dg_residual_fn(void *ctx, double t, const double *u, double *r) {
  dg_ctx *c = (dg_ctx *)ctx;
  return orc_dgsem_residual(c->m, c->riemann, c->n_bc, c->bcs, t, u, r);
}

int orc_rk_update(const orc_mesh *m, int riemann, int n_bc, const orc_bc *bcs,
                  int order, double t, double dt, double *u) {
  dg_ctx ctx = {m, riemann, n_bc, bcs};
  return orc_rk_generic(dg_residual_fn, &ctx, orc_column_size(m), order, t, dt, u,
                   NULL, NULL);
}

int orc_rk_update_limited(const orc_mesh *m, int riemann, int n_bc,
                          const orc_bc *bcs, int order, double t, double dt,
                          double *u, const orc_limiter *l, int mode, double w0,
                          double eps) {
  dg_ctx ctx = {m, riemann, n_bc, bcs};
  limit_ctx lc = {l, mode, w0, eps};
  return orc_rk_generic(dg_residual_fn, &ctx, orc_column_size(m), order, t, dt, u,
                   (l && mode != ORC_LIMITER_NONE) ? limit_hook : NULL, &lc);
}

typedef struct {
  int64_t n;
  const double *a;
} lin_ctx;

static int lin_residual_fn(void *ctx, double t, const double *u, double *r) {
  (void)t;
  lin_ctx *c = (lin_ctx *)ctx;
  for (int64_t i = 0; i < c->n; ++i) {
    double s = 0;
    for (int64_t j = 0; j < c->n; ++j) s += c->a[i * c->n + j] * u[j];
    r[i] = s;
  }
  return 0;
}

int orc_rk_update_linear(int order, int64_t n, const double *a, double t,
                         double dt, double *u) {
  lin_ctx ctx = {n, a};
  return orc_rk_generic(lin_residual_fn, &ctx, n, order, t, dt, u, NULL, NULL);
}

/* ---- output sampling: Writer<Part>::Prepare (mesh/vtk.hpp:428-493) ---- */

/* VTK Hexahedron27 local coordinates (mesh/vtk.hpp:310-330): corners, edge
 * midpoints, face centres, centre. */
const signed char orc_vtk_hex27[27][3] = {
    {-1, -1, -1}, {1, -1, -1}, {1, 1, -1}, {-1, 1, -1}, {-1, -1, 1}, {1, -1, 1},
    {1, 1, 1},    {-1, 1, 1},  {0, -1, -1}, {1, 0, -1}, {0, 1, -1},  {-1, 0, -1},
    {0, -1, 1},   {1, 0, 1},   {0, 1, 1},  {-1, 0, 1},  {-1, -1, 0}, {1, -1, 0},
    {1, 1, 0},    {-1, 1, 0},  {-1, 0, 0}, {1, 0, 0},   {0, -1, 0},  {0, 1, 0},
    {0, 0, -1},   {0, 0, 1},   {0, 0, 0}};

/* Lagrange basis on the GLL abscissae at s (basis/lagrange.hpp:53-142). */
static void lagrange_values(int q, const double *x, double s, double *l) {
  for (int i = 0; i < q; ++i) {
    double v = 1;
    for (int m = 0; m < q; ++m)
      if (m != i) v *= (s - x[m]) / (x[i] - x[m]);
    l[i] = v;
  }
}

int orc_vtk_sample(const orc_mesh *m, const double *u, double *xyz, double *values) {
  const int Q = m->q, N = m->n;
  for (int64_t c = 0; c < m->n_cells; ++c)
    for (int s = 0; s < 27; ++s) {
      double loc[3] = {orc_vtk_hex27[s][0], orc_vtk_hex27[s][1], orc_vtk_hex27[s][2]};
      double *g = &xyz[(c * 27 + s) * 3], *v = &values[(c * 27 + s) * K];
      double jz[9];
      orc_map_point(m->type[c], &m->corners[c * 81], loc, g, jz);
      double lx[MAXQ], ly[MAXQ], lz[MAXQ];
      lagrange_values(Q, m->xq, loc[0], lx);
      lagrange_values(Q, m->xq, loc[1], ly);
      lagrange_values(Q, m->xq, loc[2], lz);
      for (int k = 0; k < K; ++k) v[k] = 0;
      for (int i = 0; i < Q; ++i)
        for (int j = 0; j < Q; ++j)
          for (int kk = 0; kk < Q; ++kk) {
            const double w = lx[i] * ly[j] * lz[kk];
            const double *un = &u[(c * N + (i * Q + j) * Q + kk) * K];
            for (int k = 0; k < K; ++k) v[k] += w * un[k];
          }
    }
  return 0;
}
