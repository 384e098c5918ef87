/*
 * ORACLE (test infrastructure only): energy-based artificial viscosity on
 * fr::Lobatto over Hex8 cells, restated from the reference project.  The
 * product library never calls it.
 *
 *   EnergyBasedViscosity        include/mini/spatial/viscosity.hpp:35-602
 *     damping matrices          :299-384 (columns from the residual of one
 *                               cell with nu = 1 and zero neighbours)
 *     face jump integrals       :446-475
 *     viscosity values, min dt  :477-544, spatial factors :581-601
 *   WithViscosity               include/mini/spatial/with_viscosity.hpp:49-71
 *   DDG common gradient         include/mini/riemann/diffusive/direct.hpp:45-90
 *   viscous fluxes of FR        include/mini/spatial/fr/general.hpp:316-497,
 *                               fr/lobatto.hpp:232-317, spatial/fem.hpp:393-403
 *   distance of a face point    include/mini/spatial/fem.hpp:79-85,
 *                               mesh/part.hpp:118-132 (holder -> sharer)
 *   global gradient / Hessian   include/mini/polynomial/hexahedron.hpp:221-239,
 *                               438-595 (kLocal = false)
 *   Jacobian gradient           include/mini/coordinate/cell.hpp:100-118
 *   initial limiters            include/mini/limiter/average.hpp:11-28,
 *                               limiter/majority.hpp:14-42
 *
 * The demos run it with Diffusion = Direct<Isotropic> whose own property is
 * set to 0 (demo/euler/sourceless.cpp:117), so the base class's viscous flux
 * subtracts 0 * gradient and is left out here.
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

/* axis and sign of each local hex face (fr/lobatto.hpp:81-152) */
static const int kDir[6] = {2, 1, 0, 1, 0, 2};
static const double kSign[6] = {-1, -1, +1, +1, -1, +1};
/* CGNS Hex8 face table (coordinate/hexahedron.hpp:353-390) */
static const int kFace[6][4] = {
    {0, 3, 2, 1}, {0, 1, 5, 4}, {1, 2, 6, 5}, {2, 3, 7, 6}, {0, 4, 7, 3}, {4, 5, 6, 7}};

struct orc_visc {
  const orc_mesh *m;
  double beta0, beta1, time_scale;
  double d2[MAXQ * MAXQ];
  double *jinv;    /* [cells][N][9] J^-1, row-major */
  double *itg;     /* [cells][N][3][9] (d_j J^-1)^T = -(J^-1 d_j J J^-1)^T */
  double *volume;  /* [cells] */
  double *area;    /* [faces] */
  double *dist;    /* [faces][QF] normal . holder_to_sharer */
  int64_t *cell_face; /* [cells][6] face id * 2 + (0 holder, 1 sharer), -1 none */
  double *damping; /* [cells][N][N] */
};

const double *orc_visc_damping(const orc_visc *v) { return v->damping; }

static void mat_inverse(const double *m, double *inv) {
  double det = m[0] * (m[4] * m[8] - m[5] * m[7]) - m[1] * (m[3] * m[8] - m[5] * m[6]) +
               m[2] * (m[3] * m[7] - m[4] * m[6]);
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

static void mat_mul(const double *a, const double *b, double *c) {
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j)
      c[i * 3 + j] = a[i * 3 + 0] * b[0 * 3 + j] + a[i * 3 + 1] * b[1 * 3 + j] +
                     a[i * 3 + 2] * b[2 * 3 + j];
}

/* d_a J of the Hex8 map at loc: (d_a J)[b][e] = sum_v d_a d_b N_v x_v[e]
 * (coordinate/cell.hpp:100-118); d_a d_a N_v = 0 for the trilinear map. */
static void hex8_jacobian_grad(const double *xn, const double *loc, double *dj) {
  memset(dj, 0, sizeof(double) * 27);
  for (int v = 0; v < 8; ++v) {
    double s[3];
    orc_local_of_node(ORC_CELL_HEX8, v, s);
    for (int a = 0; a < 3; ++a)
      for (int b = 0; b < 3; ++b) {
        if (a == b) continue;
        const int c = 3 - a - b;
        const double h = s[a] * s[b] * (1 + s[c] * loc[c]) / 8;
        for (int e = 0; e < 3; ++e) dj[a * 9 + b * 3 + e] += xn[v * 3 + e] * h;
      }
  }
}

/* local gradient g [3][K] and local Hessian hl [6][K] of the nodal field uc
 * [N][K] at node q (GetLocalGradient, GetLocalHessian). */
static void local_derivatives(const orc_visc *v, const double *uc, int q, double *g,
                              double *hl) {
  const orc_mesh *m = v->m;
  const int Q = m->q, QF = m->qf;
  const int i = q / QF, j = (q / Q) % Q, l = q % Q;
  const double *D = m->d, *D2 = v->d2;
  for (int e = 0; e < 3 * K; ++e) g[e] = 0;
  for (int e = 0; e < 6 * K; ++e) hl[e] = 0;
  for (int a = 0; a < Q; ++a)
    for (int b = 0; b < Q; ++b)
      for (int c = 0; c < Q; ++c) {
        const double *un = uc + ((a * Q + b) * Q + c) * K;
        const int on_x = (b == j && c == l), on_y = (a == i && c == l), on_z = (a == i && b == j);
        double w[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
        if (on_x) { w[0] = D[i * Q + a]; w[3] = D2[i * Q + a]; }
        if (on_y) { w[1] = D[j * Q + b]; w[6] = D2[j * Q + b]; }
        if (on_z) { w[2] = D[l * Q + c]; w[8] = D2[l * Q + c]; }
        if (c == l) w[4] = D[i * Q + a] * D[j * Q + b];  /* XY */
        if (b == j) w[5] = D[i * Q + a] * D[l * Q + c];  /* XZ */
        if (a == i) w[7] = D[j * Q + b] * D[l * Q + c];  /* YZ */
        for (int k = 0; k < K; ++k) {
          g[0 * K + k] += w[0] * un[k];
          g[1 * K + k] += w[1] * un[k];
          g[2 * K + k] += w[2] * un[k];
          hl[0 * K + k] += w[3] * un[k];
          hl[1 * K + k] += w[4] * un[k];
          hl[2 * K + k] += w[5] * un[k];
          hl[3 * K + k] += w[6] * un[k];
          hl[4 * K + k] += w[7] * un[k];
          hl[5 * K + k] += w[8] * un[k];
        }
      }
}

/* _GetGlobalHessian (kLocal = false): per component
 * H = J^-1 (sym(hl) J^-T + rows g^T (d_r J^-1)^T). */
static void global_hessian(const double *jinv, const double *itg, const double *g,
                           const double *hl, double *hg) {
  for (int k = 0; k < K; ++k) {
    double s[9] = {hl[0 * K + k], hl[1 * K + k], hl[2 * K + k],
                   hl[1 * K + k], hl[3 * K + k], hl[4 * K + k],
                   hl[2 * K + k], hl[4 * K + k], hl[5 * K + k]};
    double jt[9] = {jinv[0], jinv[3], jinv[6], jinv[1], jinv[4], jinv[7], jinv[2], jinv[5], jinv[8]};
    double t[9], u[9];
    mat_mul(s, jt, t);
    for (int r = 0; r < 3; ++r) {
      const double *it = itg + r * 9;
      for (int b = 0; b < 3; ++b)
        t[r * 3 + b] += g[0 * K + k] * it[0 * 3 + b] + g[1 * K + k] * it[1 * 3 + b] +
                        g[2 * K + k] * it[2 * 3 + b];
    }
    mat_mul(jinv, t, u);
    hg[0 * K + k] = u[0];
    hg[1 * K + k] = u[1];
    hg[2 * K + k] = u[2];
    hg[3 * K + k] = u[4];
    hg[4 * K + k] = u[5];
    hg[5 * K + k] = u[8];
  }
}

/* GetGlobalValueGradientHessian (kLocal = false): gradient J^-1 g; uc is
 * the nodal block [N][K] of cell c. */
static void cell_node_derivatives(const orc_visc *v, const double *uc, int64_t c, int q,
                                  double *gg, double *hg) {
  const orc_mesh *m = v->m;
  const int N = m->n;
  double g[3 * K], hl[6 * K];
  local_derivatives(v, uc, q, g, hl);
  const double *ji = &v->jinv[(c * N + q) * 9];
  for (int d = 0; d < 3; ++d)
    for (int k = 0; k < K; ++k)
      gg[d * K + k] = ji[d * 3 + 0] * g[0 * K + k] + ji[d * 3 + 1] * g[1 * K + k] +
                      ji[d * 3 + 2] * g[2 * K + k];
  global_hessian(ji, &v->itg[(c * N + q) * 27], g, hl, hg);
}

static void node_derivatives(const orc_visc *v, const double *u, int64_t c, int q, double *gg,
                             double *hg) {
  cell_node_derivatives(v, u + c * v->m->n * K, c, q, gg, hg);
}

void orc_visc_node_derivatives(const orc_visc *v, const double *u, int64_t c, int q,
                               double *grad, double *hess) {
  node_derivatives(v, u, c, q, grad, hess);
}

/* Direct::GetCommonGradient with the Hessian penalty (direct.hpp:45-78),
 * dotted with the normal: normal . common_gradient[:, k]. */
static void common_normal_gradient(const double *n, double b0, double b1, const double *ul,
                                   const double *ur, const double *gl, const double *gr,
                                   const double *hl, const double *hr, double *out) {
  double cg[3 * K];
  for (int e = 0; e < 3 * K; ++e) cg[e] = (gl[e] + gr[e]) / 2;
  const double nv[3] = {n[0] * b0, n[1] * b0, n[2] * b0};
  for (int k = 0; k < K; ++k) {
    const double jump = ur[k] - ul[k];
    cg[0 * K + k] += nv[0] * jump;
    cg[1 * K + k] += nv[1] * jump;
    cg[2 * K + k] += nv[2] * jump;
  }
  const double nh[3] = {n[0] * b1, n[1] * b1, n[2] * b1};
  for (int k = 0; k < K; ++k) {
    double hj[6];
    for (int e = 0; e < 6; ++e) hj[e] = hr[e * K + k] - hl[e * K + k];
    cg[0 * K + k] += nh[0] * hj[0];
    cg[0 * K + k] += nh[1] * hj[1];
    cg[0 * K + k] += nh[2] * hj[2];
    cg[1 * K + k] += nh[0] * hj[1];
    cg[1 * K + k] += nh[1] * hj[3];
    cg[1 * K + k] += nh[2] * hj[4];
    cg[2 * K + k] += nh[0] * hj[2];
    cg[2 * K + k] += nh[1] * hj[4];
    cg[2 * K + k] += nh[2] * hj[5];
  }
  for (int k = 0; k < K; ++k)
    out[k] = n[0] * cg[0 * K + k] + n[1] * cg[1 * K + k] + n[2] * cg[2 * K + k];
}

orc_visc *orc_visc_create(const orc_mesh *m, double beta0, double beta1, double time_scale) {
  if (!m || m->scheme != ORC_SCHEME_FR) return NULL;
  for (int64_t c = 0; c < m->n_cells; ++c)
    if (m->type[c] != ORC_CELL_HEX8) return NULL;
  const int Q = m->q, N = m->n, QF = m->qf;
  orc_visc *v = (orc_visc *)calloc(1, sizeof(orc_visc));
  v->m = m;
  v->beta0 = beta0;
  v->beta1 = beta1;
  v->time_scale = time_scale;
  orc_lagrange_second(Q, m->xq, v->d2);
  v->jinv = (double *)malloc(sizeof(double) * m->n_cells * N * 9);
  v->itg = (double *)malloc(sizeof(double) * m->n_cells * N * 27);
  v->volume = (double *)malloc(sizeof(double) * m->n_cells);
  v->area = (double *)malloc(sizeof(double) * (m->n_faces + 1));
  v->dist = (double *)malloc(sizeof(double) * (m->n_faces * QF + 1));
  v->cell_face = (int64_t *)malloc(sizeof(int64_t) * m->n_cells * 6);
  v->damping = (double *)calloc((size_t)m->n_cells * N * N, sizeof(double));
  for (int64_t e = 0; e < m->n_cells * 6; ++e) v->cell_face[e] = -1;
#pragma omp parallel for schedule(static) num_threads(orc_get_threads())
  for (int64_t c = 0; c < m->n_cells; ++c) {
    const double *xn = &m->corners[c * 81];
    double vol = 0;
    for (int q = 0; q < N; ++q) {
      const int i = q / QF, j = (q / Q) % Q, l = q % Q;
      const double loc[3] = {m->xq[i], m->xq[j], m->xq[l]};
      double x[3], J[9], dj[27];
      orc_map_point(ORC_CELL_HEX8, xn, loc, x, J);
      double *ji = &v->jinv[(c * N + q) * 9];
      mat_inverse(J, ji);
      hex8_jacobian_grad(xn, loc, dj);
      for (int r = 0; r < 3; ++r) {
        double a[9], b[9];
        mat_mul(ji, &dj[r * 9], a);
        mat_mul(a, ji, b);
        for (int x0 = 0; x0 < 3; ++x0)
          for (int x1 = 0; x1 < 3; ++x1) v->itg[(c * N + q) * 27 + r * 9 + x0 * 3 + x1] = -b[x1 * 3 + x0];
      }
      vol += m->node_w[c * N + q];
    }
    v->volume[c] = vol;
  }
  for (int64_t f = 0; f < m->n_faces; ++f) {
    const int64_t h = m->face_cells[f * 2], s = m->face_cells[f * 2 + 1];
    double a = 0;
    for (int fp = 0; fp < QF; ++fp) a += m->face_w[f * QF + fp];
    v->area[f] = a;
    v->cell_face[h * 6 + m->face_sides[f * 2]] = f * 2;
    if (s >= 0) v->cell_face[s * 6 + m->face_sides[f * 2 + 1]] = f * 2 + 1;
    /* holder_to_sharer: sharer centre - holder centre, or twice the way to
     * the face centre (Quad4 LocalToGlobal(0, 0)) on a boundary; a periodic
     * sharer is seen through its shift */
    double hs[3];
    const double *ch = &m->cell_center[h * 3];
    if (s >= 0) {
      for (int d = 0; d < 3; ++d)
        hs[d] = (m->cell_center[s * 3 + d] + m->face_shift[f * 3 + d]) - ch[d];
    } else {
      const int side = m->face_sides[f * 2];
      for (int d = 0; d < 3; ++d) {
        double fc = 0;
        for (int w = 0; w < 4; ++w) fc += m->corners[h * 81 + kFace[side][w] * 3 + d];
        fc *= 0.25;
        hs[d] = (fc - ch[d]) * 2;
      }
    }
    for (int fp = 0; fp < QF; ++fp) {
      const double *n = &m->face_frame[(f * QF + fp) * 9];
      v->dist[f * QF + fp] = n[0] * hs[0] + n[1] * hs[1] + n[2] * hs[2];
    }
  }
  /* BuildDampingMatrices: column c of a cell's matrix is the residual of the
   * cell holding the unit state at node c with nu = 1 there and on its
   * neighbours, minus the same residual with nu = 0 (viscosity.hpp:311-339).
   * The probe states (all ones, and zero) have no positive pressure, so the
   * convective part of both residuals is the zero flux of a clamped state
   * and the difference is the viscous operator evaluated below. */
  const double g1 = orc_fr_g_prime(m->p);
#pragma omp parallel for schedule(dynamic, 16) num_threads(orc_get_threads())
  for (int64_t c = 0; c < m->n_cells; ++c) {
    double *cell_u = (double *)malloc(sizeof(double) * N * K);
    double *ft = (double *)malloc(sizeof(double) * N * 3);
    double *res = (double *)malloc(sizeof(double) * N);
    for (int col = 0; col < N; ++col) {
      memset(cell_u, 0, sizeof(double) * N * K);
      for (int k = 0; k < K; ++k) cell_u[col * K + k] = 1;
      for (int q = 0; q < N; ++q) res[q] = 0;
      /* AddFluxDivergence: local flux of -grad(u) (component 0) */
      for (int q = 0; q < N; ++q) {
        const double *gr = &m->grad[((c * N + q) * 3) * N];
        double gu[3] = {0, 0, 0};
        for (int d = 0; d < 3; ++d)
          for (int nb = 0; nb < N; ++nb) gu[d] += gr[d * N + nb] * cell_u[nb * K];
        const double F[3] = {0 - 1 * gu[0], 0 - 1 * gu[1], 0 - 1 * gu[2]};
        const double *jd = &m->jdi[(c * N + q) * 9];
        for (int e = 0; e < 3; ++e) ft[q * 3 + e] = F[0] * jd[0 * 3 + e] + F[1] * jd[1 * 3 + e] + F[2] * jd[2 * 3 + e];
      }
      for (int q = 0; q < N; ++q) {
        const int i = q / QF, j = (q / Q) % Q, l = q % Q;
        double value = 0;
        for (int kb = 0; kb < N; ++kb) {
          const int a = kb / QF, b = (kb / Q) % Q, cc = kb % Q;
          const double g0 = (b == j && cc == l) ? m->d[i * Q + a] : 0;
          const double gy = (a == i && cc == l) ? m->d[j * Q + b] : 0;
          const double gz = (a == i && b == j) ? m->d[l * Q + cc] : 0;
          value += ft[kb * 3 + 0] * g0 + ft[kb * 3 + 1] * gy + ft[kb * 3 + 2] * gz;
        }
        res[q] -= value;
      }
      /* AddFluxToHolder / AddFluxToSharer with the other side zero */
      for (int side = 0; side < 6; ++side) {
        const int64_t cf = v->cell_face[c * 6 + side];
        if (cf < 0) continue;
        const int64_t f = cf / 2;
        const int is_sharer = (int)(cf % 2);
        for (int fp = 0; fp < QF; ++fp) {
          const int nn = is_sharer ? m->map_s[f * QF + fp] : m->map_h[f * QF + fp];
          double gg[3 * K], hg[6 * K], zero_g[3 * K], zero_h[6 * K], zero_u[K], cn[K];
          memset(zero_g, 0, sizeof(zero_g));
          memset(zero_h, 0, sizeof(zero_h));
          memset(zero_u, 0, sizeof(zero_u));
          cell_node_derivatives(v, cell_u, c, nn, gg, hg);
          const double *n = &m->face_frame[(f * QF + fp) * 9];
          const double d = v->dist[f * QF + fp];
          const double b0 = v->beta0 / d, b1 = v->beta1 * d;
          const double *un = cell_u + nn * K;
          if (is_sharer)
            common_normal_gradient(n, b0, b1, zero_u, un, zero_g, gg, zero_h, hg, cn);
          else
            common_normal_gradient(n, b0, b1, un, zero_u, gg, zero_g, hg, zero_h, cn);
          const double f_up = 0 - 1 * cn[0];
          const double *jd = &m->jdi[(c * N + nn) * 9];
          const int dir = kDir[side];
          const double nrm = sqrt(jd[0 * 3 + dir] * jd[0 * 3 + dir] + jd[1 * 3 + dir] * jd[1 * 3 + dir] +
                                  jd[2 * 3 + dir] * jd[2 * 3 + dir]);
          const double scale = kSign[side] * nrm, gp = kSign[side] * g1;
          const double fc = (is_sharer ? f_up * (-scale) : f_up * scale) - ft[nn * 3 + dir];
          res[nn] -= fc * gp;
        }
      }
      for (int q = 0; q < N; ++q) {
        const int i = q / QF, j = (q / Q) % Q, l = q % Q;
        const double det = m->detj[c * N + q];
        double value = res[q] * (1. / det);
        double scale = m->wq[i] * m->wq[j] * m->wq[l];
        scale *= det;
        v->damping[((size_t)c * N + q) * N + col] = value * scale;
      }
    }
    free(cell_u); free(ft); free(res);
  }
  return v;
}

void orc_visc_destroy(orc_visc *v) {
  if (!v) return;
  free(v->jinv); free(v->itg); free(v->volume); free(v->area); free(v->dist);
  free(v->cell_face); free(v->damping);
  free(v);
}

void orc_visc_jumps(const orc_visc *v, const double *u, double *jumps) {
  const orc_mesh *m = v->m;
  const int N = m->n, QF = m->qf;
  memset(jumps, 0, sizeof(double) * m->n_cells * K);
  for (int64_t f = 0; f < m->n_faces; ++f) {
    const int64_t h = m->face_cells[f * 2], s = m->face_cells[f * 2 + 1];
    if (s < 0) continue;
    const double hh = v->volume[h] / v->area[f], hs = v->volume[s] / v->area[f];
    for (int fp = 0; fp < QF; ++fp) {
      const double *uh = u + (h * N + m->map_h[f * QF + fp]) * K;
      const double *us = u + (s * N + m->map_s[f * QF + fp]) * K;
      const double w = m->face_w[f * QF + fp];
      for (int k = 0; k < K; ++k) {
        double jump = uh[k] - us[k];
        jump *= jump;
        jumps[h * K + k] += jump * (w * hh);
        jumps[s * K + k] += jump * (w * hs);
      }
    }
  }
}

static double spatial_factor(int p) {
  static const double kF[7] = {1., 4., 10., 40., 28., 50., 90.};
  return (p >= 0 && p < 7) ? kF[p] : -1;
}

void orc_visc_properties(const orc_visc *v, const double *u, double *nu, double *min_dt_out) {
  const orc_mesh *m = v->m;
  const int N = m->n, P = m->p;
  double *jumps = (double *)malloc(sizeof(double) * m->n_cells * K);
  orc_visc_jumps(v, u, jumps);
  double min_dt = 1.e+100;
#pragma omp parallel for schedule(static) reduction(min : min_dt) num_threads(orc_get_threads())
  for (int64_t c = 0; c < m->n_cells; ++c) {
    const double *uc = u + c * N * K;
    double max_speed = 1e-5, max_sq[K];
    for (int k = 0; k < K; ++k) max_sq[k] = 1e-5;
    for (int i = 0; i < N; ++i) {
      const double *ui = uc + i * K;
      double sq[K];
      sq[0] = ui[0] * ui[0];
      sq[4] = ui[4] * ui[4];
      const double speed = orc_max_speed(ui);
      for (int d = 1; d < 4; ++d) sq[d] = sq[0] * speed * speed;
      max_speed = (max_speed < speed) ? speed : max_speed;
      for (int k = 0; k < K; ++k) max_sq[k] = (max_sq[k] < sq[k]) ? sq[k] : max_sq[k];
    }
    const double L = m->length[c];
    double t0 = L / max_speed;
    min_dt = (t0 < min_dt) ? t0 : min_dt;
    const double max_viscosity = max_speed * L / P;
    const double time_base = L / max_speed;
    const double lp = pow(L, (P + 1) + 3);
    for (int k = 0; k < K; ++k) max_sq[k] *= lp;
    for (int k = 0; k < K; ++k) {
      if (jumps[c * K + k] < max_sq[k]) {
        nu[c * K + k] = 0.;
        continue;
      }
      const double *D = &v->damping[(size_t)c * N * N];
      double rate = 0;
      for (int r = 0; r < N; ++r) {
        double du = 0;
        for (int cc = 0; cc < N; ++cc) du += D[r * N + cc] * uc[cc * K + k];
        rate += uc[r * K + k] * du;
      }
      rate = -rate;
      const double damping_time = time_base * v->time_scale;
      const double ratio = jumps[c * K + k] / (rate * damping_time);
      const double lo = (0.0 < ratio) ? ratio : 0.0;  /* std::max(0.0, ratio) */
      const double val = (lo < max_viscosity) ? lo : max_viscosity;  /* std::min */
      nu[c * K + k] = val;
      const double t1 = L / (max_speed + spatial_factor(P) * val / L);
      min_dt = (t1 < min_dt) ? t1 : min_dt;
    }
  }
  free(jumps);
  if (min_dt_out) *min_dt_out = min_dt;
}

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

int orc_visc_residual(const orc_visc *v, int riemann, int n_bc, const orc_bc *bcs, double t,
                      const double *u, const double *nu, double *r) {
  const orc_mesh *m = v->m;
  const int Q = m->q, N = m->n, QF = m->qf, KN = K * m->n;
  const int64_t L = orc_column_size(m);
  memset(r, 0, sizeof(double) * L);
  const double g1 = orc_fr_g_prime(m->p);
  double *cflux = (double *)malloc(sizeof(double) * m->n_cells * N * 15);
  /* AddFluxDivergence over GetFluxMatrix with the viscous part
   * (fem.hpp:393-403: flux.row(k) -= nu[k] * grad.col(k)) */
#pragma omp parallel for schedule(static) num_threads(orc_get_threads())
  for (int64_t c = 0; c < m->n_cells; ++c) {
    const double *uc = u + c * KN;
    double *fc = cflux + c * N * 15;
    for (int q = 0; q < N; ++q) {
      double f[15];
      orc_flux_matrix(uc + q * K, f);
      const double *gr = &m->grad[((c * N + q) * 3) * N];
      for (int k = 0; k < K; ++k) {
        double gu[3] = {0, 0, 0};
        for (int d = 0; d < 3; ++d)
          for (int nb = 0; nb < N; ++nb) gu[d] += gr[d * N + nb] * uc[nb * K + k];
        for (int d = 0; d < 3; ++d) f[k * 3 + d] -= nu[c * K + k] * gu[d];
      }
      const double *jd = &m->jdi[(c * N + q) * 9];
      for (int k = 0; k < K; ++k)
        for (int e = 0; e < 3; ++e)
          fc[q * 15 + k * 3 + e] = f[k * 3 + 0] * jd[0 * 3 + e] + f[k * 3 + 1] * jd[1 * 3 + e] +
                                   f[k * 3 + 2] * jd[2 * 3 + e];
    }
    for (int q = 0; q < N; ++q) {
      const int i = q / QF, j = (q / Q) % Q, l = q % Q;
      double value[K] = {0, 0, 0, 0, 0};
      for (int kb = 0; kb < N; ++kb) {
        const int a = kb / QF, b = (kb / Q) % Q, cc = kb % Q;
        const double g0 = (b == j && cc == l) ? m->d[i * Q + a] : 0;
        const double gy = (a == i && cc == l) ? m->d[j * Q + b] : 0;
        const double gz = (a == i && b == j) ? m->d[l * Q + cc] : 0;
        for (int k = 0; k < K; ++k)
          value[k] += fc[kb * 15 + k * 3 + 0] * g0 + fc[kb * 15 + k * 3 + 1] * gy +
                      fc[kb * 15 + k * 3 + 2] * gz;
      }
      for (int k = 0; k < K; ++k) r[c * KN + q * K + k] -= value[k];
    }
  }
  /* face corrections (fr/lobatto.hpp:232-428 over fr/general.hpp:316-515):
   * the upwind fluxes of every face point in parallel, then the corrections
   * in face order */
  double *fup = (double *)malloc(sizeof(double) * (m->n_faces * QF * K + 1));
  char *skip = (char *)calloc(m->n_faces + 1, 1);
#pragma omp parallel for schedule(dynamic, 64) num_threads(orc_get_threads())
  for (int64_t f = 0; f < m->n_faces; ++f) {
    const int64_t h = m->face_cells[f * 2], s = m->face_cells[f * 2 + 1];
    const int g = m->face_group[f];
    if (s < 0 && !(g >= 0 && g < n_bc && bcs[g].kind != ORC_BC_NONE)) { skip[f] = 1; continue; }
    for (int fp = 0; fp < QF; ++fp) {
      const double *fr = &m->face_frame[(f * QF + fp) * 9];
      const int nh = m->map_h[f * QF + fp];
      const double *uh = u + h * KN + nh * K;
      double *flux = &fup[(f * QF + fp) * K];
      if (s >= 0) {
        const int ns = m->map_s[f * QF + fp];
        const double *us = u + s * KN + ns * K;
        orc_flux_rotated(riemann, fr, uh, us, flux);
        double gh[3 * K], hh[6 * K], gs[3 * K], hs[6 * K], cn[K];
        node_derivatives(v, u, h, nh, gh, hh);
        node_derivatives(v, u, s, ns, gs, hs);
        const double d = v->dist[f * QF + fp];
        common_normal_gradient(fr, v->beta0 / d, v->beta1 * d, uh, us, gh, gs, hh, hs, cn);
        for (int k = 0; k < K; ++k) {
          double prop = nu[h * K + k];
          prop += nu[s * K + k];
          prop *= 0.5;
          flux[k] -= prop * cn[k];
        }
      } else if (bcs[g].kind == ORC_BC_NO_SLIP_WALL) {
        /* GetFluxOnNoSlipWall: wall flux minus nu normal . grad(u_holder)
         * (fr/general.hpp:460-476) */
        orc_flux_boundary(riemann, ORC_BC_INVISCID_WALL, fr, uh, uh, flux);
        const double *gr = &m->grad[((h * N + nh) * 3) * N];
        for (int k = 0; k < K; ++k) {
          double gu[3] = {0, 0, 0};
          for (int dd = 0; dd < 3; ++dd)
            for (int nb = 0; nb < N; ++nb) gu[dd] += gr[dd * N + nb] * u[h * KN + nb * K + k];
          flux[k] -= nu[h * K + k] * (fr[0] * gu[0] + fr[1] * gu[1] + fr[2] * gu[2]);
        }
      } else {
        double given[K];
        given_value(&bcs[g], &m->face_xyz[(f * QF + fp) * 3], t, f * QF + fp, given);
        orc_flux_boundary(riemann, bcs[g].kind, fr, uh, given, flux);
      }
    }
  }
  for (int64_t f = 0; f < m->n_faces; ++f) {
    if (skip[f]) continue;
    const int64_t h = m->face_cells[f * 2], s = m->face_cells[f * 2 + 1];
    const int sh = m->face_sides[f * 2], ss = s >= 0 ? m->face_sides[f * 2 + 1] : 0;
    for (int fp = 0; fp < QF; ++fp) {
      const int nh = m->map_h[f * QF + fp];
      const double *flux = &fup[(f * QF + fp) * K];
      {
        const double *jd = &m->jdi[(h * N + nh) * 9];
        const int dir = kDir[sh];
        const double nrm = sqrt(jd[0 * 3 + dir] * jd[0 * 3 + dir] + jd[1 * 3 + dir] * jd[1 * 3 + dir] +
                                jd[2 * 3 + dir] * jd[2 * 3 + dir]);
        const double scale = kSign[sh] * nrm, gp = kSign[sh] * g1;
        for (int k = 0; k < K; ++k) {
          const double fh = flux[k] * scale - cflux[(h * N + nh) * 15 + k * 3 + dir];
          r[h * KN + nh * K + k] -= fh * gp;
        }
      }
      if (s >= 0) {
        const int ns = m->map_s[f * QF + fp];
        const double *jd = &m->jdi[(s * N + ns) * 9];
        const int dir = kDir[ss];
        const double nrm = sqrt(jd[0 * 3 + dir] * jd[0 * 3 + dir] + jd[1 * 3 + dir] * jd[1 * 3 + dir] +
                                jd[2 * 3 + dir] * jd[2 * 3 + dir]);
        const double scale = kSign[ss] * nrm, gp = kSign[ss] * g1;
        for (int k = 0; k < K; ++k) {
          const double fs = flux[k] * (-scale) - cflux[(s * N + ns) * 15 + k * 3 + dir];
          r[s * KN + ns * K + k] -= fs * gp;
        }
      }
    }
  }
  free(fup);
  free(skip);
  free(cflux);
#pragma omp parallel for schedule(static) num_threads(orc_get_threads())
  for (int64_t c = 0; c < m->n_cells; ++c)
    for (int q = 0; q < N; ++q) {
      const double scale = 1.0 / m->detj[c * N + q];
      for (int k = 0; k < K; ++k) r[c * KN + q * K + k] *= scale;
    }
  return 0;
}

static const double kCflTable[5][9] = {
    {1.000},
    {1.000, 0.333},
    {1.000, 0.333, 0.209, 0.130, 0.089, 0.066, 0.051, 0.040, 0.033},
    {1.256, 0.409, 0.209, 0.130, 0.089, 0.066, 0.051, 0.040, 0.033},
    {1.392, 0.464, 0.235, 0.145, 0.100, 0.073, 0.056, 0.045, 0.037},
};

double orc_visc_time_step(const orc_visc *v, const double *u, double dt_guess, int rk_order,
                          double cfl) {
  const orc_mesh *m = v->m;
  double *nu = (double *)malloc(sizeof(double) * m->n_cells * K);
  double min_dt = 0;
  orc_visc_properties(v, u, nu, &min_dt);
  free(nu);
  if (cfl <= 0) {
    const int ro = rk_order < 0 ? 0 : (rk_order > 4 ? 4 : rk_order);
    cfl = kCflTable[ro][m->p > 8 ? 8 : m->p];
  }
  /* fr::Lobatto::GetCflNumber doubles the table (fr/lobatto.hpp:431-433) */
  const double dt = (2 * cfl) * min_dt;
  return fmin(dt, dt_guess);
}

typedef struct {
  const orc_visc *v;
  int riemann, n_bc;
  const orc_bc *bcs;
  double *nu;
} visc_ctx;

static int visc_residual_fn(void *ctx, double t, const double *u, double *r) {
  visc_ctx *c = (visc_ctx *)ctx;
  orc_visc_properties(c->v, u, c->nu, NULL);
  return orc_visc_residual(c->v, c->riemann, c->n_bc, c->bcs, t, u, c->nu, r);
}

int orc_visc_rk_update(const orc_visc *v, int riemann, int n_bc, const orc_bc *bcs, int order,
                       double t, double dt, double *u) {
  visc_ctx ctx = {v, riemann, n_bc, bcs, NULL};
  ctx.nu = (double *)malloc(sizeof(double) * v->m->n_cells * K);
  const int rc = orc_rk_generic(visc_residual_fn, &ctx, orc_column_size(v->m), order, t, dt, u,
                                NULL, NULL);
  free(ctx.nu);
  return rc;
}

int64_t orc_initial_limiter(const orc_mesh *m, int kind, double *u) {
  const int N = m->n;
  int64_t missing = 0;
  if (kind == ORC_INIT_AVERAGE) {
    for (int64_t c = 0; c < m->n_cells; ++c) {
      double *uc = u + c * N * K;
      double avg[K] = {0, 0, 0, 0, 0}, vol = 0;
      for (int q = 0; q < N; ++q) {
        const double w = m->node_w[c * N + q];
        for (int k = 0; k < K; ++k) avg[k] += uc[q * K + k] * w;
      }
      for (int q = 0; q < N; ++q) vol += m->node_w[c * N + q];
      for (int k = 0; k < K; ++k) avg[k] /= vol;
      for (int q = 0; q < N; ++q)
        for (int k = 0; k < K; ++k) uc[q * K + k] = avg[k];
    }
  } else if (kind == ORC_INIT_MAJORITY) {
    if (m->p < 2) return 0;
    for (int64_t c = 0; c < m->n_cells; ++c) {
      double *uc = u + c * N * K;
      double value[K];
      int found_all = 1;
      for (int k = 0; k < K; ++k) {
        int found = 0;
        for (int q = 0; q < N && !found; ++q) {
          const double val = uc[q * K + k];
          int count = 0;
          for (int e = 0; e <= q; ++e) count += (uc[e * K + k] == val);
          if (count * 2 > N) { value[k] = val; found = 1; }
        }
        found_all &= found;
      }
      if (!found_all) { ++missing; continue; }
      for (int q = 0; q < N; ++q)
        for (int k = 0; k < K; ++k) uc[q * K + k] = value[k];
    }
  }
  return missing;
}
