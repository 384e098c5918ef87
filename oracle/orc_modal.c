/*
 * ORACLE (test infrastructure only): modal DG (dg::General over
 * polynomial::Projection) on Hex8, Tet4, Wedge6 and Pyra5 cells (and the
 * curved Hex20 / Hex27 / Tet10 / Wedge15 / Wedge18 / Pyra13 / Pyra14),
 * restated from the reference project.  Parity checker and CPU baseline; the product library
 * never calls it.
 *
 *   residual (volume, faces, boundaries)  spatial/dg/general.hpp:58-202
 *   orchestration                          spatial/fem.hpp:248-307
 *   Projection value / gradient / project  polynomial/projection.hpp:28-176
 *   orthonormal basis                      basis/linear.hpp:86-141,
 *                                          integrator/function.hpp:139-172
 *   Taylor monomials                       basis/taylor.hpp:198-218, 387-472
 *   Gauss-Legendre rules                   integrator/legendre.hpp:40-110
 *   Hex8 / Tet4 / Quad4 / Tri3 maps        coordinate/{hexahedron,tetrahedron,
 *                                          quadrangle,triangle}.hpp
 *   face frames                            coordinate/face.hpp:50-62
 *   quadrature points and weights          integrator/element.hpp:102-115
 *   time step (GetValue(i) for i < M)      spatial/fem.hpp:417-435
 *
 * Quadrature choices (the reference leaves tetrahedra unwired; these are
 * its own rules): Hex8 cells Gauss-Legendre (p+1)^3 and Quad4 faces
 * (p+1)^2; Tet4 cells the 14-point degree-5 rule for p <= 2 and the
 * 24-point degree-6 rule for p = 3; Tri3 faces the 6-point degree-4 rule for
 * p <= 2 and the 12-point degree-6 rule for p = 3
 * (integrator/tetrahedron.hpp:149-275, integrator/triangle.hpp:163-228);
 * Wedge6 cells the triangle rule times Gauss-Legendre p+1 in z, triangle
 * point outer (integrator/wedge.hpp:63-88); Pyra5 cells Gauss-Legendre
 * (p+1)^2 times Gauss-Jacobi (alpha 2, beta 0) p+1 in z, local weight
 * w_x w_y w_z (1 - z)^-2 (integrator/pyramid.hpp:63-91); the Gauss-Jacobi
 * points are the roots of P_{p+1}^(2,0) found by bisection and Newton, the
 * weights 8 / ((1 - x^2) P'(x)^2).
 *
 * Periodic faces (an extension; the reference has none): the sharer's
 * polynomial is evaluated at x - shift.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "orc.h"
#include "orc_internal.h"

#define K ORC_K
#define MAXM 20
#define MAXVQ 64
#define MAXFQ 16

/* ---------------- quadrature rules ---------------- */

static void gauss_rule(int q, double *x, double *w) {
  if (q == 2) {
    double a = sqrt(1.0 / 3.0);
    x[0] = -a; x[1] = a; w[0] = w[1] = 1.0;
  } else if (q == 3) {
    double a = sqrt(0.6);
    x[0] = -a; x[1] = 0.0; x[2] = a;
    w[0] = 5.0 / 9.0; w[1] = 8.0 / 9.0; w[2] = 5.0 / 9.0;
  } else {
    double r = sqrt(1.2);
    double a = sqrt((3 + 2 * r) / 7), b = sqrt((3 - 2 * r) / 7);
    double s = sqrt(30.0);
    x[0] = -a; x[1] = -b; x[2] = b; x[3] = a;
    w[0] = w[3] = (18 - s) / 36;
    w[1] = w[2] = (18 + s) / 36;
  }
}

/* symmetric orbits of the simplex rules, in the reference's point order */
static int orbit_s31(double a, double (*x)[3]) {
  double c = 1 - 3 * a;
  double p[4][3] = {{a, a, a}, {a, a, c}, {a, c, a}, {c, a, a}};
  memcpy(x, p, sizeof(p));
  return 4;
}
static int orbit_s22(double a, double (*x)[3]) {
  double c = (1 - 2 * a) * .5;
  double p[6][3] = {{a, a, c}, {a, c, a}, {a, c, c}, {c, a, a}, {c, a, c}, {c, c, a}};
  memcpy(x, p, sizeof(p));
  return 6;
}
static int orbit_s211(double a, double b, double (*x)[3]) {
  double c = 1 - a - a - b;
  double p[12][3] = {{a, a, b}, {a, a, c}, {a, b, a}, {a, b, c}, {a, c, a}, {a, c, b},
                     {b, a, a}, {b, a, c}, {b, c, a}, {c, a, a}, {c, a, b}, {c, b, a}};
  memcpy(x, p, sizeof(p));
  return 12;
}

/* Tetrahedron rules on the unit simplex (local weights sum to 1/6). */
static int tet_rule(int p, double (*x)[3], double *w) {
  int q = 0;
  if (p <= 2) { /* 14 points, degree 5 */
    static const double a31[2] = {0.31088591926330060979734573376345783,
                                  0.09273525031089122640232391373703061};
    static const double w31[2] = {0.11268792571801585079918565233328633,
                                  0.07349304311636194954371020548632750};
    for (int o = 0; o < 2; ++o) {
      int n = orbit_s31(a31[o], &x[q]);
      for (int i = 0; i < n; ++i) w[q + i] = w31[o];
      q += n;
    }
    int n = orbit_s22(0.04550370412564964949188052627933943, &x[q]);
    for (int i = 0; i < n; ++i) w[q + i] = 0.04254602077708146643806942812025744;
    q += n;
  } else { /* 24 points, degree 6 */
    static const double a31[3] = {0.21460287125915202928883921938628499,
                                  0.04067395853461135311557944895641006,
                                  0.32233789014227551034399447076249213};
    static const double w31[3] = {0.03992275025816749209969062755747998,
                                  0.01007721105532064294801323744593686,
                                  0.05535718154365472209515327785372602};
    for (int o = 0; o < 3; ++o) {
      int n = orbit_s31(a31[o], &x[q]);
      for (int i = 0; i < n; ++i) w[q + i] = w31[o];
      q += n;
    }
    int n = orbit_s211(0.06366100187501752529923552760572698,
                       0.60300566479164914136743113906093969, &x[q]);
    for (int i = 0; i < n; ++i) w[q + i] = 27. / 560.;
    q += n;
  }
  for (int i = 0; i < q; ++i) w[i] /= 6.0;
  return q;
}

/* Triangle rules on the unit simplex (local weights sum to 1/2). */
static int tri_rule(int p, double (*x)[2], double *w) {
  int q = 0;
  static const double a6[2] = {.44594849091596488631832925388305199,
                               .09157621350977074345957146340220151};
  static const double w6[2] = {.22338158967801146569500700843312280,
                               .10995174365532186763832632490021053};
  static const double a12[2] = {.06308901449150222834033160287081916,
                                .24928674517091042129163855310701908};
  static const double w12[3] = {.05084490637020681692093680910686898,
                                .11678627572637936602528961138557944,
                                .08285107561837357519355345642044245};
  const double *a21 = p <= 2 ? a6 : a12;
  for (int o = 0; o < 2; ++o) {
    double a = a21[o], b = 1 - a - a;
    double pts[3][2] = {{a, a}, {a, b}, {b, a}};
    for (int i = 0; i < 3; ++i) {
      x[q][0] = pts[i][0]; x[q][1] = pts[i][1];
      w[q] = p <= 2 ? w6[o] : w12[o];
      ++q;
    }
  }
  if (p > 2) {
    double a = .05314504984481694735324967163139815, b = .31035245103378440541660773395655215;
    double c = 1 - a - b;
    double pts[6][2] = {{a, b}, {a, c}, {b, a}, {b, c}, {c, a}, {c, b}};
    for (int i = 0; i < 6; ++i) {
      x[q][0] = pts[i][0]; x[q][1] = pts[i][1];
      w[q] = w12[2];
      ++q;
    }
  }
  for (int i = 0; i < q; ++i) w[i] /= 2.0;
  return q;
}

/* ---------------- element maps ---------------- */

static const int kHexLocal[8][3] = {
    {-1, -1, -1}, {+1, -1, -1}, {+1, +1, -1}, {-1, +1, -1},
    {-1, -1, +1}, {+1, -1, +1}, {+1, +1, +1}, {-1, +1, +1}};

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

static double hex8_det(const double *xn, const double *loc) {
  double j[9] = {0};
  for (int n = 0; n < 8; ++n) {
    double fx = (1 + kHexLocal[n][0] * loc[0]);
    double fy = (1 + kHexLocal[n][1] * loc[1]);
    double fz = (1 + kHexLocal[n][2] * loc[2]);
    double g[3] = {kHexLocal[n][0] * (fy * fz / 8), kHexLocal[n][1] * (fz * fx / 8),
                   kHexLocal[n][2] * (fx * fy / 8)};
    for (int a = 0; a < 3; ++a)
      for (int b = 0; b < 3; ++b) j[a * 3 + b] += g[a] * xn[n * 3 + b];
  }
  return j[0] * (j[4] * j[8] - j[5] * j[7]) - j[1] * (j[3] * j[8] - j[5] * j[6]) +
         j[2] * (j[3] * j[7] - j[4] * j[6]);
}

static void cross(const double *a, const double *b, double *c) {
  c[0] = a[1] * b[2] - a[2] * b[1];
  c[1] = a[2] * b[0] - a[0] * b[2];
  c[2] = a[0] * b[1] - a[1] * b[0];
}

static double norm3(const double *a) { return sqrt(a[0] * a[0] + a[1] * a[1] + a[2] * a[2]); }

/* ---------------- mesh ---------------- */

int64_t orc_modal_column_size(const orc_modal *m) { return m->n_cells * m->m * K; }
int orc_modal_basis_count(const orc_modal *m) { return m->m; }
int64_t orc_modal_point_count(const orc_modal *m) { return m->vp_off[m->n_cells]; }
int64_t orc_modal_face_point_count(const orc_modal *m) { return m->fp_off[m->n_faces]; }

void orc_modal_destroy(orc_modal *m) {
  if (!m) return;
  free(m->vp_off); free(m->vx); free(m->vw); free(m->center); free(m->s);
  free(m->length); free(m->fp_off); free(m->fx); free(m->fw); free(m->ff);
  free(m->face_cells); free(m->face_group); free(m->face_shift);
  free(m->corners); free(m->type);
  free(m);
}

static int cell_points(int type, int p) {
  if (orc_type_is_wedge(type)) return (p <= 2 ? 6 : 12) * (p + 1);
  if (!orc_type_is_tet(type)) return (p + 1) * (p + 1) * (p + 1);
  return p <= 2 ? 14 : 24;
}

/* points of local face `side` of a cell of the type: quadrangle or triangle */
static int face_points(int type, int side, int p) {
  int v[4];
  if (orc_type_face_corners(type, side, v) == 4) return (p + 1) * (p + 1);
  return p <= 2 ? 6 : 12;
}

/* P_n^(2,0)(x) by the three-term recurrence and its derivative from
 * (2n+a+b)(1-x^2) P_n' = n((a-b) - (2n+a+b)x) P_n + 2(n+a)(n+b) P_{n-1} */
static void jacobi20(int n, double x, double *pn, double *dpn) {
  const double a = 2, b = 0;
  double p0 = 1, p1 = ((a + b + 2) * x + (a - b)) / 2;
  for (int k = 2; k <= n; ++k) {
    const double c = 2 * k + a + b;
    const double p2 = (((c - 1) * (a * a - b * b) + (c - 2) * (c - 1) * c * x) * p1 -
                       2 * (k + a - 1) * (k + b - 1) * c * p0) /
                      (2 * k * (k + a + b) * (c - 2));
    p0 = p1;
    p1 = p2;
  }
  const double c = 2 * n + a + b;
  *pn = p1;
  *dpn = (n * ((a - b) - c * x) * p1 + 2 * (n + a) * (n + b) * p0) / (c * (1 - x * x));
}

/* Gauss-Jacobi rule of the weight (1 - x)^2, n points ascending */
static void gauss_jacobi20(int n, double *x, double *w) {
  int found = 0;
  double xl = -1 + 1e-12, fl, d;
  jacobi20(n, xl, &fl, &d);
  for (int g = 1; g <= 4000 && found < n; ++g) {
    double xr = -1 + 2.0 * g / 4000 - (g == 4000 ? 1e-12 : 0.0), fr;
    jacobi20(n, xr, &fr, &d);
    if ((fl < 0) != (fr < 0)) {
      double lo = xl, hi = xr, flo = fl;
      for (int it = 0; it < 200 && hi - lo > 1e-15; ++it) {
        double mid = 0.5 * (lo + hi), fm;
        jacobi20(n, mid, &fm, &d);
        if ((fm < 0) == (flo < 0)) { lo = mid; flo = fm; } else { hi = mid; }
      }
      double r = 0.5 * (lo + hi);
      for (int it = 0; it < 3; ++it) {
        double f, df;
        jacobi20(n, r, &f, &df);
        if (df != 0) r -= f / df;
      }
      x[found++] = r;
    }
    xl = xr;
    fl = fr;
  }
  for (int i = 0; i < n; ++i) {
    double f, df;
    jacobi20(n, x[i], &f, &df);
    w[i] = 8.0 / ((1 - x[i] * x[i]) * df * df);
  }
}

void orc_gauss_jacobi20(int n, double *x, double *w) { gauss_jacobi20(n, x, w); }

orc_modal *orc_modal_create(int64_t n_nodes, const double *xyz, int64_t n_cells,
                            const int64_t *cell_nodes, const int32_t *cell_type,
                            int32_t stride, int64_t n_faces, const int64_t *face_cells,
                            const int32_t *face_sides, const int32_t *face_group,
                            const double *face_shift, int degree) {
  if (degree < 1 || degree > 3 || n_cells <= 0) return NULL;
  orc_modal *m = (orc_modal *)calloc(1, sizeof(orc_modal));
  const int p = degree, M = orc_modal_count(p), Q = p + 1;
  m->p = p; m->m = M; m->n_cells = n_cells; m->n_faces = n_faces;
  m->vp_off = (int64_t *)malloc(sizeof(int64_t) * (n_cells + 1));
  m->vp_off[0] = 0;
  for (int64_t c = 0; c < n_cells; ++c) {
    int t = cell_type ? cell_type[c] : ORC_CELL_HEX8;
    m->vp_off[c + 1] = m->vp_off[c] + cell_points(t, p);
  }
  int64_t NP = m->vp_off[n_cells];
  m->vx = (double *)malloc(sizeof(double) * NP * 3);
  m->vw = (double *)malloc(sizeof(double) * NP);
  m->center = (double *)malloc(sizeof(double) * n_cells * 3);
  m->s = (double *)calloc(n_cells * M * M, sizeof(double));
  m->length = (double *)malloc(sizeof(double) * n_cells);
  m->corners = (double *)calloc(n_cells * 81, sizeof(double));
  const int64_t NS = stride > 0 ? stride : 8;
  for (int64_t c = 0; c < n_cells; ++c) {
    int t = cell_type ? cell_type[c] : ORC_CELL_HEX8;
    if (orc_type_nodes(t) == 0 || orc_type_nodes(t) > NS) {
      free(m->corners);
      m->corners = NULL;
      orc_modal_destroy(m);
      return NULL;
    }
  }
  m->type = (int32_t *)malloc(sizeof(int32_t) * n_cells);
  double gx[4], gw[4];
  gauss_rule(Q, gx, gw);
  double tx[24][3], tw[24];
  int ntet = tet_rule(p, tx, tw);
  double sx[12][2], sw[12];
  int ntri = tri_rule(p, sx, sw);
  double jx[4], jw[4];
  gauss_jacobi20(Q, jx, jw);
  int bad = 0;
#pragma omp parallel for schedule(static) num_threads(orc_get_threads())
  for (int64_t c = 0; c < n_cells; ++c) {
    int t = cell_type ? cell_type[c] : ORC_CELL_HEX8;
    int nv = orc_type_nodes(t);
    double xn[81];
    for (int v = 0; v < nv; ++v) {
      int64_t id = cell_nodes[c * NS + v];
      if (id < 0 || id >= n_nodes) { bad = 1; id = 0; }
      for (int d = 0; d < 3; ++d) xn[v * 3 + d] = xyz[id * 3 + d];
    }
    memcpy(&m->corners[c * 81], xn, sizeof(double) * 3 * nv);
    m->type[c] = t;
    double *ctr = &m->center[c * 3];
    double *X = &m->vx[m->vp_off[c] * 3], *W = &m->vw[m->vp_off[c]];
    double volume = 0;
    if (t != ORC_CELL_HEX8 && t != ORC_CELL_TET4) {
      /* points and det J from the shape functions; the centre at the type's
       * local centre */
      const int tet = t == ORC_CELL_TET10;
      double cl[3], J[9];
      orc_type_center(t, cl);
      orc_map_point(t, xn, cl, ctr, J);
      int nq = (int)(m->vp_off[c + 1] - m->vp_off[c]);
      for (int q = 0; q < nq; ++q) {
        double loc[3], wl;
        if (tet) {
          loc[0] = tx[q][0]; loc[1] = tx[q][1]; loc[2] = tx[q][2];
          wl = tw[q];
        } else if (orc_type_is_wedge(t)) {
          int i = q / Q, k = q % Q;
          loc[0] = sx[i][0]; loc[1] = sx[i][1]; loc[2] = gx[k];
          wl = sw[i] * gw[k];
        } else if (orc_type_is_pyramid(t)) {
          int i = q / (Q * Q), j = (q / Q) % Q, k = q % Q;
          loc[0] = gx[i]; loc[1] = gx[j]; loc[2] = jx[k];
          wl = gw[i] * gw[j] * jw[k] * pow(1 - jx[k], -2);
        } else {
          int i = q / (Q * Q), j = (q / Q) % Q, k = q % Q;
          loc[0] = gx[i]; loc[1] = gx[j]; loc[2] = gx[k];
          wl = gw[i] * gw[j] * gw[k];
        }
        orc_map_point(t, xn, loc, &X[q * 3], J);
        double det = J[0] * (J[4] * J[8] - J[5] * J[7]) - J[1] * (J[3] * J[8] - J[5] * J[6]) +
                     J[2] * (J[3] * J[7] - J[4] * J[6]);
        if (det == 0) bad = 1;
        W[q] = wl * fabs(det);
        volume += W[q];
      }
    } else if (t == ORC_CELL_HEX8) {
      const double zero[3] = {0, 0, 0};
      hex8_global(xn, zero, ctr);
      for (int i = 0; i < Q; ++i)
        for (int j = 0; j < Q; ++j)
          for (int k = 0; k < Q; ++k) {
            int q = (i * Q + j) * Q + k;
            double loc[3] = {gx[i], gx[j], gx[k]};
            hex8_global(xn, loc, &X[q * 3]);
            W[q] = gw[i] * gw[j] * gw[k] * hex8_det(xn, loc);
            volume += W[q];
          }
    } else {
      /* Tetrahedron4: shapes (x, y, z, 1 - x - y - z); centre at 1/4 */
      double e[3][3], det;
      for (int d = 0; d < 3; ++d) {
        e[0][d] = xn[0 * 3 + d] - xn[3 * 3 + d];
        e[1][d] = xn[1 * 3 + d] - xn[3 * 3 + d];
        e[2][d] = xn[2 * 3 + d] - xn[3 * 3 + d];
      }
      det = e[0][0] * (e[1][1] * e[2][2] - e[1][2] * e[2][1]) -
            e[0][1] * (e[1][0] * e[2][2] - e[1][2] * e[2][0]) +
            e[0][2] * (e[1][0] * e[2][1] - e[1][1] * e[2][0]);
      for (int d = 0; d < 3; ++d) {
        double a = 0.25;
        ctr[d] = xn[0 * 3 + d] * a + xn[1 * 3 + d] * a + xn[2 * 3 + d] * a +
                 xn[3 * 3 + d] * (1.0 - a - a - a);
      }
      for (int q = 0; q < ntet; ++q) {
        double l0 = tx[q][0], l1 = tx[q][1], l2 = tx[q][2];
        double l3 = 1.0 - l0 - l1 - l2;
        for (int d = 0; d < 3; ++d)
          X[q * 3 + d] = xn[0 * 3 + d] * l0 + xn[1 * 3 + d] * l1 +
                         xn[2 * 3 + d] * l2 + xn[3 * 3 + d] * l3;
        W[q] = tw[q] * fabs(det);
        volume += W[q];
      }
    }
    m->length[c] = cbrt(volume) * 0.5;
    int nq = (int)(m->vp_off[c + 1] - m->vp_off[c]);
    double T[MAXVQ * MAXM];
    for (int q = 0; q < nq; ++q) {
      double d[3] = {X[q * 3] - ctr[0], X[q * 3 + 1] - ctr[1], X[q * 3 + 2] - ctr[2]};
      orc_taylor_values(M, d, &T[q * M]);
    }
    orc_orthonormalize(M, nq, T, W, &m->s[c * M * M]);
  }
  /* faces */
  m->fp_off = (int64_t *)malloc(sizeof(int64_t) * (n_faces + 1));
  m->fp_off[0] = 0;
  for (int64_t f = 0; f < n_faces; ++f) {
    int64_t h = face_cells[f * 2];
    int t = (cell_type && h >= 0 && h < n_cells) ? cell_type[h] : ORC_CELL_HEX8;
    int sd = face_sides[f * 2];
    if (sd < 0 || sd >= orc_type_faces(t)) sd = 0;
    m->fp_off[f + 1] = m->fp_off[f] + face_points(t, sd, p);
  }
  int64_t NF = m->fp_off[n_faces];
  m->fx = (double *)malloc(sizeof(double) * (NF * 3 + 1));
  m->fw = (double *)malloc(sizeof(double) * (NF + 1));
  m->ff = (double *)malloc(sizeof(double) * (NF * 9 + 1));
  m->face_cells = (int64_t *)malloc(sizeof(int64_t) * (n_faces * 2 + 1));
  m->face_group = (int32_t *)malloc(sizeof(int32_t) * (n_faces + 1));
  m->face_shift = (double *)calloc(n_faces * 3 + 1, sizeof(double));
  if (n_faces) {
    memcpy(m->face_cells, face_cells, sizeof(int64_t) * n_faces * 2);
    memcpy(m->face_group, face_group, sizeof(int32_t) * n_faces);
    if (face_shift) memcpy(m->face_shift, face_shift, sizeof(double) * n_faces * 3);
  }
#pragma omp parallel for schedule(static) num_threads(orc_get_threads())
  for (int64_t f = 0; f < n_faces; ++f) {
    int64_t h = face_cells[f * 2];
    int side = face_sides[f * 2];
    if (h < 0 || h >= n_cells) { bad = 1; continue; }
    int t = cell_type ? cell_type[h] : ORC_CELL_HEX8;
    double *X = &m->fx[m->fp_off[f] * 3], *W = &m->fw[m->fp_off[f]];
    double *F = &m->ff[m->fp_off[f] * 9];
    int fvs[4] = {0, 0, 0, 0};
    const int nfvs = (side >= 0 && side < orc_type_faces(t)) ? orc_type_face_corners(t, side, fvs) : 0;
    if (t == ORC_CELL_PYRA13 || t == ORC_CELL_PYRA14) {
      /* quadratic pyramid: the face's own Triangle6 / Quadrangle8 / 9 map */
      if (side < 0 || side >= 5) { bad = 1; continue; }
      int fn[9];
      const int n = orc_pyramid_face_nodes(t, side, fn), quad = n != 6;
      double xf[27];
      for (int v = 0; v < n; ++v)
        for (int d = 0; d < 3; ++d) xf[v * 3 + d] = xyz[cell_nodes[h * NS + fn[v]] * 3 + d];
      int nq = quad ? Q * Q : ntri;
      for (int q = 0; q < nq; ++q) {
        double s = quad ? gx[q / Q] : sx[q][0], tt = quad ? gx[q % Q] : sx[q][1];
        double wl = quad ? gw[q / Q] * gw[q % Q] : sw[q];
        double jac[6];
        orc_face_map(n, xf, s, tt, &X[q * 3], &jac[0], &jac[3]);
        double *fr = &F[q * 9];
        cross(&jac[0], &jac[3], &fr[0]);
        double nn = norm3(&fr[0]);
        W[q] = wl * nn;
        for (int d = 0; d < 3; ++d) fr[d] /= nn;
        double tn = norm3(&jac[0]);
        for (int d = 0; d < 3; ++d) fr[3 + d] = jac[d] / tn;
        cross(&fr[0], &fr[3], &fr[6]);
      }
    } else if (t == ORC_CELL_HEX27 || t == ORC_CELL_HEX20 || t == ORC_CELL_TET10 || t == ORC_CELL_WEDGE15 ||
               t == ORC_CELL_WEDGE18) {
      /* quadratic holder through its cell map: face points at the face's local
       * points; tangents J^T dloc/da, J^T dloc/db (quad: corner 0 -> 1,
       * 0 -> 3; triangle: corner 0 - corner 2, corner 1 - corner 2) */
      if (side < 0 || side >= orc_type_faces(t)) { bad = 1; continue; }
      int fv[4];
      const int hex = orc_type_face_corners(t, side, fv) == 4;  /* quadrangle face */
      double lc[4][3], da[3], db[3];
      for (int v = 0; v < (hex ? 4 : 3); ++v) orc_local_of_node(t, fv[v], lc[v]);
      for (int d = 0; d < 3; ++d) {
        da[d] = hex ? (lc[1][d] - lc[0][d]) / 2 : lc[0][d] - lc[2][d];
        db[d] = hex ? (lc[3][d] - lc[0][d]) / 2 : lc[1][d] - lc[2][d];
      }
      int nq = hex ? Q * Q : ntri;
      for (int q = 0; q < nq; ++q) {
        double loc[3], wl;
        if (hex) {
          int i = q / Q, j = q % Q;
          for (int d = 0; d < 3; ++d) loc[d] = lc[0][d] + (gx[i] + 1) * da[d] + (gx[j] + 1) * db[d];
          wl = gw[i] * gw[j];
        } else {
          double x = sx[q][0], y = sx[q][1], z = 1.0 - x - y;
          for (int d = 0; d < 3; ++d) loc[d] = lc[0][d] * x + lc[1][d] * y + lc[2][d] * z;
          wl = sw[q];
        }
        double J[9], jac[6];
        orc_map_point(t, &m->corners[h * 81], loc, &X[q * 3], J);
        for (int d = 0; d < 3; ++d) {
          jac[d] = J[0 * 3 + d] * da[0] + J[1 * 3 + d] * da[1] + J[2 * 3 + d] * da[2];
          jac[3 + d] = J[0 * 3 + d] * db[0] + J[1 * 3 + d] * db[1] + J[2 * 3 + d] * db[2];
        }
        double *fr = &F[q * 9];
        cross(&jac[0], &jac[3], &fr[0]);
        double nn = norm3(&fr[0]);
        W[q] = wl * nn;
        for (int d = 0; d < 3; ++d) fr[d] /= nn;
        double tn = norm3(&jac[0]);
        for (int d = 0; d < 3; ++d) fr[3 + d] = jac[d] / tn;
        cross(&fr[0], &fr[3], &fr[6]);
      }
    } else if (nfvs == 4) {
      /* Quadrangle4 map of the holder's face corners (Hex8, Wedge6, Pyra5) */
      double xn[12];
      for (int v = 0; v < 4; ++v)
        for (int d = 0; d < 3; ++d)
          xn[v * 3 + d] = xyz[cell_nodes[h * NS + fvs[v]] * 3 + d];
      for (int i = 0; i < Q; ++i)
        for (int j = 0; j < Q; ++j) {
          int q = i * Q + j;
          double x = gx[i], y = gx[j], jac[6] = {0};
          X[q * 3] = X[q * 3 + 1] = X[q * 3 + 2] = 0;
          for (int n = 0; n < 4; ++n) {
            double v = (1 + kQuadLocal[n][0] * x) * (1 + kQuadLocal[n][1] * y) / 4;
            double fx = (1 + kQuadLocal[n][0] * x) / 4, fy = (1 + kQuadLocal[n][1] * y) / 4;
            for (int d = 0; d < 3; ++d) {
              X[q * 3 + d] += xn[n * 3 + d] * v;
              jac[d] += kQuadLocal[n][0] * fy * xn[n * 3 + d];
              jac[3 + d] += kQuadLocal[n][1] * fx * xn[n * 3 + d];
            }
          }
          double a = jac[0] * jac[0] + jac[1] * jac[1] + jac[2] * jac[2];
          double b = jac[0] * jac[3] + jac[1] * jac[4] + jac[2] * jac[5];
          double cc = jac[3] * jac[3] + jac[4] * jac[4] + jac[5] * jac[5];
          W[q] = gw[i] * gw[j] * sqrt(a * cc - b * b);
          double *fr = &F[q * 9];
          cross(&jac[0], &jac[3], &fr[0]);
          double nn = norm3(&fr[0]);
          for (int d = 0; d < 3; ++d) fr[d] /= nn;
          double tn = norm3(&jac[0]);
          for (int d = 0; d < 3; ++d) fr[3 + d] = jac[d] / tn;
          cross(&fr[0], &fr[3], &fr[6]);
        }
    } else {
      /* Triangle3 map of the holder's face corners (Tet4, Wedge6, Pyra5) */
      if (nfvs != 3) { bad = 1; continue; }
      double xn[9];
      for (int v = 0; v < 3; ++v)
        for (int d = 0; d < 3; ++d)
          xn[v * 3 + d] = xyz[cell_nodes[h * NS + fvs[v]] * 3 + d];
      /* Triangle3: shapes (x, y, 1 - x - y); Jacobian rows X0 - X2, X1 - X2 */
      double jac[6];
      for (int d = 0; d < 3; ++d) {
        jac[d] = xn[0 * 3 + d] - xn[2 * 3 + d];
        jac[3 + d] = xn[1 * 3 + d] - xn[2 * 3 + d];
      }
      double nrm[3];
      cross(&jac[0], &jac[3], nrm);
      double area2 = norm3(nrm);
      for (int q = 0; q < ntri; ++q) {
        double x = sx[q][0], y = sx[q][1], z = 1.0 - x - y;
        for (int d = 0; d < 3; ++d)
          X[q * 3 + d] = xn[0 * 3 + d] * x + xn[1 * 3 + d] * y + xn[2 * 3 + d] * z;
        W[q] = sw[q] * area2;
        double *fr = &F[q * 9];
        for (int d = 0; d < 3; ++d) fr[d] = nrm[d] / area2;
        double tn = norm3(&jac[0]);
        for (int d = 0; d < 3; ++d) fr[3 + d] = jac[d] / tn;
        cross(&fr[0], &fr[3], &fr[6]);
      }
    }
  }
  if (bad) {
    orc_modal_destroy(m);
    return NULL;
  }
  return m;
}

int orc_modal_points(const orc_modal *m, double *xyz, double *weights) {
  int64_t n = orc_modal_point_count(m);
  if (xyz) memcpy(xyz, m->vx, sizeof(double) * n * 3);
  if (weights) memcpy(weights, m->vw, sizeof(double) * n);
  return 0;
}

int orc_modal_face_points(const orc_modal *m, double *xyz, double *weights,
                          double *frames) {
  int64_t n = orc_modal_face_point_count(m);
  if (xyz) memcpy(xyz, m->fx, sizeof(double) * n * 3);
  if (weights) memcpy(weights, m->fw, sizeof(double) * n);
  if (frames) memcpy(frames, m->ff, sizeof(double) * n * 9);
  return 0;
}

double orc_modal_cell_length(const orc_modal *m, int64_t c) { return m->length[c]; }

/* basis values psi [M] of cell c at x (OrthoNormal::operator()) */
static void basis_at(const orc_modal *m, int64_t c, const double *x, double *psi) {
  const int M = m->m;
  double d[3], t[MAXM];
  for (int e = 0; e < 3; ++e) d[e] = x[e] - m->center[c * 3 + e];
  orc_taylor_values(M, d, t);
  const double *S = &m->s[c * M * M];
  for (int i = 0; i < M; ++i) {
    double s = 0;
    for (int j = 0; j < M; ++j) s += S[i * M + j] * t[j];
    psi[i] = s;
  }
}

/* Projection::GlobalToValue: coeff (K x M, stored [m][k]) * basis(x) */
static void value_at(const orc_modal *m, int64_t c, const double *u,
                     const double *x, double *v, double *psi) {
  const int M = m->m;
  basis_at(m, c, x, psi);
  const double *uc = u + c * M * K;
  for (int k = 0; k < K; ++k) {
    double s = 0;
    for (int i = 0; i < M; ++i) s += uc[i * K + k] * psi[i];
    v[k] = s;
  }
}

int orc_modal_values(const orc_modal *m, const double *u, double *values) {
#pragma omp parallel for schedule(static) num_threads(orc_get_threads())
  for (int64_t c = 0; c < m->n_cells; ++c) {
    double psi[MAXM];
    for (int64_t q = m->vp_off[c]; q < m->vp_off[c + 1]; ++q)
      value_at(m, c, u, &m->vx[q * 3], &values[q * K], psi);
  }
  return 0;
}

/* Projection::Approximate (projection.hpp:28-42): coeff = Integrate(f * basis). */
int orc_modal_project(const orc_modal *m, const double *values, double *u) {
  const int M = m->m;
#pragma omp parallel for schedule(static) num_threads(orc_get_threads())
  for (int64_t c = 0; c < m->n_cells; ++c) {
    double acc[MAXM * K] = {0}, psi[MAXM];
    for (int64_t q = m->vp_off[c]; q < m->vp_off[c + 1]; ++q) {
      basis_at(m, c, &m->vx[q * 3], psi);
      for (int i = 0; i < M; ++i)
        for (int k = 0; k < K; ++k) acc[i * K + k] += values[q * K + k] * psi[i] * m->vw[q];
    }
    memcpy(u + c * M * K, acc, sizeof(double) * M * K);
  }
  return 0;
}

static void given_value(const orc_bc *bc, const double *x, double t, int64_t point, double *v) {
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

/* residual += flux (K) x psi (M) */
static void add_outer(int M, const double *flux, const double *psi, double *r) {
  for (int i = 0; i < M; ++i)
    for (int k = 0; k < K; ++k) r[i * K + k] += flux[k] * psi[i];
}

int orc_modal_residual(const orc_modal *m, int riemann, int n_bc,
                       const orc_bc *bcs, double t, const double *u, double *r) {
  const int M = m->m, KM = K * m->m;
  memset(r, 0, sizeof(double) * orc_modal_column_size(m));
  /* AddFluxDivergence (general.hpp:58-69) */
#pragma omp parallel for schedule(static) num_threads(orc_get_threads())
  for (int64_t c = 0; c < m->n_cells; ++c) {
    double *rc = r + c * KM;
    const double *S = &m->s[c * M * M];
    for (int64_t q = m->vp_off[c]; q < m->vp_off[c + 1]; ++q) {
      const double *x = &m->vx[q * 3];
      double v[K], psi[MAXM], f[15];
      value_at(m, c, u, x, v, psi);
      orc_flux_matrix(v, f);
      for (int i = 0; i < 15; ++i) f[i] *= m->vw[q];
      double d[3], g[3 * MAXM], grad[3 * MAXM];
      for (int e = 0; e < 3; ++e) d[e] = x[e] - m->center[c * 3 + e];
      orc_taylor_grad(M, d, g);
      for (int e = 0; e < 3; ++e)
        for (int i = 0; i < M; ++i) {
          double s = 0;
          for (int j = 0; j < M; ++j) s += S[i * M + j] * g[e * M + j];
          grad[e * M + i] = s;
        }
      for (int i = 0; i < M; ++i)
        for (int k = 0; k < K; ++k)
          rc[i * K + k] += f[k * 3 + 0] * grad[0 * M + i] + f[k * 3 + 1] * grad[1 * M + i] +
                           f[k * 3 + 2] * grad[2 * M + i];
    }
  }
  /* face fluxes in parallel, scattered in face order */
  int64_t NF = orc_modal_face_point_count(m);
  double *flux = (double *)malloc(sizeof(double) * (NF * K + 1));
#pragma omp parallel for schedule(static) num_threads(orc_get_threads())
  for (int64_t f = 0; f < m->n_faces; ++f) {
    int64_t h = m->face_cells[f * 2], s = m->face_cells[f * 2 + 1];
    int g = m->face_group[f];
    for (int64_t q = m->fp_off[f]; q < m->fp_off[f + 1]; ++q) {
      const double *x = &m->fx[q * 3];
      double uh[K], psi[MAXM], *out = &flux[q * K];
      value_at(m, h, u, x, uh, psi);
      if (s >= 0) {
        double xs[3], us[K];
        for (int e = 0; e < 3; ++e) xs[e] = x[e] - m->face_shift[f * 3 + e];
        value_at(m, s, u, xs, us, psi);
        orc_flux_rotated(riemann, &m->ff[q * 9], uh, us, out);
      } else if (g >= 0 && g < n_bc && bcs[g].kind != ORC_BC_NONE) {
        double given[K];
        given_value(&bcs[g], x, t, q, given);
        orc_flux_boundary(riemann, bcs[g].kind, &m->ff[q * 9], uh, given, out);
      } else {
        memset(out, 0, sizeof(double) * K);
      }
      for (int k = 0; k < K; ++k) out[k] *= -m->fw[q];
    }
  }
  /* AddFluxToHolderAndSharer (general.hpp:70-89) */
  for (int64_t f = 0; f < m->n_faces; ++f) {
    int64_t h = m->face_cells[f * 2], s = m->face_cells[f * 2 + 1];
    if (s < 0) continue;
    for (int64_t q = m->fp_off[f]; q < m->fp_off[f + 1]; ++q) {
      const double *x = &m->fx[q * 3];
      double psi[MAXM], neg[K], xs[3];
      basis_at(m, h, x, psi);
      add_outer(M, &flux[q * K], psi, r + h * KM);
      for (int e = 0; e < 3; ++e) xs[e] = x[e] - m->face_shift[f * 3 + e];
      basis_at(m, s, xs, psi);
      for (int k = 0; k < K; ++k) neg[k] = -flux[q * K + k];
      add_outer(M, neg, psi, r + s * KM);
    }
  }
  /* boundaries in the order of fem.hpp:260-307 */
  static const int order[6] = {ORC_BC_SUPERSONIC_INLET, ORC_BC_SUPERSONIC_OUTLET,
                               ORC_BC_SUBSONIC_INLET, ORC_BC_SUBSONIC_OUTLET,
                               ORC_BC_INVISCID_WALL, ORC_BC_SMART};
  for (int o = 0; o < 6; ++o)
    for (int g = 0; g < n_bc; ++g) {
      if (bcs[g].kind != order[o]) continue;
      for (int64_t f = 0; f < m->n_faces; ++f) {
        if (m->face_cells[f * 2 + 1] >= 0 || m->face_group[f] != g) continue;
        int64_t h = m->face_cells[f * 2];
        for (int64_t q = m->fp_off[f]; q < m->fp_off[f + 1]; ++q) {
          double psi[MAXM];
          basis_at(m, h, &m->fx[q * 3], psi);
          add_outer(M, &flux[q * K], psi, r + h * KM);
        }
      }
    }
  free(flux);
  return 0;
}

static const double kCflModal[5][9] = {
    {1.000},
    {1.000, 0.333},
    {1.000, 0.333, 0.209, 0.130, 0.089, 0.066, 0.051, 0.040, 0.033},
    {1.256, 0.409, 0.209, 0.130, 0.089, 0.066, 0.051, 0.040, 0.033},
    {1.392, 0.464, 0.235, 0.145, 0.100, 0.073, 0.056, 0.045, 0.037},
};

/* FiniteElement::GetTimeStep: the maximum speed of a cell runs over
 * GetValue(i) for i < Cell::N, which for a Projection is the value at the
 * cell's first M quadrature points (fem.hpp:421-425). */
double orc_modal_time_step(const orc_modal *m, const double *u, double dt_guess,
                           int rk_order, double cfl) {
  double min_dt = 1.e+100;
#pragma omp parallel for reduction(min : min_dt) schedule(static) num_threads(orc_get_threads())
  for (int64_t c = 0; c < m->n_cells; ++c) {
    double max_speed = 1e-5;
    for (int i = 0; i < m->m; ++i) {
      double v[K], psi[MAXM];
      value_at(m, c, u, &m->vx[(m->vp_off[c] + i) * 3], v, psi);
      max_speed = fmax(max_speed, orc_max_speed(v));
    }
    double dt_c = m->length[c] / max_speed;
    if (dt_c < min_dt) min_dt = dt_c;
  }
  if (cfl <= 0) {
    int ro = rk_order < 0 ? 0 : (rk_order > 4 ? 4 : rk_order);
    cfl = kCflModal[ro][m->p];
  }
  return fmin(cfl * min_dt, dt_guess);
}

typedef struct {
  const orc_modal *m;
  int riemann, n_bc;
  const orc_bc *bcs;
} modal_ctx;

static int modal_residual_fn(void *ctx, double t, const double *u, double *r) {
  modal_ctx *c = (modal_ctx *)ctx;
  return orc_modal_residual(c->m, c->riemann, c->n_bc, c->bcs, t, u, r);
}

int orc_modal_rk_update(const orc_modal *m, int riemann, int n_bc,
                        const orc_bc *bcs, int order, double t, double dt,
                        double *u) {
  modal_ctx ctx = {m, riemann, n_bc, bcs};
  return orc_rk_generic(modal_residual_fn, &ctx, orc_modal_column_size(m), order,
                        t, dt, u, NULL, NULL);
}

typedef struct {
  const orc_limiter *l;
  int mode;
  double w0, eps;
} modal_limit_ctx;

static void modal_limit_hook(void *ctx, double *u) {
  modal_limit_ctx *c = (modal_limit_ctx *)ctx;
  orc_limit(c->l, c->mode, c->w0, c->eps, u);
}

int orc_modal_rk_update_limited(const orc_modal *m, int riemann, int n_bc,
                                const orc_bc *bcs, int order, double t, double dt,
                                double *u, const orc_limiter *l, int mode, double w0,
                                double eps) {
  modal_ctx ctx = {m, riemann, n_bc, bcs};
  modal_limit_ctx lc = {l, mode, w0, eps};
  return orc_rk_generic(modal_residual_fn, &ctx, orc_modal_column_size(m), order, t, dt, u,
                        (l && mode != ORC_LIMITER_NONE) ? modal_limit_hook : NULL, &lc);
}

/* ---- output sampling: Writer<Part>::Prepare (mesh/vtk.hpp:428-493) ----
 * Hex8 cells at the VTK Hexahedron27 locals, Tet4 cells at the VTK
 * Tetrahedron10 locals (vtk.hpp:214-224); global point from the cell map,
 * value = Projection::GlobalToValue there.  Points cell by cell. */
extern const signed char orc_vtk_hex27[27][3];
/* Wedge15 locals (vtk.hpp:251-270) */
static const double kWedge15[15][3] = {
    {1, 0, -1}, {0, 1, -1}, {0, 0, -1}, {1, 0, 1}, {0, 1, 1}, {0, 0, 1},
    {0.5, 0.5, -1}, {0, 0.5, -1}, {0.5, 0, -1}, {0.5, 0.5, 1}, {0, 0.5, 1}, {0.5, 0, 1},
    {1, 0, 0}, {0, 1, 0}, {0, 0, 0}};
static const double kTet10[10][3] = {
    {1, 0, 0}, {0, 1, 0}, {0, 0, 1}, {0, 0, 0}, {0.5, 0.5, 0},
    {0, 0.5, 0.5}, {0.5, 0, 0.5}, {0.5, 0, 0}, {0, 0.5, 0}, {0, 0, 0.5}};

int64_t orc_modal_vtk_sample(const orc_modal *m, const double *u, double *xyz,
                             double *values, uint8_t *types) {
  int64_t pt = 0;
  double psi[MAXM];
  for (int64_t c = 0; c < m->n_cells; ++c) {
    const double *xn = &m->corners[c * 81];
    const int tet = orc_type_is_tet(m->type[c]), wedge = orc_type_is_wedge(m->type[c]);
    if (orc_type_is_pyramid(m->type[c])) return -1; /* no pyramid in the writer (vtk.hpp:400-414) */
    types[c] = tet ? 24 : wedge ? 26 : 29;
    const int n = tet ? 10 : wedge ? 15 : 27;
    for (int s = 0; s < n; ++s, ++pt) {
      double *g = &xyz[pt * 3];
      if (m->type[c] != ORC_CELL_HEX8 && m->type[c] != ORC_CELL_TET4) {
        double loc[3], J[9];
        for (int d = 0; d < 3; ++d) loc[d] = tet ? kTet10[s][d] : wedge ? kWedge15[s][d] : orc_vtk_hex27[s][d];
        orc_map_point(m->type[c], xn, loc, g, J);
      } else if (!tet) {
        double loc[3] = {orc_vtk_hex27[s][0], orc_vtk_hex27[s][1], orc_vtk_hex27[s][2]};
        hex8_global(xn, loc, g);
      } else {
        double l0 = kTet10[s][0], l1 = kTet10[s][1], l2 = kTet10[s][2];
        double l3 = 1.0 - l0 - l1 - l2;
        for (int d = 0; d < 3; ++d)
          g[d] = xn[d] * l0 + xn[3 + d] * l1 + xn[6 + d] * l2 + xn[9 + d] * l3;
      }
      value_at(m, c, u, g, &values[pt * K], psi);
    }
  }
  return pt;
}
