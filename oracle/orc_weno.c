/*
 * ORACLE (test infrastructure only): WENO limiter on DGSEM cells, restated
 * from the reference project.  Parity checker and CPU baseline; the product
 * library never calls it.
 *
 *   per-cell modal basis: Taylor monomials about the cell centre
 *       (basis/taylor.hpp:79-218, index order constant/index.hpp via
 *       taylor.hpp:40-55), orthonormalised by the cell's quadrature
 *       (basis/linear.hpp:86-110, integrator/function.hpp:139-172)
 *   nodal <-> modal: modal = nodal * modal_to_nodal, modal_to_nodal[n][m] =
 *       w_n psi_m(x_n); nodal = modal evaluated at the nodes
 *       (polynomial/extrapolation.hpp:59-89, 114-125)
 *   projection average and offset: polynomial/projection.hpp:45-51, 260-264
 *   smoothness beta: limiter/weno.hpp:25-95
 *   Lazy reconstruct: limiter/weno.hpp:97-195
 *   Eigen (jump) detector: limiter/weno.hpp:230-258
 *   Eigen characteristic-wise reconstruction: limiter/weno.hpp:259-348,
 *       EigenMatrices riemann/euler/eigen.hpp:27-56 in the frame of the
 *       face's first quadrature point (rotated/euler.hpp:330-338)
 *   detect all, reconstruct all, then write back: limiter/reconstruct.hpp:21-54
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "orc.h"
#include "orc_internal.h"

#define K ORC_K

/* exponents (x, y, z) of the Taylor monomials in the reference's order */
static const int kTaylorExp[20][3] = {
    {0, 0, 0},
    {1, 0, 0}, {0, 1, 0}, {0, 0, 1},
    {2, 0, 0}, {1, 1, 0}, {1, 0, 1}, {0, 2, 0}, {0, 1, 1}, {0, 0, 2},
    {3, 0, 0}, {2, 1, 0}, {2, 0, 1}, {1, 2, 0}, {1, 1, 1}, {1, 0, 2},
    {0, 3, 0}, {0, 2, 1}, {0, 1, 2}, {0, 0, 3}};

int orc_modal_count(int p) { return (p + 1) * (p + 2) * (p + 3) / 6; }

static double ipow(double x, int e) {
  double r = 1;
  for (int i = 0; i < e; ++i) r *= x;
  return r;
}

void orc_taylor_values(int M, const double *d, double *t) {
  for (int j = 0; j < M; ++j)
    t[j] = ipow(d[0], kTaylorExp[j][0]) * ipow(d[1], kTaylorExp[j][1]) *
           ipow(d[2], kTaylorExp[j][2]);
}

/* Taylor::GetGradValue with the identity coefficient: g[d][j] = d T_j / d x_d. */
void orc_taylor_grad(int M, const double *d, double *g) {
  for (int dd = 0; dd < 3; ++dd)
    for (int j = 0; j < M; ++j) {
      int e = kTaylorExp[j][dd];
      if (e == 0) { g[dd * M + j] = 0; continue; }
      double v = e;
      for (int o = 0; o < 3; ++o) v *= ipow(d[o], kTaylorExp[j][o] - (o == dd));
      g[dd * M + j] = v;
    }
}

/* OrthoNormalize (integrator/function.hpp:139-172): the lower-triangular S
 * whose rows are the Gram-Schmidt orthonormalised Taylor monomials under the
 * quadrature (T [nq][M] monomial values, w [nq] global weights); S [M][M]. */
void orc_orthonormalize(int M, int nq, const double *T, const double *W, double *S) {
  double A[20 * 20] = {0};
  const int N = nq;
  /* A = Integrate(T T^T) with global weights */
  for (int i = 0; i < M; ++i)
    for (int j = 0; j < M; ++j) {
      double s = 0;
      for (int q = 0; q < N; ++q) s += T[q * M + i] * T[q * M + j] * W[q];
      A[i * M + j] = s;
    }
  /* OrthoNormalize (integrator/function.hpp:139-172) */
  for (int i = 0; i < M; ++i)
    for (int j = 0; j < M; ++j) S[i * M + j] = (i == j);
  S[0] = 1 / sqrt(A[0]);
  for (int i = 1; i < M; ++i) {
    for (int j = 0; j < i; ++j) {
      double temp = 0;
      for (int k = 0; k <= j; ++k) temp += S[j * M + k] * A[k * M + i];
      for (int ll = 0; ll <= j; ++ll) S[i * M + ll] -= temp * S[j * M + ll];
    }
    double norm_sq = 0;
    for (int j = 0; j <= i; ++j) {
      double sum = 0, sij = S[i * M + j];
      for (int k = 0; k < j; ++k) sum += 2 * S[i * M + k] * A[k * M + j];
      norm_sq += sij * (sij * A[j * M + j] + sum);
    }
    double inv = sqrt(norm_sq);
    for (int j = 0; j < M; ++j) S[i * M + j] /= inv;
  }
}

static double falling(int e, int a) { /* e! / (e - a)! */
  double r = 1;
  for (int i = 0; i < a; ++i) r *= (e - i);
  return r;
}

/* GetPartialDerivatives: column a = d^alpha_a p (x), column 0 = 0. */
static void taylor_pdv(int M, const double *d, const double *tc, double *out) {
  out[0] = 0;
  for (int a = 1; a < M; ++a) {
    double s = 0;
    for (int j = 0; j < M; ++j) {
      int ok = 1;
      double f = 1;
      for (int dd = 0; dd < 3; ++dd) {
        int e = kTaylorExp[j][dd], al = kTaylorExp[a][dd];
        if (e < al) { ok = 0; break; }
        f *= falling(e, al) * ipow(d[dd], e - al);
      }
      if (ok) s += tc[j] * f;
    }
    out[a] = s;
  }
}

static int degree_of(int j) {
  return kTaylorExp[j][0] + kTaylorExp[j][1] + kTaylorExp[j][2];
}

struct orc_limiter {
  int p, n, m;
  int64_t n_cells;
  int modal_column; /* 1: the column holds the modal coefficients [cells][M][K]
                       (dg::General over Projection); 0: nodal values [cells][N][K]
                       with Extrapolation (DGSEM) */
  int64_t *off;    /* [cells + 1] quadrature points of cell c: off[c] .. off[c+1]-1
                      (DGSEM: its N nodes; modal: its volume quadrature) */
  double *center;  /* [cells][3] */
  double *s;       /* [cells][M][M] lower triangular */
  double *psi;     /* [points][M] basis values at the cell's own points */
  double *w;       /* [points] global weights */
  double *xyz;     /* [points][3] */
  double *volume;  /* [cells] */
  int *adj;        /* [cells][6] */
  int *n_adj;      /* [cells] */
  double *adj_shift; /* [cells][6][3]: a point x of this cell is x - shift in
                        the neighbour's frame (periodic faces; the reference
                        has none, so its shift is always zero) */
  double *adj_frame; /* [cells][6][9]: normal frame of the shared face at its
                        first quadrature point (holder -> sharer) */
};

orc_limiter *orc_limiter_create(const orc_mesh *mesh) {
  const int p = orc_mesh_degree(mesh), N = orc_nodes_per_cell(mesh);
  const int M = orc_modal_count(p);
  const int64_t C = orc_mesh_cells(mesh);
  orc_limiter *l = (orc_limiter *)calloc(1, sizeof(orc_limiter));
  l->p = p; l->n = N; l->m = M; l->n_cells = C;
  l->off = (int64_t *)malloc(sizeof(int64_t) * (C + 1));
  for (int64_t c = 0; c <= C; ++c) l->off[c] = c * N;
  l->center = (double *)malloc(sizeof(double) * C * 3);
  l->s = (double *)calloc(C * M * M, sizeof(double));
  l->psi = (double *)malloc(sizeof(double) * C * N * M);
  l->w = (double *)malloc(sizeof(double) * C * N);
  l->xyz = (double *)malloc(sizeof(double) * C * N * 3);
  l->volume = (double *)malloc(sizeof(double) * C);
  l->adj = (int *)malloc(sizeof(int) * C * 6);
  l->n_adj = (int *)calloc(C, sizeof(int));
  l->adj_shift = (double *)calloc(C * 6 * 3, sizeof(double));
  l->adj_frame = (double *)calloc(C * 6 * 9, sizeof(double));
  const int QF = (p + 1) * (p + 1);
  double *frames = (double *)malloc(sizeof(double) * (orc_mesh_faces(mesh) * QF * 9 + 1));
  orc_face_geometry(mesh, NULL, NULL, frames);
  orc_node_geometry(mesh, l->xyz, l->w);
  orc_cell_centers(mesh, l->center);
  /* adjacency in face order (part.hpp:957-960 appends per local face) */
  const int64_t F = orc_mesh_faces(mesh);
  const int64_t *fc = orc_mesh_face_cells(mesh);
  const double *fs = orc_mesh_face_shift(mesh);
  for (int64_t f = 0; f < F; ++f) {
    int64_t h = fc[f * 2], s = fc[f * 2 + 1];
    if (s < 0) continue;
    if (l->n_adj[h] < 6) {
      for (int e = 0; e < 3; ++e) l->adj_shift[(h * 6 + l->n_adj[h]) * 3 + e] = fs[f * 3 + e];
      memcpy(&l->adj_frame[(h * 6 + l->n_adj[h]) * 9], &frames[f * QF * 9], sizeof(double) * 9);
      l->adj[h * 6 + l->n_adj[h]++] = (int)s;
    }
    if (l->n_adj[s] < 6) {
      for (int e = 0; e < 3; ++e) l->adj_shift[(s * 6 + l->n_adj[s]) * 3 + e] = -fs[f * 3 + e];
      memcpy(&l->adj_frame[(s * 6 + l->n_adj[s]) * 9], &frames[f * QF * 9], sizeof(double) * 9);
      l->adj[s * 6 + l->n_adj[s]++] = (int)h;
    }
  }
  free(frames);
#pragma omp parallel for schedule(static) num_threads(orc_get_threads())
  for (int64_t c = 0; c < C; ++c) {
    double T[64 * 20];
    double *S = &l->s[c * M * M];
    const double *W = &l->w[c * N];
    double vol = 0;
    for (int q = 0; q < N; ++q) {
      double d[3];
      for (int e = 0; e < 3; ++e) d[e] = l->xyz[(c * N + q) * 3 + e] - l->center[c * 3 + e];
      orc_taylor_values(M, d, &T[q * M]);
      vol += W[q];
    }
    l->volume[c] = vol;
    orc_orthonormalize(M, N, T, W, S);
    for (int q = 0; q < N; ++q)
      for (int m = 0; m < M; ++m) {
        double s = 0;
        for (int j = 0; j <= m; ++j) s += S[m * M + j] * T[q * M + j];
        l->psi[(c * N + q) * M + m] = s;
      }
  }
  return l;
}

/* The limiter of WithLimiter<dg::General> over Projection (the reference's
 * DGFEM build, demo/euler/sourceless.hpp:28-32, 74-80): the cells' own
 * orthonormal bases and volume quadratures (any cell type), neighbours in
 * face order, frames of the shared faces at their first quadrature point. */
orc_limiter *orc_modal_limiter_create(const orc_modal *mm) {
  const int p = mm->p, M = mm->m;
  const int64_t C = mm->n_cells, NP = mm->vp_off[C];
  orc_limiter *l = (orc_limiter *)calloc(1, sizeof(orc_limiter));
  l->p = p; l->n = 0; l->m = M; l->n_cells = C; l->modal_column = 1;
  l->off = (int64_t *)malloc(sizeof(int64_t) * (C + 1));
  memcpy(l->off, mm->vp_off, sizeof(int64_t) * (C + 1));
  l->center = (double *)malloc(sizeof(double) * C * 3);
  memcpy(l->center, mm->center, sizeof(double) * C * 3);
  l->s = (double *)malloc(sizeof(double) * C * M * M);
  memcpy(l->s, mm->s, sizeof(double) * C * M * M);
  l->psi = (double *)malloc(sizeof(double) * NP * M);
  l->w = (double *)malloc(sizeof(double) * NP);
  memcpy(l->w, mm->vw, sizeof(double) * NP);
  l->xyz = (double *)malloc(sizeof(double) * NP * 3);
  memcpy(l->xyz, mm->vx, sizeof(double) * NP * 3);
  l->volume = (double *)malloc(sizeof(double) * C);
  l->adj = (int *)malloc(sizeof(int) * C * 6);
  l->n_adj = (int *)calloc(C, sizeof(int));
  l->adj_shift = (double *)calloc(C * 6 * 3, sizeof(double));
  l->adj_frame = (double *)calloc(C * 6 * 9, sizeof(double));
  for (int64_t f = 0; f < mm->n_faces; ++f) {
    int64_t h = mm->face_cells[f * 2], s = mm->face_cells[f * 2 + 1];
    if (s < 0) continue;
    const double *fs = &mm->face_shift[f * 3];
    const double *fr = &mm->ff[mm->fp_off[f] * 9];
    if (l->n_adj[h] < 6) {
      for (int e = 0; e < 3; ++e) l->adj_shift[(h * 6 + l->n_adj[h]) * 3 + e] = fs[e];
      memcpy(&l->adj_frame[(h * 6 + l->n_adj[h]) * 9], fr, sizeof(double) * 9);
      l->adj[h * 6 + l->n_adj[h]++] = (int)s;
    }
    if (l->n_adj[s] < 6) {
      for (int e = 0; e < 3; ++e) l->adj_shift[(s * 6 + l->n_adj[s]) * 3 + e] = -fs[e];
      memcpy(&l->adj_frame[(s * 6 + l->n_adj[s]) * 9], fr, sizeof(double) * 9);
      l->adj[s * 6 + l->n_adj[s]++] = (int)h;
    }
  }
#pragma omp parallel for schedule(static) num_threads(orc_get_threads())
  for (int64_t c = 0; c < C; ++c) {
    const double *S = &l->s[c * M * M];
    double vol = 0;
    for (int64_t q = l->off[c]; q < l->off[c + 1]; ++q) {
      double d[3], t[20];
      for (int e = 0; e < 3; ++e) d[e] = l->xyz[q * 3 + e] - l->center[c * 3 + e];
      orc_taylor_values(M, d, t);
      for (int m = 0; m < M; ++m) {
        double s = 0;
        for (int j = 0; j <= m; ++j) s += S[m * M + j] * t[j];
        l->psi[q * M + m] = s;
      }
      vol += l->w[q];
    }
    l->volume[c] = vol;
  }
  return l;
}

void orc_limiter_destroy(orc_limiter *l) {
  if (!l) return;
  free(l->off); free(l->center); free(l->s); free(l->psi); free(l->w); free(l->xyz);
  free(l->volume); free(l->adj); free(l->n_adj); free(l->adj_shift); free(l->adj_frame);
  free(l);
}

int orc_limiter_modal_count(const orc_limiter *l) { return l->m; }

/* ProjectionWrapper GlobalToValue of cell c with modal coeff cm (K x M). */
static void modal_value(const orc_limiter *l, int64_t c, const double *cm,
                        const double *x, double *v) {
  const int M = l->m;
  double d[3], t[20], psi[20];
  for (int e = 0; e < 3; ++e) d[e] = x[e] - l->center[c * 3 + e];
  orc_taylor_values(M, d, t);
  const double *S = &l->s[c * M * M];
  for (int m = 0; m < M; ++m) {
    double s = 0;
    for (int j = 0; j <= m; ++j) s += S[m * M + j] * t[j];
    psi[m] = s;
  }
  for (int k = 0; k < K; ++k) {
    double s = 0;
    for (int m = 0; m < M; ++m) s += cm[k * M + m] * psi[m];
    v[k] = s;
  }
}

/* UpdateModalCoeff: modal (K x M) = nodal values (K x N) * modal_to_nodal;
 * for the modal scheme the coefficients are the column itself. */
void orc_limiter_modal(const orc_limiter *l, const double *u, double *modal) {
  const int M = l->m;
#pragma omp parallel for schedule(static) num_threads(orc_get_threads())
  for (int64_t c = 0; c < l->n_cells; ++c) {
    for (int k = 0; k < K; ++k)
      for (int m = 0; m < M; ++m) {
        if (l->modal_column) {
          modal[(c * K + k) * M + m] = u[(c * M + m) * K + k];
          continue;
        }
        double s = 0;
        for (int64_t q = l->off[c]; q < l->off[c + 1]; ++q)
          s += u[q * K + k] * (l->w[q] * l->psi[q * M + m]);
        modal[(c * K + k) * M + m] = s;
      }
  }
}

/* GetSmoothness (weno.hpp:78-95) of modal coeff cm on cell c. */
static void smoothness(const orc_limiter *l, int64_t c, const double *cm,
                       double *beta) {
  const int M = l->m, P = l->p;
  const double *S = &l->s[c * M * M];
  double tc[K * 20], integral[K * 20];
  for (int k = 0; k < K; ++k)
    for (int j = 0; j < M; ++j) {
      double s = 0;
      for (int m = j; m < M; ++m) s += cm[k * M + m] * S[m * M + j];
      tc[k * M + j] = s;
    }
  memset(integral, 0, sizeof(integral));
  for (int64_t q = l->off[c]; q < l->off[c + 1]; ++q) {
    double d[3], pdv[20];
    for (int e = 0; e < 3; ++e) d[e] = l->xyz[q * 3 + e] - l->center[c * 3 + e];
    double w = l->w[q];
    for (int k = 0; k < K; ++k) {
      taylor_pdv(M, d, &tc[k * M], pdv);
      for (int a = 0; a < M; ++a) integral[k * M + a] += pdv[a] * pdv[a] * w;
    }
  }
  double s00 = S[0];
  double volume = 1 / (s00 * s00);
  for (int k = 0; k < K; ++k) {
    double b = 0;
    for (int deg = 1; deg <= P; ++deg) {
      double kf = tgamma(deg + 1);
      double weight = pow(volume, deg * 2. / 3 - 1) / (kf * kf);
      double s = 0;
      for (int a = 1; a < M; ++a)
        if (degree_of(a) == deg) s += integral[k * M + a];
      b += s * weight;
    }
    beta[k] = b;
  }
}

void orc_limiter_smoothness(const orc_limiter *l, int64_t c, const double *cm,
                            double *beta) {
  smoothness(l, c, cm, beta);
}

/* weno::Eigen::IsNotSmooth (weno.hpp:230-258). */
static int is_not_smooth(const orc_limiter *l, int64_t c, const double *modal) {
  const int M = l->m, P = l->p;
  const int comps[2] = {0, K - 1};
  const double *cm = &modal[c * K * M];
  double s00 = l->s[c * M * M];
  double max_abs[K], sum_abs[K] = {0, 0, 0, 0, 0}, mine[K];
  for (int k = 0; k < K; ++k) max_abs[k] = cm[k * M] * s00;
  for (int i = 0; i < 2; ++i) max_abs[comps[i]] = fmax(1e-9, fabs(max_abs[comps[i]]));
  modal_value(l, c, cm, &l->center[c * 3], mine);
  for (int a = 0; a < l->n_adj[c]; ++a) {
    int64_t b = l->adj[c * 6 + a];
    const double *cb = &modal[b * K * M];
    const double *sh = &l->adj_shift[(c * 6 + a) * 3];
    double adjv[K], xc[3];
    for (int e = 0; e < 3; ++e) xc[e] = l->center[c * 3 + e] - sh[e];
    modal_value(l, b, cb, xc, adjv);
    double bs00 = l->s[b * M * M];
    for (int i = 0; i < 2; ++i) {
      int k = comps[i];
      sum_abs[k] += fabs(mine[k] - adjv[k]);
      max_abs[k] = fmax(max_abs[k], fabs(cb[k * M] * bs00));
    }
  }
  double volume_power = (P + 1.0) / 2.0 / 3;
  double divisor = pow(l->volume[c], volume_power) * l->n_adj[c];
  double ref = P < 3 ? 1.0 : 3.0;
  for (int i = 0; i < 2; ++i) {
    int k = comps[i];
    if (sum_abs[k] / max_abs[k] / divisor > ref) return 1;
  }
  return 0;
}

/* weno::Lazy::Reconstruct (weno.hpp:125-194) of cell c -> new modal coeff. */
static void lazy_reconstruct(const orc_limiter *l, int64_t c,
                             const double *modal, double w0, double eps,
                             double *out) {
  const int M = l->m;
  const int n_adj = l->n_adj[c];
  double cand[7][K * 20];
  const double *own = &modal[c * K * M];
  double s00 = l->s[c * M * M];
  /* Borrow: neighbours projected onto my basis, shifted to my average */
  for (int a = 0; a < n_adj; ++a) {
    int64_t b = l->adj[c * 6 + a];
    const double *sh = &l->adj_shift[(c * 6 + a) * 3];
    double *pj = cand[a];
    memset(pj, 0, sizeof(double) * K * M);
    for (int64_t q = l->off[c]; q < l->off[c + 1]; ++q) {
      double v[K], xq[3];
      for (int e = 0; e < 3; ++e) xq[e] = l->xyz[q * 3 + e] - sh[e];
      modal_value(l, b, &modal[b * K * M], xq, v);
      double w = l->w[q];
      for (int k = 0; k < K; ++k)
        for (int m = 0; m < M; ++m) pj[k * M + m] += v[k] * l->psi[q * M + m] * w;
    }
    for (int k = 0; k < K; ++k) {
      double my_avg = own[k * M] * s00;
      double adj_avg = pj[k * M] * s00;
      pj[k * M] += (my_avg - adj_avg) / s00;
    }
  }
  memcpy(cand[n_adj], own, sizeof(double) * K * M);
  /* weights */
  double weights[7][K], sum[K] = {0, 0, 0, 0, 0};
  for (int i = 0; i <= n_adj; ++i)
    for (int k = 0; k < K; ++k) weights[i][k] = w0;
  for (int k = 0; k < K; ++k) {
    weights[n_adj][k] *= -n_adj;
    weights[n_adj][k] += 1.0;
  }
  for (int i = 0; i <= n_adj; ++i) {
    double beta[K];
    smoothness(l, c, cand[i], beta);
    for (int k = 0; k < K; ++k) {
      double b = beta[k] + eps;
      b *= b;
      weights[i][k] /= b;
    }
  }
  for (int i = 0; i <= n_adj; ++i)
    for (int k = 0; k < K; ++k) sum[k] += weights[i][k];
  for (int i = 0; i <= n_adj; ++i)
    for (int k = 0; k < K; ++k) weights[i][k] /= sum[k];
  for (int k = 0; k < K; ++k)
    for (int m = 0; m < M; ++m) out[k * M + m] = cand[n_adj][k * M + m] * weights[n_adj][k];
  for (int i = 0; i < n_adj; ++i)
    for (int k = 0; k < K; ++k)
      for (int m = 0; m < M; ++m) out[k * M + m] += cand[i][k * M + m] * weights[i][k];
}

void orc_eigen_matrices(const double *cons, const double *frame9, double *L, double *R) {
  double prim[K];
  orc_cons_to_prim(cons, prim);
  const double *nu = &frame9[0], *mu = &frame9[3], *pi = &frame9[6];
  const double gamma = 1.4;
  double u_x = prim[1], u_y = prim[2], u_z = prim[3];
  double u_nu = (u_x * nu[0] + u_y * nu[1] + u_z * nu[2]);
  double u_mu = (u_x * mu[0] + u_y * mu[1] + u_z * mu[2]);
  double u_pi = (u_x * pi[0] + u_y * pi[1] + u_z * pi[2]);
  double a = sqrt(gamma * prim[4] / prim[0]);
  double ek = (u_x * u_x + u_y * u_y + u_z * u_z) / 2;
  double e0 = a * a * (1 / (gamma - 1));
  double h0 = e0 + ek;
  const double Rc[5][5] = {
      {1, u_x - a * nu[0], u_y - a * nu[1], u_z - a * nu[2], h0 - a * u_nu},
      {1, u_x, u_y, u_z, ek},
      {0, mu[0], mu[1], mu[2], u_mu},
      {0, pi[0], pi[1], pi[2], u_pi},
      {1, u_x + a * nu[0], u_y + a * nu[1], u_z + a * nu[2], h0 + a * u_nu}};
  double b1 = 1 / e0, b2 = b1 * ek;
  const double Lc[5][5] = {
      {(b2 + u_nu / a) / 2, 1 - b2, -u_mu, -u_pi, (b2 - u_nu / a) / 2},
      {-(b1 * u_x + nu[0] / a) / 2, b1 * u_x, mu[0], pi[0], -(b1 * u_x - nu[0] / a) / 2},
      {-(b1 * u_y + nu[1] / a) / 2, b1 * u_y, mu[1], pi[1], -(b1 * u_y - nu[1] / a) / 2},
      {-(b1 * u_z + nu[2] / a) / 2, b1 * u_z, mu[2], pi[2], -(b1 * u_z - nu[2] / a) / 2},
      {b1 / 2, -b1, 0, 0, b1 / 2}};
  /* the reference fills columns: X.col(j) << rows 0..4 */
  for (int i = 0; i < 5; ++i)
    for (int j = 0; j < 5; ++j) {
      R[i * 5 + j] = Rc[j][i];
      L[i * 5 + j] = Lc[j][i];
    }
}

/* weno::Eigen::Reconstruct (weno.hpp:259-348) of cell c -> new modal coeff. */
static void eigen_reconstruct(const orc_limiter *l, int64_t c,
                              const double *modal, double w0, double eps,
                              double *out) {
  const int M = l->m;
  const int n_adj = l->n_adj[c];
  double cand[7][K * 20], rot[7][K * 20];
  const double *own = &modal[c * K * M];
  double s00 = l->s[c * M * M];
  /* Borrow (weno.hpp:275-291), as in Lazy */
  for (int a = 0; a < n_adj; ++a) {
    int64_t b = l->adj[c * 6 + a];
    const double *sh = &l->adj_shift[(c * 6 + a) * 3];
    double *pj = cand[a];
    memset(pj, 0, sizeof(double) * K * M);
    for (int64_t q = l->off[c]; q < l->off[c + 1]; ++q) {
      double v[K], xq[3];
      for (int e = 0; e < 3; ++e) xq[e] = l->xyz[q * 3 + e] - sh[e];
      modal_value(l, b, &modal[b * K * M], xq, v);
      double w = l->w[q];
      for (int k = 0; k < K; ++k)
        for (int m = 0; m < M; ++m) pj[k * M + m] += v[k] * l->psi[q * M + m] * w;
    }
    for (int k = 0; k < K; ++k) {
      double my_avg = own[k * M] * s00;
      double adj_avg = pj[k * M] * s00;
      pj[k * M] += (my_avg - adj_avg) / s00;
    }
  }
  memcpy(cand[n_adj], own, sizeof(double) * K * M);
  double big_u[K];
  for (int k = 0; k < K; ++k) big_u[k] = own[k * M] * s00;
  double acc[K * 20];
  memset(acc, 0, sizeof(acc));
  double total_volume = 0.0;
  /* ReconstructOnFace for every adjacent face (weno.hpp:297-336) */
  for (int f = 0; f < n_adj; ++f) {
    double L[25], R[25];
    orc_eigen_matrices(big_u, &l->adj_frame[(c * 6 + f) * 9], L, R);
    double weights[7][K], sum[K] = {0, 0, 0, 0, 0};
    for (int i = 0; i <= n_adj; ++i)
      for (int k = 0; k < K; ++k) weights[i][k] = w0;
    for (int k = 0; k < K; ++k) {
      weights[n_adj][k] *= -n_adj;
      weights[n_adj][k] += 1.0;
    }
    for (int i = 0; i <= n_adj; ++i) {
      for (int k = 0; k < K; ++k)
        for (int m = 0; m < M; ++m) {
          double s = 0;
          for (int j = 0; j < K; ++j) s += L[k * 5 + j] * cand[i][j * M + m];
          rot[i][k * M + m] = s;
        }
      double beta[K];
      smoothness(l, c, rot[i], beta);
      for (int k = 0; k < K; ++k) {
        double b = beta[k] + eps;
        b *= b;
        weights[i][k] /= b;
      }
    }
    for (int i = 0; i <= n_adj; ++i)
      for (int k = 0; k < K; ++k) sum[k] += weights[i][k];
    for (int i = 0; i <= n_adj; ++i)
      for (int k = 0; k < K; ++k) weights[i][k] /= sum[k];
    double nw[K * 20];
    for (int k = 0; k < K; ++k)
      for (int m = 0; m < M; ++m) nw[k * M + m] = rot[n_adj][k * M + m] * weights[n_adj][k];
    for (int i = 0; i < n_adj; ++i)
      for (int k = 0; k < K; ++k)
        for (int m = 0; m < M; ++m) nw[k * M + m] += rot[i][k * M + m] * weights[i][k];
    double adj_volume = l->volume[l->adj[c * 6 + f]];
    for (int k = 0; k < K; ++k)
      for (int m = 0; m < M; ++m) {
        double s = 0;
        for (int j = 0; j < K; ++j) s += R[k * 5 + j] * nw[j * M + m];
        acc[k * M + m] += s * adj_volume;
      }
    total_volume += adj_volume;
  }
  for (int i = 0; i < K * M; ++i) out[i] = acc[i] / total_volume;
}

/* limiter::Reconstruct (reconstruct.hpp:21-54) in place on the nodal column.
 * mode: ORC_LIMITER_LAZY (every cell) or ORC_LIMITER_DETECT_LAZY (cells the
 * jump detector flags).  Returns the number of reconstructed cells. */
int64_t orc_limit(const orc_limiter *l, int mode, double w0, double eps,
                  double *u) {
  const int M = l->m;
  const int64_t C = l->n_cells;
  double *modal = (double *)malloc(sizeof(double) * C * K * M);
  double *fresh = (double *)malloc(sizeof(double) * C * K * M);
  char *troubled = (char *)calloc(C, 1);
  orc_limiter_modal(l, u, modal);
  int64_t count = 0;
#pragma omp parallel for schedule(dynamic, 16) reduction(+ : count) num_threads(orc_get_threads())
  for (int64_t c = 0; c < C; ++c) {
    troubled[c] = (mode == ORC_LIMITER_LAZY || mode == ORC_LIMITER_EIGEN_ALL)
                      ? 1 : (char)is_not_smooth(l, c, modal);
    if (troubled[c]) {
      if (mode == ORC_LIMITER_EIGEN || mode == ORC_LIMITER_EIGEN_ALL)
        eigen_reconstruct(l, c, modal, w0, eps, &fresh[c * K * M]);
      else
        lazy_reconstruct(l, c, modal, w0, eps, &fresh[c * K * M]);
      ++count;
    }
  }
  /* SetCoeff(modal): the modal column takes the coefficients; with
   * Extrapolation UpdateNodalCoeff sets nodal = modal at the nodes */
#pragma omp parallel for schedule(static) num_threads(orc_get_threads())
  for (int64_t c = 0; c < C; ++c) {
    if (!troubled[c]) continue;
    if (l->modal_column) {
      for (int m = 0; m < M; ++m)
        for (int k = 0; k < K; ++k) u[(c * M + m) * K + k] = fresh[(c * K + k) * M + m];
      continue;
    }
    for (int64_t q = l->off[c]; q < l->off[c + 1]; ++q)
      for (int k = 0; k < K; ++k) {
        double s = 0;
        for (int m = 0; m < M; ++m) s += fresh[(c * K + k) * M + m] * l->psi[q * M + m];
        u[q * K + k] = s;
      }
  }
  free(modal); free(fresh); free(troubled);
  return count;
}

int64_t orc_limiter_troubled(const orc_limiter *l, const double *u, char *flags) {
  const int M = l->m;
  double *modal = (double *)malloc(sizeof(double) * l->n_cells * K * M);
  orc_limiter_modal(l, u, modal);
  int64_t count = 0;
  for (int64_t c = 0; c < l->n_cells; ++c) {
    flags[c] = (char)is_not_smooth(l, c, modal);
    count += flags[c];
  }
  free(modal);
  return count;
}
