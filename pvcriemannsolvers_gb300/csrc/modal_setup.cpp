// Host set-up of the modal DG scheme (dg::General over polynomial::Projection)
// on Hex8, Tet4, Wedge6 and Pyra5 cells (and the curved Hex20 / Hex27 /
// Tet10 / Wedge15 / Wedge18 / Pyra13 / Pyra14; quadratic pyramids take their
// face points from the faces' own Triangle6 / Quadrangle8 / Quadrangle9
// maps, every other curved cell from its cell map): everything the
// reference's Part / Cell / Face
// constructors and OrthoNormal bases compute, built once in FP64 and
// uploaded.
//
//   cell quadrature     Hex8: Gauss-Legendre (p+1)^3 (integrator/legendre.hpp,
//                       integrator/hexahedron.hpp:66-93); Tet4: the 14-point
//                       degree-5 rule for p <= 2 and the 24-point degree-6
//                       rule for p = 3 (integrator/tetrahedron.hpp:149-275);
//                       Wedge6: the triangle rule of the faces (below) times
//                       Gauss-Legendre p+1 in z, triangle point outer
//                       (integrator/wedge.hpp:63-88); Pyra5: Gauss-Legendre
//                       (p+1)^2 times Gauss-Jacobi (alpha 2, beta 0) p+1 in
//                       z with local weight w_x w_y w_z (1 - z)^-2
//                       (integrator/pyramid.hpp:63-91, integrator/jacobi.hpp);
//                       global weight = local weight * det J
//                       (integrator/element.hpp:102-115)
//   face quadrature     Quad4: Gauss-Legendre (p+1)^2; Tri3: the 6-point
//                       degree-4 rule for p <= 2 and the 12-point degree-6
//                       rule for p = 3 (integrator/triangle.hpp:163-228);
//                       points, weights and normals from the face's own
//                       Quadrangle4 / Triangle3 map of the holder's local
//                       face corners (coordinate/face.hpp:50-62) — also for
//                       wedges and pyramids, whose collapsed local cube does
//                       not hold a pyramid's triangles as local triangles;
//                       quadratic cells map their faces through the cell
//   cell centre         Hex8 LocalToGlobal(0, 0, 0); Tet4 LocalToGlobal(1/4,
//                       1/4, 1/4) (coordinate/tetrahedron.hpp:40-44); Wedge6
//                       (1/3, 1/3, 0) (coordinate/wedge.hpp:41-44); Pyra5
//                       (0, 0, -1/2) (coordinate/pyramid.hpp:36-38)
//   orthonormal basis   psi = S T(x - centre), S lower triangular with
//                       S^-1 S^-T the Gram matrix of the Taylor monomials
//                       under the cell quadrature, i.e. S = L^-1 of its
//                       Cholesky factor: the unique lower-triangular
//                       orthonormalisation, the one the reference's
//                       Gram-Schmidt builds (basis/linear.hpp:86-110,
//                       integrator/function.hpp:139-172)
//   length              cbrt(volume) / 2 (mesh/part.hpp:226-230)
//
// Tet4 cells use the first 4 of the 8 cell_nodes slots (CGNS order) and the
// local faces of Tetrahedron4::faces_ (coordinate/tetrahedron.hpp:141-147).
#include <cuda_runtime.h>

#include <algorithm>
#include <array>
#include <climits>
#include <cmath>
#include <cstdint>
#include <string>
#include <vector>

#include "../../include/mcfd.h"
#include "euler.cuh"
#include "geometry.hpp"
#include "handle.hpp"

namespace mcfd {
namespace {

const int kHexLocal[8][3] = {{-1, -1, -1}, {+1, -1, -1}, {+1, +1, -1},
                             {-1, +1, -1}, {-1, -1, +1}, {+1, -1, +1},
                             {+1, +1, +1}, {-1, +1, +1}};
const int kQuadLocal[4][2] = {{-1, -1}, {+1, -1}, {+1, +1}, {-1, +1}};

// exponents of the Taylor monomials in the reference's order
// (basis/taylor.hpp:198-218)
const int kTaylorExp[20][3] = {
    {0, 0, 0}, {1, 0, 0}, {0, 1, 0}, {0, 0, 1}, {2, 0, 0}, {1, 1, 0}, {1, 0, 1},
    {0, 2, 0}, {0, 1, 1}, {0, 0, 2}, {3, 0, 0}, {2, 1, 0}, {2, 0, 1}, {1, 2, 0},
    {1, 1, 1}, {1, 0, 2}, {0, 3, 0}, {0, 2, 1}, {0, 1, 2}, {0, 0, 3}};

double ipow(double x, int e) {
  double r = 1;
  for (int i = 0; i < e; ++i) r *= x;
  return r;
}

void gauss_legendre(int q, double *x, double *w) {
  if (q == 2) {
    double a = std::sqrt(1.0 / 3.0);
    x[0] = -a; x[1] = a; w[0] = w[1] = 1.0;
  } else if (q == 3) {
    double a = std::sqrt(0.6);
    x[0] = -a; x[1] = 0.0; x[2] = a;
    w[0] = 5.0 / 9.0; w[1] = 8.0 / 9.0; w[2] = 5.0 / 9.0;
  } else {
    double r = std::sqrt(1.2), s = std::sqrt(30.0);
    double a = std::sqrt((3 + 2 * r) / 7), b = std::sqrt((3 - 2 * r) / 7);
    x[0] = -a; x[1] = -b; x[2] = b; x[3] = a;
    w[0] = w[3] = (18 - s) / 36;
    w[1] = w[2] = (18 + s) / 36;
  }
}

// Symmetric simplex rules as orbits of barycentric coordinates, in the
// reference's point order.  Tetrahedron: local (x, y, z), 4th coordinate
// 1 - x - y - z, weights summing to 1/6.
struct TetRule {
  std::vector<std::array<double, 3>> x;
  std::vector<double> w;
  void s31(double a, double wt) {
    double c = 1 - 3 * a;
    for (auto p : {std::array<double, 3>{a, a, a}, {a, a, c}, {a, c, a}, {c, a, a}}) add(p, wt);
  }
  void s22(double a, double wt) {
    double c = (1 - 2 * a) * .5;
    for (auto p : {std::array<double, 3>{a, a, c}, {a, c, a}, {a, c, c}, {c, a, a}, {c, a, c}, {c, c, a}})
      add(p, wt);
  }
  void s211(double a, double b, double wt) {
    double c = 1 - a - a - b;
    for (auto p : {std::array<double, 3>{a, a, b}, {a, a, c}, {a, b, a}, {a, b, c},
                   {a, c, a}, {a, c, b}, {b, a, a}, {b, a, c}, {b, c, a}, {c, a, a},
                   {c, a, b}, {c, b, a}})
      add(p, wt);
  }
  void add(const std::array<double, 3> &p, double wt) { x.push_back(p); w.push_back(wt / 6.0); }
};

TetRule tet_rule(int p) {
  TetRule r;
  if (p <= 2) {  // 14 points, degree 5
    r.s31(0.31088591926330060979734573376345783, 0.11268792571801585079918565233328633);
    r.s31(0.09273525031089122640232391373703061, 0.07349304311636194954371020548632750);
    r.s22(0.04550370412564964949188052627933943, 0.04254602077708146643806942812025744);
  } else {       // 24 points, degree 6
    r.s31(0.21460287125915202928883921938628499, 0.03992275025816749209969062755747998);
    r.s31(0.04067395853461135311557944895641006, 0.01007721105532064294801323744593686);
    r.s31(0.32233789014227551034399447076249213, 0.05535718154365472209515327785372602);
    r.s211(0.06366100187501752529923552760572698, 0.60300566479164914136743113906093969, 27. / 560.);
  }
  return r;
}

// Triangle: local (x, y), 3rd coordinate 1 - x - y, weights summing to 1/2.
void tri_rule(int p, std::vector<std::array<double, 2>> *x, std::vector<double> *w) {
  auto s21 = [&](double a, double wt) {
    double b = 1 - a - a;
    for (auto q : {std::array<double, 2>{a, a}, {a, b}, {b, a}}) { x->push_back(q); w->push_back(wt / 2.0); }
  };
  if (p <= 2) {  // 6 points, degree 4
    s21(.44594849091596488631832925388305199, .22338158967801146569500700843312280);
    s21(.09157621350977074345957146340220151, .10995174365532186763832632490021053);
  } else {       // 12 points, degree 6
    s21(.06308901449150222834033160287081916, .05084490637020681692093680910686898);
    s21(.24928674517091042129163855310701908, .11678627572637936602528961138557944);
    double a = .05314504984481694735324967163139815, b = .31035245103378440541660773395655215;
    double c = 1 - a - b;
    for (auto q : {std::array<double, 2>{a, b}, {a, c}, {b, a}, {b, c}, {c, a}, {c, b}}) {
      x->push_back(q);
      w->push_back(.08285107561837357519355345642044245 / 2.0);
    }
  }
}

// Gauss-Jacobi rule for the weight (1 - x)^2 on [-1, 1] (alpha = 2, beta =
// 0) with n points, ascending: the roots of P_n^(2,0) bracketed on a grid and
// polished by bisection and Newton (three-term recurrence and the derivative
// identity (2n+a+b)(1-x^2) P_n' = n ((a-b) - (2n+a+b) x) P_n
// + 2 (n+a)(n+b) P_{n-1}); w_i = 8 / ((1 - x_i^2) P_n'(x_i)^2).
void jacobi20(int n, double x, double *pn, double *dpn) {
  const double a = 2, b = 0;
  double p0 = 1, p1 = ((a + b + 2) * x + (a - b)) / 2;
  if (n == 0) { *pn = 1; *dpn = 0; return; }
  for (int k = 2; k <= n; ++k) {
    const double c = 2 * k + a + b;
    const double a1 = 2 * k * (k + a + b) * (c - 2);
    const double a2 = (c - 1) * (a * a - b * b);
    const double a3 = (c - 2) * (c - 1) * c;
    const double a4 = 2 * (k + a - 1) * (k + b - 1) * c;
    const double p2 = ((a2 + a3 * x) * p1 - a4 * p0) / a1;
    p0 = p1;
    p1 = p2;
  }
  *pn = p1;
  const double c = 2 * n + a + b;
  *dpn = (n * ((a - b) - c * x) * p1 + 2 * (n + a) * (n + b) * p0) / (c * (1 - x * x));
}

void gauss_jacobi20(int n, double *x, double *w) {
  const int grid = 4000;
  int found = 0;
  double xl = -1 + 1e-12, fl, dummy;
  jacobi20(n, xl, &fl, &dummy);
  for (int g = 1; g <= grid && found < n; ++g) {
    const double xr = -1 + 2.0 * g / grid - (g == grid ? 1e-12 : 0.0);
    double fr;
    jacobi20(n, xr, &fr, &dummy);
    if ((fl < 0) != (fr < 0)) {
      double lo = xl, hi = xr, flo = fl;
      for (int it = 0; it < 200 && hi - lo > 1e-15; ++it) {
        const double mid = 0.5 * (lo + hi);
        double fm;
        jacobi20(n, mid, &fm, &dummy);
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

void hex8_map(const double *xn, const double *loc, double *x, double *det) {
  double j[9] = {0};
  x[0] = x[1] = x[2] = 0;
  for (int n = 0; n < 8; ++n) {
    double fx = (1 + kHexLocal[n][0] * loc[0]);
    double fy = (1 + kHexLocal[n][1] * loc[1]);
    double fz = (1 + kHexLocal[n][2] * loc[2]);
    double v = fx * fy * fz / 8;
    double g[3] = {kHexLocal[n][0] * (fy * fz / 8), kHexLocal[n][1] * (fz * fx / 8),
                   kHexLocal[n][2] * (fx * fy / 8)};
    for (int d = 0; d < 3; ++d) {
      x[d] += xn[n * 3 + d] * v;
      for (int a = 0; a < 3; ++a) j[a * 3 + d] += g[a] * xn[n * 3 + d];
    }
  }
  *det = j[0] * (j[4] * j[8] - j[5] * j[7]) - j[1] * (j[3] * j[8] - j[5] * j[6]) +
         j[2] * (j[3] * j[7] - j[4] * j[6]);
}

void cross(const double *a, const double *b, double *c) {
  c[0] = a[1] * b[2] - a[2] * b[1];
  c[1] = a[2] * b[0] - a[0] * b[2];
  c[2] = a[0] * b[1] - a[1] * b[0];
}

double norm3(const double *a) { return std::sqrt(a[0] * a[0] + a[1] * a[1] + a[2] * a[2]); }

int fail(mcfd_handle *h, int code, const std::string &msg) {
  h->err = msg;
  return code;
}

template <class T>
int upload(mcfd_handle *h, T **dst, const std::vector<T> &src) {
  if (src.empty()) { *dst = nullptr; return MCFD_OK; }
  cudaError_t e = cudaMalloc(dst, sizeof(T) * src.size());
  if (e == cudaSuccess) e = cudaMemcpy(*dst, src.data(), sizeof(T) * src.size(), cudaMemcpyHostToDevice);
  if (e != cudaSuccess) return fail(h, MCFD_ERR_CUDA, std::string("modal tables: ") + cudaGetErrorString(e));
  return MCFD_OK;
}

}  // namespace

int build_modal_mesh(mcfd_handle *h, const mcfd_mesh_desc *d, int degree) {
  auto &m = h->mesh;
  auto &md = h->modal;
  const int p = degree, Q = p + 1;
  const int M = (p + 1) * (p + 2) * (p + 3) / 6;
  const int64_t C = d->n_cells, F = d->n_faces;
  md.m = M;
  m.p = p;
  m.q = Q;
  m.n = M;
  m.n_cells = C;
  m.n_faces = F;
  m.column = C * kK * M;
  // ---- cells: types, node ids, point counts
  std::vector<int32_t> type(C), vol_off(C + 1, 0);
  TetRule tet = tet_rule(p);
  std::vector<std::array<double, 2>> tx;
  std::vector<double> tw;
  tri_rule(p, &tx, &tw);
  double jx[8], jw[8];
  gauss_jacobi20(Q, jx, jw);
  const int n_hex_pts = Q * Q * Q, n_tet_pts = (int)tet.w.size();
  const int n_wedge_pts = (int)tw.size() * Q, n_pyra_pts = Q * Q * Q;
  auto n_vol_pts = [&](int t) {
    return geo::is_hex(t) ? n_hex_pts : geo::is_tet(t) ? n_tet_pts : geo::is_wedge(t) ? n_wedge_pts : n_pyra_pts;
  };
  const int64_t NS = d->cell_node_stride > 0 ? d->cell_node_stride : 8;
  for (int64_t c = 0; c < C; ++c) {
    int t = d->cell_type ? d->cell_type[c] : MCFD_HEX8;
    const int nv = geo::node_count(t);
    if (nv == 0) return fail(h, MCFD_ERR_MESH, "unknown cell type in cell " + std::to_string(c));
    if (nv > NS) return fail(h, MCFD_ERR_MESH, "cell_node_stride is below the node count of cell " + std::to_string(c));
    type[c] = t;
    for (int v = 0; v < nv; ++v) {
      int64_t id = d->cell_nodes[c * NS + v];
      if (id < 0 || id >= d->n_nodes)
        return fail(h, MCFD_ERR_MESH, "cell node index out of range in cell " + std::to_string(c));
    }
    int64_t next = (int64_t)vol_off[c] + n_vol_pts(t);
    if (next > INT32_MAX) return fail(h, MCFD_ERR_UNSUPPORTED, "more than 2^31 volume points");
    vol_off[c + 1] = (int32_t)next;
  }
  const int64_t NV = vol_off[C];
  md.n_vol = NV;
  double gx[4], gw[4];
  gauss_legendre(Q, gx, gw);
  std::vector<double4> center(C), vol(NV);
  std::vector<double> S((size_t)C * M * (M + 1) / 2);
  md.host_points.assign((size_t)NV * 3, 0.0);
  int bad_jac = 0, bad_gram = 0;
#pragma omp parallel for schedule(static)
  for (int64_t c = 0; c < C; ++c) {
    double xn[geo::kMaxNodes * 3];
    const int nv = geo::node_count(type[c]);
    for (int v = 0; v < nv; ++v)
      for (int e = 0; e < 3; ++e) xn[v * 3 + e] = d->xyz[d->cell_nodes[c * NS + v] * 3 + e];
    double ctr[3], volume = 0;
    double *X = &md.host_points[(size_t)vol_off[c] * 3];
    std::vector<double> W(vol_off[c + 1] - vol_off[c]);
    if (geo::curved(type[c]) || geo::is_wedge(type[c]) || geo::is_pyramid(type[c])) {
      // x, det J from the shape functions at every point; centre at the
      // type's local centre
      const bool is_t = geo::is_tet(type[c]);
      double J[9], cl[3];
      geo::local_center(type[c], cl);
      geo::map_point(type[c], xn, cl, ctr, J);
      const int nq = (int)W.size();
      for (int q = 0; q < nq; ++q) {
        double loc[3];
        double wl;
        if (is_t) {
          for (int e = 0; e < 3; ++e) loc[e] = tet.x[q][e];
          wl = tet.w[q];
        } else if (geo::is_wedge(type[c])) {
          const int i = q / Q, k = q % Q;
          loc[0] = tx[i][0]; loc[1] = tx[i][1]; loc[2] = gx[k];
          wl = tw[i] * gw[k];
        } else if (geo::is_pyramid(type[c])) {
          const int i = q / (Q * Q), j = (q / Q) % Q, k = q % Q;
          loc[0] = gx[i]; loc[1] = gx[j]; loc[2] = jx[k];
          wl = gw[i] * gw[j] * jw[k] * std::pow(1 - jx[k], -2);
        } else {
          const int i = q / (Q * Q), j = (q / Q) % Q, k = q % Q;
          loc[0] = gx[i]; loc[1] = gx[j]; loc[2] = gx[k];
          wl = gw[i] * gw[j] * gw[k];
        }
        geo::map_point(type[c], xn, loc, &X[q * 3], J);
        const double det = geo::det3(J);
        if (is_t ? !(det != 0) : !(det > 0)) bad_jac = 1;
        W[q] = wl * (is_t ? std::fabs(det) : det);
        volume += W[q];
      }
    } else if (type[c] == MCFD_HEX8) {
      const double zero[3] = {0, 0, 0};
      double det;
      hex8_map(xn, zero, ctr, &det);
      for (int i = 0; i < Q; ++i)
        for (int j = 0; j < Q; ++j)
          for (int k = 0; k < Q; ++k) {
            int q = (i * Q + j) * Q + k;
            double loc[3] = {gx[i], gx[j], gx[k]};
            hex8_map(xn, loc, &X[q * 3], &det);
            if (!(det > 0)) bad_jac = 1;
            W[q] = gw[i] * gw[j] * gw[k] * det;
            volume += W[q];
          }
    } else {
      double e0[3], e1[3], e2[3], cr[3];
      for (int e = 0; e < 3; ++e) {
        e0[e] = xn[0 * 3 + e] - xn[3 * 3 + e];
        e1[e] = xn[1 * 3 + e] - xn[3 * 3 + e];
        e2[e] = xn[2 * 3 + e] - xn[3 * 3 + e];
      }
      cross(e1, e2, cr);
      double det = e0[0] * cr[0] + e0[1] * cr[1] + e0[2] * cr[2];
      if (!(det != 0)) bad_jac = 1;
      for (int e = 0; e < 3; ++e) {
        double a = 0.25;
        ctr[e] = xn[0 * 3 + e] * a + xn[1 * 3 + e] * a + xn[2 * 3 + e] * a +
                 xn[3 * 3 + e] * (1.0 - a - a - a);
      }
      for (int q = 0; q < n_tet_pts; ++q) {
        double l0 = tet.x[q][0], l1 = tet.x[q][1], l2 = tet.x[q][2];
        double l3 = 1.0 - l0 - l1 - l2;
        for (int e = 0; e < 3; ++e)
          X[q * 3 + e] = xn[0 * 3 + e] * l0 + xn[1 * 3 + e] * l1 + xn[2 * 3 + e] * l2 +
                         xn[3 * 3 + e] * l3;
        W[q] = tet.w[q] * std::fabs(det);
        volume += W[q];
      }
    }
    center[c] = make_double4(ctr[0], ctr[1], ctr[2], 1.0 / (std::cbrt(volume) * 0.5));
    const int nq = (int)W.size();
    std::vector<double> T((size_t)nq * M), A((size_t)M * M, 0.0), L((size_t)M * M, 0.0),
        Sc((size_t)M * M, 0.0);
    for (int q = 0; q < nq; ++q) {
      double dd[3] = {X[q * 3] - ctr[0], X[q * 3 + 1] - ctr[1], X[q * 3 + 2] - ctr[2]};
      vol[vol_off[c] + q] = make_double4(dd[0], dd[1], dd[2], W[q]);
      for (int j = 0; j < M; ++j)
        T[q * M + j] = ipow(dd[0], kTaylorExp[j][0]) * ipow(dd[1], kTaylorExp[j][1]) *
                       ipow(dd[2], kTaylorExp[j][2]);
    }
    for (int i = 0; i < M; ++i)
      for (int j = 0; j < M; ++j) {
        double s = 0;
        for (int q = 0; q < nq; ++q) s += T[q * M + i] * T[q * M + j] * W[q];
        A[i * M + j] = s;
      }
    for (int i = 0; i < M; ++i)
      for (int j = 0; j <= i; ++j) {
        double s = A[i * M + j];
        for (int k = 0; k < j; ++k) s -= L[i * M + k] * L[j * M + k];
        if (i == j) {
          if (!(s > 0)) { bad_gram = 1; s = 1; }
          L[i * M + i] = std::sqrt(s);
        } else {
          L[i * M + j] = s / L[j * M + j];
        }
      }
    for (int col = 0; col < M; ++col)
      for (int i = col; i < M; ++i) {
        double s = (i == col) ? 1.0 : 0.0;
        for (int k = col; k < i; ++k) s -= L[i * M + k] * Sc[k * M + col];
        Sc[i * M + col] = s / L[i * M + i];
      }
    double *Sp = &S[(size_t)c * M * (M + 1) / 2];
    for (int i = 0; i < M; ++i)
      for (int j = 0; j <= i; ++j) Sp[i * (i + 1) / 2 + j] = Sc[i * M + j];
  }
  if (md.keep_host) {
    md.host_weights.resize(NV);
    md.host_center.resize((size_t)C * 3);
    md.host_s.assign((size_t)C * M * M, 0.0);
    md.host_volume.assign(C, 0.0);
    md.host_vol_off = vol_off;
    for (int64_t c = 0; c < C; ++c) {
      md.host_center[c * 3] = center[c].x;
      md.host_center[c * 3 + 1] = center[c].y;
      md.host_center[c * 3 + 2] = center[c].z;
      const double *Sp = &S[(size_t)c * M * (M + 1) / 2];
      for (int i = 0; i < M; ++i)
        for (int j = 0; j <= i; ++j) md.host_s[((size_t)c * M + i) * M + j] = Sp[i * (i + 1) / 2 + j];
      for (int32_t q = vol_off[c]; q < vol_off[c + 1]; ++q) {
        md.host_weights[q] = vol[q].w;
        md.host_volume[c] += vol[q].w;
      }
    }
  }
  if (bad_jac) return fail(h, MCFD_ERR_MESH, "non-positive Jacobian in a modal cell");
  if (bad_gram) return fail(h, MCFD_ERR_MESH, "degenerate cell quadrature (Gram matrix not positive)");
  // ---- faces
  std::vector<int2> fcells(F);
  std::vector<int32_t> fgroup(F), face_off(F + 1, 0), cell_faces((size_t)C * 6, -1);
  std::vector<int> n_slot(C, 0);
  std::vector<double4> fshift(std::max<int64_t>(F, 1), make_double4(0, 0, 0, 0));
  int max_group = -1;
  for (int64_t f = 0; f < F; ++f) {
    int64_t hc = d->face_cells[f * 2], sc = d->face_cells[f * 2 + 1];
    int sh = d->face_sides[f * 2], ss = d->face_sides[f * 2 + 1];
    bool ok = hc >= 0 && hc < C && sc < C && hc <= INT32_MAX;
    if (ok) ok = sh >= 0 && sh < geo::face_count(type[hc]);
    int fv[4];
    const int nfv_h = ok ? geo::cell_face_corners(type[hc], sh, fv) : 0;
    if (ok && sc >= 0)
      ok = ss >= 0 && ss < geo::face_count(type[sc]) && geo::cell_face_corners(type[sc], ss, fv) == nfv_h;
    if (!ok) return fail(h, MCFD_ERR_MESH, "bad face record " + std::to_string(f));
    fcells[f] = make_int2((int)hc, (int)sc);
    fgroup[f] = d->face_group ? d->face_group[f] : -1;
    if (sc < 0) max_group = std::max(max_group, fgroup[f]);
    if (d->face_shift)
      fshift[f] = make_double4(d->face_shift[f * 3], d->face_shift[f * 3 + 1], d->face_shift[f * 3 + 2], 0);
    int64_t next = (int64_t)face_off[f] + (nfv_h == 4 ? Q * Q : (int)tw.size());
    if (next > INT32_MAX) return fail(h, MCFD_ERR_UNSUPPORTED, "more than 2^31 face points");
    face_off[f + 1] = (int32_t)next;
    const int64_t owners[2] = {hc, sc};
    for (int side = 0; side < 2; ++side) {
      int64_t c = owners[side];
      if (c < 0) continue;
      if (n_slot[c] >= 6) return fail(h, MCFD_ERR_MESH, "cell " + std::to_string(c) + " has more than 6 faces");
      cell_faces[(size_t)c * 6 + n_slot[c]++] = (int32_t)(f * 2 + side);
    }
  }
  m.n_groups = max_group + 1;
  const int64_t NF = face_off[F];
  md.n_fpts = NF;
  m.n_points = NF;
  std::vector<int32_t> point_face(NF);
  std::vector<double4> fpt(NF), fnrm(NF);
  // tangent (first row of the face map's Jacobian) at each face's first point:
  // with the normal, the frame of that point (coordinate/face.hpp:54-62)
  std::vector<double> ftan0(md.keep_host ? (size_t)F * 3 : 0);
  auto keep_tangent = [&](int64_t f, int q, const double *ta) {
    if (md.keep_host && q == 0)
      for (int e = 0; e < 3; ++e) ftan0[f * 3 + e] = ta[e];
  };
  int bad_face = 0;
#pragma omp parallel for schedule(static)
  for (int64_t f = 0; f < F; ++f) {
    int64_t hc = fcells[f].x, sc = fcells[f].y;
    int sh = d->face_sides[f * 2], ss = d->face_sides[f * 2 + 1];
    int hv[4], sv[4] = {0, 0, 0, 0};
    const int nfv = geo::cell_face_corners(type[hc], sh, hv);
    if (sc >= 0) geo::cell_face_corners(type[sc], ss, sv);
    const bool hex = nfv == 4;  // quadrangle face
    double xn[12], xs[12];
    for (int v = 0; v < nfv; ++v)
      for (int e = 0; e < 3; ++e) {
        xn[v * 3 + e] = d->xyz[d->cell_nodes[hc * NS + hv[v]] * 3 + e];
        if (sc >= 0) xs[v * 3 + e] = d->xyz[d->cell_nodes[sc * NS + sv[v]] * 3 + e];
      }
    // the sharer's face must hold the same corners (after the shift)
    if (sc >= 0) {
      double scale = 0;
      for (int v = 0; v < nfv; ++v) scale = std::max(scale, norm3(&xn[v * 3]));
      const double sft[3] = {fshift[f].x, fshift[f].y, fshift[f].z};
      for (int v = 0; v < nfv; ++v) {
        bool found = false;
        for (int u = 0; u < nfv && !found; ++u) {
          double e2 = 0;
          for (int e = 0; e < 3; ++e) {
            double dlt = xs[u * 3 + e] + sft[e] - xn[v * 3 + e];
            e2 += dlt * dlt;
          }
          found = std::sqrt(e2) <= 1e-10 * (1 + scale);
        }
        if (!found) bad_face = 1;
      }
    }
    int32_t base = face_off[f];
    if (geo::is_pyramid(type[hc]) && geo::curved(type[hc])) {
      // quadratic pyramid: the face's own Triangle6 / Quadrangle8 / 9 map (the
      // collapsed cube of the cell map does not hold the lateral triangles)
      int fn[9];
      const int n = geo::pyramid_face_nodes(type[hc], sh, fn);
      double xf[27];
      for (int v = 0; v < n; ++v)
        for (int e = 0; e < 3; ++e) xf[v * 3 + e] = d->xyz[d->cell_nodes[hc * NS + fn[v]] * 3 + e];
      const int nq = hex ? Q * Q : (int)tw.size();
      for (int q = 0; q < nq; ++q) {
        const double s = hex ? gx[q / Q] : tx[q][0], t = hex ? gx[q % Q] : tx[q][1];
        const double wl = hex ? gw[q / Q] * gw[q % Q] : tw[q];
        double X[3], ta[3], tb[3], nn[3];
        geo::face_map(n, xf, s, t, X, ta, tb);
        keep_tangent(f, q, ta);
        cross(ta, tb, nn);
        const double len = norm3(nn);
        point_face[base + q] = (int32_t)f;
        fpt[base + q] = make_double4(X[0], X[1], X[2], wl * len);
        fnrm[base + q] = make_double4(nn[0] / len, nn[1] / len, nn[2] / len, 0);
      }
    } else if (geo::curved(type[hc])) {
      // face points from the holder's cell map at the face's local points;
      // tangents J^T dloc/da, J^T dloc/db (quadrangle: corner 0 -> 1, 0 -> 3;
      // triangle: corner 0 - corner 2, corner 1 - corner 2 of the face)
      double xc[geo::kMaxNodes * 3];
      for (int v = 0; v < geo::node_count(type[hc]); ++v)
        for (int e = 0; e < 3; ++e) xc[v * 3 + e] = d->xyz[d->cell_nodes[hc * NS + v] * 3 + e];
      double lc[4][3];
      for (int v = 0; v < nfv; ++v) geo::local_of_node(type[hc], hv[v], lc[v]);
      double da[3], db[3];
      for (int e = 0; e < 3; ++e) {
        da[e] = hex ? (lc[1][e] - lc[0][e]) / 2 : lc[0][e] - lc[2][e];
        db[e] = hex ? (lc[3][e] - lc[0][e]) / 2 : lc[1][e] - lc[2][e];
      }
      const int nq = hex ? Q * Q : (int)tw.size();
      for (int q = 0; q < nq; ++q) {
        double loc[3], wl;
        if (hex) {
          const int i = q / Q, j = q % Q;
          for (int e = 0; e < 3; ++e) loc[e] = lc[0][e] + (gx[i] + 1) * da[e] + (gx[j] + 1) * db[e];
          wl = gw[i] * gw[j];
        } else {
          const double x = tx[q][0], y = tx[q][1], z = 1.0 - x - y;
          for (int e = 0; e < 3; ++e) loc[e] = lc[0][e] * x + lc[1][e] * y + lc[2][e] * z;
          wl = tw[q];
        }
        double X[3], J[9], ta[3], tb[3], nn[3];
        geo::map_point(type[hc], xc, loc, X, J);
        geo::tangent(J, da, ta);
        geo::tangent(J, db, tb);
        keep_tangent(f, q, ta);
        cross(ta, tb, nn);
        const double len = norm3(nn);
        point_face[base + q] = (int32_t)f;
        fpt[base + q] = make_double4(X[0], X[1], X[2], wl * len);
        fnrm[base + q] = make_double4(nn[0] / len, nn[1] / len, nn[2] / len, 0);
      }
    } else if (hex) {
      for (int i = 0; i < Q; ++i)
        for (int j = 0; j < Q; ++j) {
          int q = i * Q + j;
          double x = gx[i], y = gx[j], X[3] = {0, 0, 0}, jac[6] = {0, 0, 0, 0, 0, 0};
          for (int n = 0; n < 4; ++n) {
            double v = (1 + kQuadLocal[n][0] * x) * (1 + kQuadLocal[n][1] * y) / 4;
            double fx = (1 + kQuadLocal[n][0] * x) / 4, fy = (1 + kQuadLocal[n][1] * y) / 4;
            for (int e = 0; e < 3; ++e) {
              X[e] += xn[n * 3 + e] * v;
              jac[e] += kQuadLocal[n][0] * fy * xn[n * 3 + e];
              jac[3 + e] += kQuadLocal[n][1] * fx * xn[n * 3 + e];
            }
          }
          double a = jac[0] * jac[0] + jac[1] * jac[1] + jac[2] * jac[2];
          double b = jac[0] * jac[3] + jac[1] * jac[4] + jac[2] * jac[5];
          double cc = jac[3] * jac[3] + jac[4] * jac[4] + jac[5] * jac[5];
          double nn[3];
          cross(&jac[0], &jac[3], nn);
          keep_tangent(f, q, &jac[0]);
          double len = norm3(nn);
          point_face[base + q] = (int32_t)f;
          fpt[base + q] = make_double4(X[0], X[1], X[2], gw[i] * gw[j] * std::sqrt(a * cc - b * b));
          fnrm[base + q] = make_double4(nn[0] / len, nn[1] / len, nn[2] / len, 0);
        }
    } else {
      double jac[6], nn[3];
      for (int e = 0; e < 3; ++e) {
        jac[e] = xn[0 * 3 + e] - xn[2 * 3 + e];
        jac[3 + e] = xn[1 * 3 + e] - xn[2 * 3 + e];
      }
      cross(&jac[0], &jac[3], nn);
      keep_tangent(f, 0, &jac[0]);
      double area2 = norm3(nn);
      for (size_t q = 0; q < tw.size(); ++q) {
        double x = tx[q][0], y = tx[q][1], z = 1.0 - x - y, X[3];
        for (int e = 0; e < 3; ++e) X[e] = xn[0 * 3 + e] * x + xn[1 * 3 + e] * y + xn[2 * 3 + e] * z;
        point_face[base + q] = (int32_t)f;
        fpt[base + q] = make_double4(X[0], X[1], X[2], tw[q] * area2);
        fnrm[base + q] = make_double4(nn[0] / area2, nn[1] / area2, nn[2] / area2, 0);
      }
    }
  }
  if (bad_face) return fail(h, MCFD_ERR_MESH, "a sharer face does not match its holder face");
  if (md.keep_host) {
    md.host_frame0.assign((size_t)F * 9, 0.0);
    for (int64_t f = 0; f < F; ++f) {
      double *fr = &md.host_frame0[f * 9];
      const double4 nv = fnrm[face_off[f]];
      fr[0] = nv.x; fr[1] = nv.y; fr[2] = nv.z;
      const double tn = norm3(&ftan0[f * 3]);
      for (int e = 0; e < 3; ++e) fr[3 + e] = ftan0[f * 3 + e] / tn;
      cross(&fr[0], &fr[3], &fr[6]);
    }
  }
  // ---- upload
  int rc;
  if ((rc = upload(h, &md.center, center))) return rc;
  if ((rc = upload(h, &md.s, S))) return rc;
  if ((rc = upload(h, &md.vol_off, vol_off))) return rc;
  if ((rc = upload(h, &md.vol, vol))) return rc;
  if ((rc = upload(h, &md.cell_faces, cell_faces))) return rc;
  if ((rc = upload(h, &md.face_off, face_off))) return rc;
  if ((rc = upload(h, &md.point_face, point_face))) return rc;
  if ((rc = upload(h, &md.fpt, fpt))) return rc;
  if ((rc = upload(h, &md.fnrm, fnrm))) return rc;
  if ((rc = upload(h, &md.fshift, fshift))) return rc;
  if ((rc = upload(h, &m.face_cells, fcells))) return rc;
  if ((rc = upload(h, &m.face_group, fgroup))) return rc;
  if (h->opt.precision == MCFD_MIXED) {
    // FP32 copies for the mixed form's contractions
    std::vector<float> s32(S.size());
    for (size_t i = 0; i < S.size(); ++i) s32[i] = (float)S[i];
    std::vector<float4> vol32(NV);
    for (int64_t q = 0; q < NV; ++q)
      vol32[q] = make_float4((float)vol[q].x, (float)vol[q].y, (float)vol[q].z, (float)vol[q].w);
    std::vector<float4> foff32((size_t)NF * 2);
#pragma omp parallel for schedule(static)
    for (int64_t f = 0; f < F; ++f) {
      const int64_t hc = fcells[f].x, sc = fcells[f].y;
      for (int32_t q = face_off[f]; q < face_off[f + 1]; ++q) {
        const double4 x = fpt[q];
        foff32[(size_t)q * 2] = make_float4((float)(x.x - center[hc].x), (float)(x.y - center[hc].y),
                                            (float)(x.z - center[hc].z), 0.f);
        if (sc >= 0)
          foff32[(size_t)q * 2 + 1] =
              make_float4((float)((x.x - fshift[f].x) - center[sc].x), (float)((x.y - fshift[f].y) - center[sc].y),
                          (float)((x.z - fshift[f].z) - center[sc].z), 0.f);
        else
          foff32[(size_t)q * 2 + 1] = make_float4(0.f, 0.f, 0.f, 0.f);
      }
    }
    if ((rc = upload(h, &md.s32, s32))) return rc;
    if ((rc = upload(h, &md.vol32, vol32))) return rc;
    if ((rc = upload(h, &md.foff32, foff32))) return rc;
    cudaError_t e32 = cudaMalloc(&md.taylor32, sizeof(float) * m.column);
    if (e32 != cudaSuccess) return fail(h, MCFD_ERR_CUDA, std::string("modal tables: ") + cudaGetErrorString(e32));
  }
  cudaError_t e = cudaMalloc(&md.taylor, sizeof(double) * m.column);
  if (e != cudaSuccess) return fail(h, MCFD_ERR_CUDA, std::string("modal tables: ") + cudaGetErrorString(e));
  m.host_bcs.assign(std::max(m.n_groups, 1), BcDev{});
  if ((rc = upload(h, &m.bcs, m.host_bcs))) return rc;
  return MCFD_OK;
}

namespace {

// d^a T_j (the Taylor monomial j differentiated by multi-index a) at d.
double taylor_pdv(int j, int a, const double *d) {
  double f = 1;
  for (int e = 0; e < 3; ++e) {
    const int ej = kTaylorExp[j][e], ea = kTaylorExp[a][e];
    if (ej < ea) return 0;
    double fall = 1;
    for (int i = 0; i < ea; ++i) fall *= (ej - i);
    f *= fall * ipow(d[e], ej - ea);
  }
  return f;
}

// psi of a cell (centre ctr, full lower-triangular S [M][M]) at global x.
void modal_basis(const double *ctr, const double *S, int M, const double *x, double *psi) {
  const double d[3] = {x[0] - ctr[0], x[1] - ctr[1], x[2] - ctr[2]};
  double t[20];
  for (int j = 0; j < M; ++j) t[j] = ipow(d[0], kTaylorExp[j][0]) * ipow(d[1], kTaylorExp[j][1]) *
                                     ipow(d[2], kTaylorExp[j][2]);
  for (int i = 0; i < M; ++i) {
    double s = 0;
    for (int j = 0; j <= i; ++j) s += S[i * M + j] * t[j];
    psi[i] = s;
  }
}

}  // namespace

// WithLimiter<dg::General> over Projection: the tables of the WENO kernels
// (weno.cu) from each cell's own orthonormal basis and volume quadrature,
// the quantities limiter/weno.hpp computes on the fly:
//   proj [cells][6][M][M]  neighbour basis -> own basis over the own
//                          quadrature (Borrow: adj_proj.Approximate of the
//                          neighbour's GlobalToValue, weno.hpp:138-166)
//   beta [cells][M][M]     the smoothness quadratic form: sum over Taylor
//                          multi-indices a, |a| >= 1, of vol^(2|a|/3 - 1) /
//                          (|a|!)^2 * integral of d^a psi_i d^a psi_j
//                          (weno.hpp:25-95)
//   eval [cells][7][M]     neighbour bases (slots 0..5) and the own basis
//                          (slot 6) at the cell centre (IsNotSmooth,
//                          weno.hpp:230-258)
//   s00, divisor = vol^((p+1)/6) * n_adj, volume, adjacency in face order
//   with the periodic shifts, and each shared face's frame at its first
//   quadrature point (weno::Eigen, weno.hpp:297-336).
int build_modal_limiter(mcfd_handle *h, const mcfd_mesh_desc *d, int kind, double w0, double eps) {
  auto &md = h->modal;
  auto &l = h->lim;
  const int p = h->mesh.p, M = md.m;
  const int64_t C = h->mesh.n_cells;
  l.kind = kind;
  l.m = M;
  l.w0 = w0 > 0 ? w0 : 0.001;
  l.eps = eps > 0 ? eps : 1e-6;
  std::vector<int32_t> adj((size_t)C * 6, -1);
  std::vector<double> adj_shift((size_t)C * 6 * 3, 0.0), adj_frame((size_t)C * 6 * 9, 0.0);
  std::vector<int> n_adj(C, 0);
  for (int64_t f = 0; f < d->n_faces; ++f) {
    const int64_t hc = d->face_cells[f * 2], sc = d->face_cells[f * 2 + 1];
    if (sc < 0) continue;
    double sh[3] = {0, 0, 0};
    if (d->face_shift)
      for (int e = 0; e < 3; ++e) sh[e] = d->face_shift[f * 3 + e];
    const double *fr = &md.host_frame0[f * 9];
    const int64_t owner[2] = {hc, sc}, other[2] = {sc, hc};
    for (int side = 0; side < 2; ++side) {
      const int64_t c = owner[side];
      if (n_adj[c] >= 6) continue;
      const size_t slot = (size_t)c * 6 + n_adj[c];
      for (int e = 0; e < 3; ++e) adj_shift[slot * 3 + e] = side == 0 ? sh[e] : -sh[e];
      for (int e = 0; e < 9; ++e) adj_frame[slot * 9 + e] = fr[e];
      adj[slot] = (int32_t)other[side];
      ++n_adj[c];
    }
  }
  const double *X = md.host_points.data(), *W = md.host_weights.data();
  const double *ctr = md.host_center.data(), *S = md.host_s.data();
  std::vector<double> proj((size_t)C * 6 * M * M, 0.0), beta((size_t)C * M * M, 0.0);
  std::vector<double> eval((size_t)C * 7 * M, 0.0), s00(C), divisor(C);
#pragma omp parallel for schedule(static)
  for (int64_t c = 0; c < C; ++c) {
    const double *Sc = &S[(size_t)c * M * M];
    const double vol = md.host_volume[c];
    s00[c] = Sc[0];
    divisor[c] = std::pow(vol, (p + 1.0) / 2.0 / 3) * n_adj[c];
    double weight[4] = {0, 0, 0, 0};
    const double measure = 1 / (Sc[0] * Sc[0]);
    for (int deg = 1; deg <= p; ++deg) {
      const double kf = std::tgamma(deg + 1);
      weight[deg] = std::pow(measure, deg * 2. / 3 - 1) / (kf * kf);
    }
    double *B = &beta[(size_t)c * M * M];
    double psi[20], pb[20], dpsi[20];
    for (int32_t q = md.host_vol_off[c]; q < md.host_vol_off[c + 1]; ++q) {
      const double *x = &X[(size_t)q * 3];
      const double dd[3] = {x[0] - ctr[c * 3], x[1] - ctr[c * 3 + 1], x[2] - ctr[c * 3 + 2]};
      for (int a = 1; a < M; ++a) {
        const int deg = kTaylorExp[a][0] + kTaylorExp[a][1] + kTaylorExp[a][2];
        for (int i = 0; i < M; ++i) {
          double s = 0;
          for (int j = 0; j <= i; ++j) s += Sc[i * M + j] * taylor_pdv(j, a, dd);
          dpsi[i] = s;
        }
        for (int i = 0; i < M; ++i)
          for (int j = 0; j < M; ++j) B[i * M + j] += W[q] * weight[deg] * dpsi[i] * dpsi[j];
      }
      modal_basis(&ctr[c * 3], Sc, M, x, psi);
      for (int s = 0; s < n_adj[c]; ++s) {
        const int32_t nb = adj[(size_t)c * 6 + s];
        const double *sh = &adj_shift[((size_t)c * 6 + s) * 3];
        const double xs[3] = {x[0] - sh[0], x[1] - sh[1], x[2] - sh[2]};
        modal_basis(&ctr[(size_t)nb * 3], &S[(size_t)nb * M * M], M, xs, pb);
        double *P = &proj[(((size_t)c * 6 + s) * M) * M];
        for (int i = 0; i < M; ++i)
          for (int j = 0; j < M; ++j) P[i * M + j] += pb[i] * (W[q] * psi[j]);
      }
    }
    for (int s = 0; s < n_adj[c]; ++s) {
      const int32_t nb = adj[(size_t)c * 6 + s];
      const double *sh = &adj_shift[((size_t)c * 6 + s) * 3];
      const double xc[3] = {ctr[c * 3] - sh[0], ctr[c * 3 + 1] - sh[1], ctr[c * 3 + 2] - sh[2]};
      modal_basis(&ctr[(size_t)nb * 3], &S[(size_t)nb * M * M], M, xc, &eval[((size_t)c * 7 + s) * M]);
    }
    modal_basis(&ctr[c * 3], Sc, M, &ctr[c * 3], &eval[((size_t)c * 7 + 6) * M]);
  }
  int rc;
  if ((rc = upload(h, &l.proj, proj))) return rc;
  if ((rc = upload(h, &l.beta, beta))) return rc;
  if ((rc = upload(h, &l.eval, eval))) return rc;
  if ((rc = upload(h, &l.s00, s00))) return rc;
  if ((rc = upload(h, &l.divisor, divisor))) return rc;
  if ((rc = upload(h, &l.adj, adj))) return rc;
  if ((rc = upload(h, &l.frame, adj_frame))) return rc;
  if ((rc = upload(h, &l.volume, md.host_volume))) return rc;
  cudaError_t e = cudaMalloc(&l.modal, sizeof(double) * C * kK * M);
  if (e == cudaSuccess) e = cudaMalloc(&l.list, sizeof(int32_t) * C);
  if (e == cudaSuccess) e = cudaMalloc(&l.list_count, sizeof(unsigned));
  if (e == cudaSuccess) e = cudaMalloc(&l.troubled, sizeof(unsigned long long));
  if (e == cudaSuccess) e = cudaMemset(l.troubled, 0, sizeof(unsigned long long));
  if (e != cudaSuccess) return fail(h, MCFD_ERR_CUDA, std::string("limiter tables: ") + cudaGetErrorString(e));
  // the host copies are no longer needed
  std::vector<double>().swap(md.host_weights);
  std::vector<double>().swap(md.host_center);
  std::vector<double>().swap(md.host_s);
  std::vector<double>().swap(md.host_frame0);
  std::vector<double>().swap(md.host_volume);
  std::vector<int32_t>().swap(md.host_vol_off);
  md.keep_host = false;
  return MCFD_OK;
}

}  // namespace mcfd
