// Cell maps of the element types (host set-up): shape functions of
// coordinate/hexahedron.hpp (Hexahedron8, Hexahedron20, Hexahedron27) and
// coordinate/tetrahedron.hpp (Tetrahedron4, Tetrahedron10), in CGNS node
// order, and the point / Jacobian of x(local) = sum_a N_a(local) x_a.
//
//   Hex8   trilinear, corners at (+-1, +-1, +-1)
//   Hex27  triquadratic Lagrange on {-1, 0, 1}^3: corners, mid-edges of the
//          bottom face (8-11), of the vertical edges (12-15), of the top face
//          (16-19), face centres bottom / -y / +x / +y / -x / top (20-25),
//          centre (26)
//   Hex20  serendipity: the corners and mid-edges of Hex27
//   Tet4   (a, b, c, 1 - a - b - c) for corners A (1,0,0), B (0,1,0),
//          C (0,0,1), D (0,0,0)
//   Tet10  quadratic: corners, then mid-edges AB, BC, CA, DA, DB, DC
//   Wedge6 (coordinate/wedge.hpp:127-138): local (a, b, z) with c = 1 - a - b,
//          nodes (1,0,-1) (0,1,-1) (0,0,-1) (1,0,1) (0,1,1) (0,0,1);
//          N = {a, b, c} x {(1 - z) / 2, (1 + z) / 2}
//   Pyra5  (coordinate/pyramid.hpp:124-135): the base corners of the local
//          cube (+-1, +-1, -1) with the trilinear shape functions, the apex
//          (0, 0, 1) with (1 + z) / 2: the cube collapses onto the pyramid
//   Wedge15 (coordinate/wedge.hpp:234-449): Wedge6 plus mid-edge nodes of the
//          bottom triangle (ab, bc, ca), the vertical edges, the top triangle;
//          built hierarchically: the new nodes' functions 4ab (1 - z) / 2,
//          a (1 - z^2), ... and N_a -= N6_a(node j) B_j for the corners
//   Wedge18 (coordinate/wedge.hpp:456-690): the quadratic triangle times the
//          quadratic Lagrange polynomials in z; nodes 15-17 at the centres of
//          the quadrangles (ab, bc, ca at z = 0)
//   Pyra13 (coordinate/pyramid.hpp:219-412): Pyra5 plus mid-edge nodes of the
//          base (5-8) and of the lateral edges (9-12, at z = 0 of the local
//          cube), hierarchically as Wedge15
//   Pyra14 (coordinate/pyramid.hpp:415-560): Pyra13 plus the base centre (13)
//          with (1 - x^2)(1 - y^2)(1 - z) / 2
//
// Local faces of every type (cell_face_corners) in the reference's node
// order, each parametrised so that its normal points out of the cell:
//   hexahedron  coordinate/hexahedron.hpp:353-390 (6 quadrangles)
//   tetrahedron coordinate/tetrahedron.hpp:141-147 (4 triangles)
//   wedge       coordinate/wedge.hpp:211-223: triangles {0,2,1} {3,4,5}, then
//               quadrangles {0,1,4,3} {1,2,5,4} {0,3,5,2}
//   pyramid     coordinate/pyramid.hpp:110-121, 199-208: the base {0,3,2,1},
//               then triangles {0,1,4} {1,2,4} {2,3,4} {3,0,4}
#pragma once

#include <cmath>

#include "../../include/mcfd.h"

namespace mcfd {
namespace geo {

constexpr int kMaxNodes = 27;

inline bool is_tet(int type) { return type == MCFD_TET4 || type == MCFD_TET10; }
inline bool is_hex(int type) { return type == MCFD_HEX8 || type == MCFD_HEX27 || type == MCFD_HEX20; }
inline bool is_wedge(int type) { return type == MCFD_WEDGE6 || type == MCFD_WEDGE15 || type == MCFD_WEDGE18; }
inline bool is_pyramid(int type) { return type == MCFD_PYRA5 || type == MCFD_PYRA13 || type == MCFD_PYRA14; }
inline bool curved(int type) {
  return type == MCFD_HEX27 || type == MCFD_HEX20 || type == MCFD_TET10 || type == MCFD_WEDGE15 ||
         type == MCFD_WEDGE18 || type == MCFD_PYRA13 || type == MCFD_PYRA14;
}
inline int node_count(int type) {
  switch (type) {
    case MCFD_HEX8: return 8;
    case MCFD_TET4: return 4;
    case MCFD_HEX27: return 27;
    case MCFD_TET10: return 10;
    case MCFD_HEX20: return 20;
    case MCFD_WEDGE6: return 6;
    case MCFD_PYRA5: return 5;
    case MCFD_WEDGE15: return 15;
    case MCFD_WEDGE18: return 18;
    case MCFD_PYRA13: return 13;
    case MCFD_PYRA14: return 14;
    default: return 0;
  }
}
// corner count (the straight-sided type the corners span)
inline int corner_count(int type) {
  return is_tet(type) ? 4 : is_wedge(type) ? 6 : is_pyramid(type) ? 5 : 8;
}

// Number of local faces, and the corners of local face `side` in v[] (3 or
// 4 entries; the return value).
inline int face_count(int type) { return is_tet(type) ? 4 : (is_wedge(type) || is_pyramid(type)) ? 5 : 6; }
inline int cell_face_corners(int type, int side, int *v) {
  static const int hex[6][4] = {{0, 3, 2, 1}, {0, 1, 5, 4}, {1, 2, 6, 5},
                                {2, 3, 7, 6}, {0, 4, 7, 3}, {4, 5, 6, 7}};
  static const int tet[4][3] = {{0, 2, 1}, {0, 1, 3}, {0, 3, 2}, {1, 2, 3}};
  static const int wedge[5][4] = {{0, 2, 1, -1}, {3, 4, 5, -1}, {0, 1, 4, 3}, {1, 2, 5, 4}, {0, 3, 5, 2}};
  static const int pyra[5][4] = {{0, 3, 2, 1}, {0, 1, 4, -1}, {1, 2, 4, -1}, {2, 3, 4, -1}, {3, 0, 4, -1}};
  const int *row;
  if (is_tet(type)) {
    for (int i = 0; i < 3; ++i) v[i] = tet[side][i];
    return 3;
  }
  row = is_wedge(type) ? wedge[side] : is_pyramid(type) ? pyra[side] : hex[side];
  const int n = row[3] < 0 ? 3 : 4;
  for (int i = 0; i < n; ++i) v[i] = row[i];
  return n;
}

inline double lq(int c, double x);
inline double dlq(int c, double x);

// Nodes of local face `side` of a quadratic pyramid in its face map's order
// (coordinate/pyramid.hpp Pyramid13::faces_ and SortNodesOnFace): the base
// Quadrangle8 / Quadrangle9 {0, 3, 2, 1, 8, 7, 6, 5 (, 13)}, the lateral
// Triangle6 faces {i, i + 1, 4, mid(i, i + 1), mid(i + 1, 4), mid(4, i)}.
inline int pyramid_face_nodes(int type, int side, int *v) {
  static const int tri[4][6] = {{0, 1, 4, 5, 10, 9}, {1, 2, 4, 6, 11, 10}, {2, 3, 4, 7, 12, 11}, {3, 0, 4, 8, 9, 12}};
  static const int base[9] = {0, 3, 2, 1, 8, 7, 6, 5, 13};
  if (side == 0) {
    const int n = type == MCFD_PYRA14 ? 9 : 8;
    for (int i = 0; i < n; ++i) v[i] = base[i];
    return n;
  }
  for (int i = 0; i < 6; ++i) v[i] = tri[side - 1][i];
  return 6;
}

// Point X and tangents dX/ds, dX/dt of a quadratic face map with n nodes
// xf[n][3] at face-local (s, t): n = 6 Triangle6 (coordinate/triangle.hpp:
// nodes (1, 0) (0, 1) (0, 0), then the mid-edges 01, 12, 20), n = 8 / 9
// Quadrangle8 / Quadrangle9 (coordinate/quadrangle.hpp: corners (-1, -1)
// (1, -1) (1, 1) (-1, 1), the mid-edges 01, 12, 23, 30, the centre).
inline void face_map(int n, const double *xf, double s, double t, double *X, double *ts, double *tt) {
  double N[9], Ds[9], Dt[9];
  if (n == 6) {
    const double L[3] = {s, t, 1 - s - t}, dLs[3] = {1, 0, -1}, dLt[3] = {0, 1, -1};
    for (int i = 0; i < 3; ++i) {
      const int j = (i + 1) % 3;
      N[i] = L[i] * (2 * L[i] - 1);
      Ds[i] = (4 * L[i] - 1) * dLs[i];
      Dt[i] = (4 * L[i] - 1) * dLt[i];
      N[3 + i] = 4 * L[i] * L[j];
      Ds[3 + i] = 4 * (dLs[i] * L[j] + L[i] * dLs[j]);
      Dt[3 + i] = 4 * (dLt[i] * L[j] + L[i] * dLt[j]);
    }
  } else {
    static const int q[9][2] = {{-1, -1}, {1, -1}, {1, 1}, {-1, 1}, {0, -1}, {1, 0}, {0, 1}, {-1, 0}, {0, 0}};
    for (int a = 0; a < n; ++a) {
      const int qs = q[a][0], qt = q[a][1];
      if (n == 9) {
        N[a] = lq(qs, s) * lq(qt, t);
        Ds[a] = dlq(qs, s) * lq(qt, t);
        Dt[a] = lq(qs, s) * dlq(qt, t);
      } else if (a < 4) {  // serendipity corner (1 + s qs)(1 + t qt)(s qs + t qt - 1) / 4
        const double fs = 1 + qs * s, ft = 1 + qt * t, w = qs * s + qt * t - 1;
        N[a] = fs * ft * w / 4;
        Ds[a] = qs * ft * (w + fs) / 4;
        Dt[a] = qt * fs * (w + ft) / 4;
      } else if (qs == 0) {  // (1 - s^2)(1 + t qt) / 2
        N[a] = (1 - s * s) * (1 + qt * t) / 2;
        Ds[a] = -s * (1 + qt * t);
        Dt[a] = (1 - s * s) * qt / 2;
      } else {  // (1 + s qs)(1 - t^2) / 2
        N[a] = (1 + qs * s) * (1 - t * t) / 2;
        Ds[a] = qs * (1 - t * t) / 2;
        Dt[a] = -t * (1 + qs * s);
      }
    }
  }
  for (int e = 0; e < 3; ++e) X[e] = ts[e] = tt[e] = 0;
  for (int a = 0; a < n; ++a)
    for (int e = 0; e < 3; ++e) {
      X[e] += N[a] * xf[a * 3 + e];
      ts[e] += Ds[a] * xf[a * 3 + e];
      tt[e] += Dt[a] * xf[a * 3 + e];
    }
}

// CGNS local coordinates of the Hex27 nodes (Hex8 and Hex20 are prefixes).
inline const int (*hex27_local())[3] {
  static const int l[27][3] = {
      {-1, -1, -1}, {1, -1, -1}, {1, 1, -1}, {-1, 1, -1}, {-1, -1, 1}, {1, -1, 1},
      {1, 1, 1},    {-1, 1, 1},  {0, -1, -1}, {1, 0, -1}, {0, 1, -1},  {-1, 0, -1},
      {-1, -1, 0},  {1, -1, 0},  {1, 1, 0},  {-1, 1, 0},  {0, -1, 1},  {1, 0, 1},
      {0, 1, 1},    {-1, 0, 1},  {0, 0, -1}, {0, -1, 0},  {1, 0, 0},   {0, 1, 0},
      {-1, 0, 0},   {0, 0, 1},   {0, 0, 0}};
  return l;
}

// Tet4 / Tet10 local coordinates in units of 1/2.
inline const int (*tet10_local_half())[3] {
  static const int l[10][3] = {{2, 0, 0}, {0, 2, 0}, {0, 0, 2}, {0, 0, 0}, {1, 1, 0},
                               {0, 1, 1}, {1, 0, 1}, {1, 0, 0}, {0, 1, 0}, {0, 0, 1}};
  return l;
}

// Wedge18 / Pyra14 local coordinates (the lower orders are prefixes).
inline const double (*wedge18_local())[3] {
  static const double l[18][3] = {{1, 0, -1},    {0, 1, -1},   {0, 0, -1},    {1, 0, 1},   {0, 1, 1},
                                  {0, 0, 1},     {.5, .5, -1}, {0, .5, -1},   {.5, 0, -1}, {1, 0, 0},
                                  {0, 1, 0},     {0, 0, 0},    {.5, .5, 1},   {0, .5, 1},  {.5, 0, 1},
                                  {.5, .5, 0},   {0, .5, 0},   {.5, 0, 0}};
  return l;
}
inline const double (*pyra14_local())[3] {
  static const double l[14][3] = {{-1, -1, -1}, {1, -1, -1}, {1, 1, -1}, {-1, 1, -1}, {0, 0, 1},
                                  {0, -1, -1},  {1, 0, -1},  {0, 1, -1}, {-1, 0, -1}, {-1, -1, 0},
                                  {1, -1, 0},   {1, 1, 0},   {-1, 1, 0}, {0, 0, -1}};
  return l;
}

inline void local_of_node(int type, int a, double *loc) {
  if (is_tet(type)) {
    for (int e = 0; e < 3; ++e) loc[e] = 0.5 * tet10_local_half()[a][e];
  } else if (is_wedge(type)) {
    for (int e = 0; e < 3; ++e) loc[e] = wedge18_local()[a][e];
  } else if (is_pyramid(type)) {
    for (int e = 0; e < 3; ++e) loc[e] = pyra14_local()[a][e];
  } else {
    for (int e = 0; e < 3; ++e) loc[e] = hex27_local()[a][e];
  }
}

// Local centre of a type (the reference's BuildCenter): hexahedron (0, 0, 0),
// tetrahedron (1/4, 1/4, 1/4), wedge (1/3, 1/3, 0), pyramid (0, 0, -1/2)
// (coordinate/{hexahedron,tetrahedron,wedge,pyramid}.hpp).
inline void local_center(int type, double *loc) {
  if (is_tet(type)) {
    loc[0] = loc[1] = loc[2] = 0.25;
  } else if (is_wedge(type)) {
    loc[0] = loc[1] = 1.0 / 3;
    loc[2] = 0;
  } else if (is_pyramid(type)) {
    loc[0] = loc[1] = 0;
    loc[2] = -0.5;
  } else {
    loc[0] = loc[1] = loc[2] = 0;
  }
}

// 1D quadratic Lagrange basis on {-1, 0, 1} at x for node value c, and its derivative.
inline double lq(int c, double x) {
  return c == 0 ? 1 - x * x : 0.5 * x * (x + c);
}
inline double dlq(int c, double x) {
  return c == 0 ? -2 * x : x + 0.5 * c;
}

inline void shapes(int type, const double *loc, double *N, double (*G)[3]);

// Hierarchical enrichment: with the functions B_j of the new nodes
// j in [n0, n1) (at locals l[j]) already in N / G, the functions of the
// lower type's nodes a < n0 become N_a - sum_j N_lower,a(l_j) B_j, so every
// function is 1 at its own node and 0 at the others.
inline void enrich(int lower, int n0, int n1, const double (*l)[3], double *N, double (*G)[3]) {
  double Nl[kMaxNodes], Gl[kMaxNodes][3];
  for (int j = n0; j < n1; ++j) {
    shapes(lower, l[j], Nl, Gl);
    for (int a = 0; a < n0; ++a) {
      N[a] -= Nl[a] * N[j];
      for (int e = 0; e < 3; ++e) G[a][e] -= Nl[a] * G[j][e];
    }
  }
}

// Shape functions N[a] and gradients G[a][3] at loc.
inline void shapes(int type, const double *loc, double *N, double (*G)[3]) {
  const double x = loc[0], y = loc[1], z = loc[2];
  const auto L = hex27_local();
  switch (type) {
    case MCFD_HEX8:
      for (int a = 0; a < 8; ++a) {
        const double fx = 1 + L[a][0] * x, fy = 1 + L[a][1] * y, fz = 1 + L[a][2] * z;
        N[a] = fx * fy * fz / 8;
        G[a][0] = L[a][0] * fy * fz / 8;
        G[a][1] = L[a][1] * fx * fz / 8;
        G[a][2] = L[a][2] * fx * fy / 8;
      }
      break;
    case MCFD_HEX27:
      for (int a = 0; a < 27; ++a) {
        const double bx = lq(L[a][0], x), by = lq(L[a][1], y), bz = lq(L[a][2], z);
        N[a] = bx * by * bz;
        G[a][0] = dlq(L[a][0], x) * by * bz;
        G[a][1] = bx * dlq(L[a][1], y) * bz;
        G[a][2] = bx * by * dlq(L[a][2], z);
      }
      break;
    case MCFD_HEX20:
      for (int a = 0; a < 20; ++a) {
        const double ax = L[a][0], ay = L[a][1], az = L[a][2];
        if (a < 8) {
          const double fx = 1 + ax * x, fy = 1 + ay * y, fz = 1 + az * z;
          const double s = ax * x + ay * y + az * z - 2;
          N[a] = fx * fy * fz * s / 8;
          G[a][0] = ax * fy * fz * (s + fx) / 8;
          G[a][1] = ay * fx * fz * (s + fy) / 8;
          G[a][2] = az * fx * fy * (s + fz) / 8;
        } else if (ax == 0) {
          const double fy = 1 + ay * y, fz = 1 + az * z;
          N[a] = (1 - x * x) * fy * fz / 4;
          G[a][0] = -2 * x * fy * fz / 4;
          G[a][1] = (1 - x * x) * ay * fz / 4;
          G[a][2] = (1 - x * x) * fy * az / 4;
        } else if (ay == 0) {
          const double fx = 1 + ax * x, fz = 1 + az * z;
          N[a] = (1 - y * y) * fx * fz / 4;
          G[a][0] = (1 - y * y) * ax * fz / 4;
          G[a][1] = -2 * y * fx * fz / 4;
          G[a][2] = (1 - y * y) * fx * az / 4;
        } else {
          const double fx = 1 + ax * x, fy = 1 + ay * y;
          N[a] = (1 - z * z) * fx * fy / 4;
          G[a][0] = (1 - z * z) * ax * fy / 4;
          G[a][1] = (1 - z * z) * fx * ay / 4;
          G[a][2] = -2 * z * fx * fy / 4;
        }
      }
      break;
    case MCFD_WEDGE6: {
      const double c = 1 - x - y, lo = (1 - z) / 2, hi = lo + z;
      N[0] = x * lo; N[1] = y * lo; N[2] = c * lo;
      N[3] = x * hi; N[4] = y * hi; N[5] = c * hi;
      const double g[6][3] = {{lo, 0, -0.5 * x}, {0, lo, -0.5 * y}, {-lo, -lo, -0.5 * c},
                              {hi, 0, 0.5 * x},  {0, hi, 0.5 * y},  {-hi, -hi, 0.5 * c}};
      for (int a = 0; a < 6; ++a)
        for (int e = 0; e < 3; ++e) G[a][e] = g[a][e];
      break;
    }
    case MCFD_PYRA5:
      for (int a = 0; a < 4; ++a) {
        const double fx = 1 + L[a][0] * x, fy = 1 + L[a][1] * y, fz = 1 + L[a][2] * z;
        N[a] = fx * fy * fz / 8;
        G[a][0] = L[a][0] * fy * fz / 8;
        G[a][1] = L[a][1] * fx * fz / 8;
        G[a][2] = L[a][2] * fx * fy / 8;
      }
      N[4] = (1 + z) / 2;
      G[4][0] = G[4][1] = 0;
      G[4][2] = 0.5;
      break;
    case MCFD_WEDGE15: {
      shapes(MCFD_WEDGE6, loc, N, G);
      // the new nodes' functions: 4 L_i L_j (1 -+ z) / 2 on the triangles,
      // L_i (1 - z^2) on the vertical edges
      const double L[3] = {x, y, 1 - x - y}, dL[3][2] = {{1, 0}, {0, 1}, {-1, -1}};
      const double fz[3] = {(1 - z) / 2, 1 - z * z, (1 + z) / 2}, dfz[3] = {-0.5, -2 * z, 0.5};
      for (int lev = 0; lev < 3; ++lev)
        for (int i = 0; i < 3; ++i) {
          const int a = 6 + lev * 3 + i, j = (i + 1) % 3;
          const double t = lev == 1 ? L[i] : 4 * L[i] * L[j];
          for (int r = 0; r < 2; ++r)
            G[a][r] = (lev == 1 ? dL[i][r] : 4 * (dL[i][r] * L[j] + L[i] * dL[j][r])) * fz[lev];
          N[a] = t * fz[lev];
          G[a][2] = t * dfz[lev];
        }
      enrich(MCFD_WEDGE6, 6, 15, wedge18_local(), N, G);
      break;
    }
    case MCFD_WEDGE18: {
      // quadratic triangle (corners, then mid-edges ab, bc, ca) x quadratic
      // Lagrange in z on {-1, 0, 1}
      const double L[3] = {x, y, 1 - x - y}, dL[3][2] = {{1, 0}, {0, 1}, {-1, -1}};
      double T[6], dT[6][2];
      for (int i = 0; i < 3; ++i) {
        const int j = (i + 1) % 3;
        T[i] = L[i] * (2 * L[i] - 1);
        T[3 + i] = 4 * L[i] * L[j];
        for (int r = 0; r < 2; ++r) {
          dT[i][r] = (4 * L[i] - 1) * dL[i][r];
          dT[3 + i][r] = 4 * (dL[i][r] * L[j] + L[i] * dL[j][r]);
        }
      }
      // node -> (triangle node, z level): 0-2 / 3-5 corners at z = -1 / +1,
      // 6-8 / 12-14 mid-edges at -1 / +1, 9-11 corners at 0, 15-17 mid-edges at 0
      static const int tri[18] = {0, 1, 2, 0, 1, 2, 3, 4, 5, 0, 1, 2, 3, 4, 5, 3, 4, 5};
      static const int lev[18] = {-1, -1, -1, 1, 1, 1, -1, -1, -1, 0, 0, 0, 1, 1, 1, 0, 0, 0};
      for (int a = 0; a < 18; ++a) {
        const double bz = lq(lev[a], z);
        N[a] = T[tri[a]] * bz;
        G[a][0] = dT[tri[a]][0] * bz;
        G[a][1] = dT[tri[a]][1] * bz;
        G[a][2] = T[tri[a]] * dlq(lev[a], z);
      }
      break;
    }
    case MCFD_PYRA13: {
      shapes(MCFD_PYRA5, loc, N, G);
      const auto P = pyra14_local();
      const double qx = 1 - x * x, qy = 1 - y * y, qz = (1 - z * z) / 4;
      for (int a = 5; a < 13; ++a) {
        const double ax = P[a][0], ay = P[a][1], az = P[a][2];
        if (a >= 9) {  // lateral mid-edges: (1 + x ax)(1 + y ay)(1 - z^2) / 4
          const double fx = 1 + ax * x, fy = 1 + ay * y;
          N[a] = fx * fy * qz;
          G[a][0] = ax * fy * qz;
          G[a][1] = ay * fx * qz;
          G[a][2] = fx * fy * (-z / 2);
        } else {  // base mid-edges: bubble of one axis x (1 + t at) / 2 x ((1 + z az) / 2 - qz)
          const double fz = (1 + az * z) / 2 - qz, dfz = (az + z) / 2;
          if (ax == 0) {
            const double fy = (1 + ay * y) / 2;
            N[a] = qx * fy * fz;
            G[a][0] = -2 * x * fy * fz;
            G[a][1] = ay / 2 * qx * fz;
            G[a][2] = qx * fy * dfz;
          } else {
            const double fx = (1 + ax * x) / 2;
            N[a] = fx * qy * fz;
            G[a][0] = ax / 2 * qy * fz;
            G[a][1] = -2 * y * fx * fz;
            G[a][2] = fx * qy * dfz;
          }
        }
      }
      enrich(MCFD_PYRA5, 5, 13, P, N, G);
      break;
    }
    case MCFD_PYRA14: {
      shapes(MCFD_PYRA13, loc, N, G);
      const double qx = 1 - x * x, qy = 1 - y * y, fz = (1 - z) / 2;
      N[13] = qx * qy * fz;
      G[13][0] = -2 * x * qy * fz;
      G[13][1] = -2 * y * qx * fz;
      G[13][2] = -qx * qy / 2;
      enrich(MCFD_PYRA13, 13, 14, pyra14_local(), N, G);
      break;
    }
    case MCFD_TET4: {
      N[0] = x; N[1] = y; N[2] = z; N[3] = 1 - x - y - z;
      const double g[4][3] = {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}, {-1, -1, -1}};
      for (int a = 0; a < 4; ++a)
        for (int e = 0; e < 3; ++e) G[a][e] = g[a][e];
      break;
    }
    default: {  // MCFD_TET10
      const double d = 1 - x - y - z;
      N[0] = x * (2 * x - 1); N[1] = y * (2 * y - 1); N[2] = z * (2 * z - 1); N[3] = d * (2 * d - 1);
      N[4] = 4 * x * y; N[5] = 4 * y * z; N[6] = 4 * z * x;
      N[7] = 4 * d * x; N[8] = 4 * d * y; N[9] = 4 * d * z;
      const double gd = 1 - 4 * d;  // d N_D / d(x|y|z) = -(4 d - 1)
      const double g[10][3] = {{4 * x - 1, 0, 0}, {0, 4 * y - 1, 0}, {0, 0, 4 * z - 1}, {gd, gd, gd},
                               {4 * y, 4 * x, 0}, {0, 4 * z, 4 * y}, {4 * z, 0, 4 * x},
                               {4 * (d - x), -4 * x, -4 * x}, {-4 * y, 4 * (d - y), -4 * y},
                               {-4 * z, -4 * z, 4 * (d - z)}};
      for (int a = 0; a < 10; ++a)
        for (int e = 0; e < 3; ++e) G[a][e] = g[a][e];
    }
  }
}

// x(loc) and J[r * 3 + d] = d x_d / d loc_r for node coordinates xn [n][3].
inline void map_point(int type, const double *xn, const double *loc, double *x, double *J) {
  double N[kMaxNodes], G[kMaxNodes][3];
  shapes(type, loc, N, G);
  const int n = node_count(type);
  for (int e = 0; e < 3; ++e) x[e] = 0;
  for (int e = 0; e < 9; ++e) J[e] = 0;
  for (int a = 0; a < n; ++a)
    for (int d = 0; d < 3; ++d) {
      x[d] += N[a] * xn[a * 3 + d];
      for (int r = 0; r < 3; ++r) J[r * 3 + d] += G[a][r] * xn[a * 3 + d];
    }
}

inline double det3(const double *J) {
  return J[0] * (J[4] * J[8] - J[5] * J[7]) - J[1] * (J[3] * J[8] - J[5] * J[6]) +
         J[2] * (J[3] * J[7] - J[4] * J[6]);
}

// Tangent J^T v of the local direction v.
inline void tangent(const double *J, const double *v, double *t) {
  for (int d = 0; d < 3; ++d) t[d] = J[0 * 3 + d] * v[0] + J[1 * 3 + d] * v[1] + J[2 * 3 + d] * v[2];
}

}  // namespace geo
}  // namespace mcfd
