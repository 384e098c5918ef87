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
inline bool is_wedge(int type) { return type == MCFD_WEDGE6; }
inline bool is_pyramid(int type) { return type == MCFD_PYRA5; }
inline bool curved(int type) { return type == MCFD_HEX27 || type == MCFD_HEX20 || type == MCFD_TET10; }
inline int node_count(int type) {
  switch (type) {
    case MCFD_HEX8: return 8;
    case MCFD_TET4: return 4;
    case MCFD_HEX27: return 27;
    case MCFD_TET10: return 10;
    case MCFD_HEX20: return 20;
    case MCFD_WEDGE6: return 6;
    case MCFD_PYRA5: return 5;
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

inline void local_of_node(int type, int a, double *loc) {
  static const double wedge[6][3] = {{1, 0, -1}, {0, 1, -1}, {0, 0, -1}, {1, 0, 1}, {0, 1, 1}, {0, 0, 1}};
  static const double pyra[5][3] = {{-1, -1, -1}, {1, -1, -1}, {1, 1, -1}, {-1, 1, -1}, {0, 0, 1}};
  if (is_tet(type)) {
    for (int e = 0; e < 3; ++e) loc[e] = 0.5 * tet10_local_half()[a][e];
  } else if (is_wedge(type)) {
    for (int e = 0; e < 3; ++e) loc[e] = wedge[a][e];
  } else if (is_pyramid(type)) {
    for (int e = 0; e < 3; ++e) loc[e] = pyra[a][e];
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
