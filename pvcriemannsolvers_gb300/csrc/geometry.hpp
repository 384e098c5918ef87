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
#pragma once

#include <cmath>

#include "../../include/mcfd.h"

namespace mcfd {
namespace geo {

constexpr int kMaxNodes = 27;

inline bool is_tet(int type) { return type == MCFD_TET4 || type == MCFD_TET10; }
inline bool is_hex(int type) { return type == MCFD_HEX8 || type == MCFD_HEX27 || type == MCFD_HEX20; }
inline bool curved(int type) { return type == MCFD_HEX27 || type == MCFD_HEX20 || type == MCFD_TET10; }
inline int node_count(int type) {
  switch (type) {
    case MCFD_HEX8: return 8;
    case MCFD_TET4: return 4;
    case MCFD_HEX27: return 27;
    case MCFD_TET10: return 10;
    case MCFD_HEX20: return 20;
    default: return 0;
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

inline void local_of_node(int type, int a, double *loc) {
  if (is_tet(type)) {
    for (int e = 0; e < 3; ++e) loc[e] = 0.5 * tet10_local_half()[a][e];
  } else {
    for (int e = 0; e < 3; ++e) loc[e] = hex27_local()[a][e];
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
