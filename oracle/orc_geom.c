/*
 * ORACLE (test infrastructure only): cell maps of the element types, the
 * shape functions of coordinate/hexahedron.hpp (Hexahedron8 / 20 / 27) and
 * coordinate/tetrahedron.hpp (Tetrahedron4 / 10) in CGNS node order, written
 * from their definitions: Hex27 is the tensor product of the quadratic
 * Lagrange polynomials on {-1, 0, 1}; Hex20 the serendipity element (corner
 * shapes (1+xx_a)(1+yy_a)(1+zz_a)(xx_a+yy_a+zz_a-2)/8, mid-edge shapes
 * (1-x^2)(1+yy_a)(1+zz_a)/4 and permutations); Tet10 the quadratic simplex
 * element (corner shapes L(2L-1), mid-edge shapes 4 L_i L_j) with barycentric
 * coordinates (x, y, z, 1 - x - y - z) for corners A, B, C, D.  Wedge6
 * (coordinate/wedge.hpp:127-138): {a, b, 1 - a - b} times {(1 - z)/2,
 * (1 + z)/2}; Pyra5 (coordinate/pyramid.hpp:124-135): trilinear shapes of the
 * base corners (+-1, +-1, -1) of the local cube and (1 + z)/2 for the apex.
 * Local faces (orc_type_face_corners) in the reference's node order:
 * hexahedron.hpp:353-390, tetrahedron.hpp:141-147, wedge.hpp:211-223,
 * pyramid.hpp:110-121 and 199-208.
 */
#include <math.h>

#include "orc_internal.h"

/* Hex27 local coordinates (Hexahedron27::local_coords_ order). */
static const int kHex27[27][3] = {
    {-1, -1, -1}, {1, -1, -1}, {1, 1, -1}, {-1, 1, -1}, {-1, -1, 1}, {1, -1, 1}, {1, 1, 1},
    {-1, 1, 1},   {0, -1, -1}, {1, 0, -1}, {0, 1, -1},  {-1, 0, -1}, {-1, -1, 0}, {1, -1, 0},
    {1, 1, 0},    {-1, 1, 0},  {0, -1, 1}, {1, 0, 1},   {0, 1, 1},   {-1, 0, 1},  {0, 0, -1},
    {0, -1, 0},   {1, 0, 0},   {0, 1, 0},  {-1, 0, 0},  {0, 0, 1},   {0, 0, 0}};
/* Tet10 corners A B C D, then edges AB BC CA DA DB DC (as vertex pairs). */
static const int kTetEdge[6][2] = {{0, 1}, {1, 2}, {2, 0}, {3, 0}, {3, 1}, {3, 2}};

int orc_type_nodes(int type) {
  switch (type) {
    case ORC_CELL_HEX8: return 8;
    case ORC_CELL_TET4: return 4;
    case ORC_CELL_HEX27: return 27;
    case ORC_CELL_TET10: return 10;
    case ORC_CELL_HEX20: return 20;
    case ORC_CELL_WEDGE6: return 6;
    case ORC_CELL_PYRA5: return 5;
    default: return 0;
  }
}

int orc_type_faces(int type) {
  if (orc_type_is_tet(type)) return 4;
  return (type == ORC_CELL_WEDGE6 || type == ORC_CELL_PYRA5) ? 5 : 6;
}

int orc_type_face_corners(int type, int side, int *v) {
  static const int hex[6][4] = {{0, 3, 2, 1}, {0, 1, 5, 4}, {1, 2, 6, 5},
                                {2, 3, 7, 6}, {0, 4, 7, 3}, {4, 5, 6, 7}};
  static const int tet[4][4] = {{0, 2, 1, -1}, {0, 1, 3, -1}, {0, 3, 2, -1}, {1, 2, 3, -1}};
  static const int wedge[5][4] = {{0, 2, 1, -1}, {3, 4, 5, -1}, {0, 1, 4, 3}, {1, 2, 5, 4}, {0, 3, 5, 2}};
  static const int pyra[5][4] = {{0, 3, 2, 1}, {0, 1, 4, -1}, {1, 2, 4, -1}, {2, 3, 4, -1}, {3, 0, 4, -1}};
  const int *row = orc_type_is_tet(type) ? tet[side]
                   : type == ORC_CELL_WEDGE6 ? wedge[side]
                   : type == ORC_CELL_PYRA5  ? pyra[side]
                                             : hex[side];
  int n = row[3] < 0 ? 3 : 4;
  for (int i = 0; i < n; ++i) v[i] = row[i];
  return n;
}

void orc_type_center(int type, double *loc) {
  if (orc_type_is_tet(type)) {
    loc[0] = loc[1] = loc[2] = 0.25;
  } else if (type == ORC_CELL_WEDGE6) {
    loc[0] = loc[1] = 1.0 / 3;
    loc[2] = 0;
  } else if (type == ORC_CELL_PYRA5) {
    loc[0] = loc[1] = 0;
    loc[2] = -0.5;
  } else {
    loc[0] = loc[1] = loc[2] = 0;
  }
}

int orc_type_is_tet(int type) { return type == ORC_CELL_TET4 || type == ORC_CELL_TET10; }

void orc_local_of_node(int type, int a, double *loc) {
  static const double wedge[6][3] = {{1, 0, -1}, {0, 1, -1}, {0, 0, -1}, {1, 0, 1}, {0, 1, 1}, {0, 0, 1}};
  static const double pyra[5][3] = {{-1, -1, -1}, {1, -1, -1}, {1, 1, -1}, {-1, 1, -1}, {0, 0, 1}};
  if (type == ORC_CELL_WEDGE6) {
    for (int e = 0; e < 3; ++e) loc[e] = wedge[a][e];
  } else if (type == ORC_CELL_PYRA5) {
    for (int e = 0; e < 3; ++e) loc[e] = pyra[a][e];
  } else if (orc_type_is_tet(type)) {
    double b[4] = {0, 0, 0, 0};
    if (a < 4) {
      b[a] = 1;
    } else {
      b[kTetEdge[a - 4][0]] = 0.5;
      b[kTetEdge[a - 4][1]] = 0.5;
    }
    loc[0] = b[0]; loc[1] = b[1]; loc[2] = b[2];
  } else {
    for (int e = 0; e < 3; ++e) loc[e] = kHex27[a][e];
  }
}

/* quadratic Lagrange polynomial of node c in {-1, 0, 1} on {-1, 0, 1} */
static double quad1(int c, double x) {
  if (c == 0) return (1 - x) * (1 + x);
  return c > 0 ? x * (1 + x) / 2 : x * (x - 1) / 2;
}
static double dquad1(int c, double x) {
  if (c == 0) return -2 * x;
  return c > 0 ? (1 + 2 * x) / 2 : (2 * x - 1) / 2;
}

static void shapes(int type, const double *p, double *N, double (*G)[3]) {
  const double x = p[0], y = p[1], z = p[2];
  if (type == ORC_CELL_HEX8) {
    for (int a = 0; a < 8; ++a) {
      double fx = 1 + kHex27[a][0] * x, fy = 1 + kHex27[a][1] * y, fz = 1 + kHex27[a][2] * z;
      N[a] = fx * fy * fz / 8;
      G[a][0] = kHex27[a][0] * fy * fz / 8;
      G[a][1] = kHex27[a][1] * fx * fz / 8;
      G[a][2] = kHex27[a][2] * fx * fy / 8;
    }
  } else if (type == ORC_CELL_WEDGE6) {
    const double c = 1 - x - y, lo = (1 - z) / 2, hi = (1 + z) / 2;
    const double L[3] = {x, y, c};
    const double dL[3][2] = {{1, 0}, {0, 1}, {-1, -1}};
    for (int a = 0; a < 3; ++a) {
      N[a] = L[a] * lo;
      N[3 + a] = L[a] * hi;
      G[a][0] = dL[a][0] * lo; G[a][1] = dL[a][1] * lo; G[a][2] = -0.5 * L[a];
      G[3 + a][0] = dL[a][0] * hi; G[3 + a][1] = dL[a][1] * hi; G[3 + a][2] = 0.5 * L[a];
    }
  } else if (type == ORC_CELL_PYRA5) {
    for (int a = 0; a < 4; ++a) {
      double fx = 1 + kHex27[a][0] * x, fy = 1 + kHex27[a][1] * y, fz = 1 + kHex27[a][2] * z;
      N[a] = fx * fy * fz / 8;
      G[a][0] = kHex27[a][0] * fy * fz / 8;
      G[a][1] = kHex27[a][1] * fx * fz / 8;
      G[a][2] = kHex27[a][2] * fx * fy / 8;
    }
    N[4] = (1 + z) / 2;
    G[4][0] = G[4][1] = 0;
    G[4][2] = 0.5;
  } else if (type == ORC_CELL_HEX27) {
    for (int a = 0; a < 27; ++a) {
      double qx = quad1(kHex27[a][0], x), qy = quad1(kHex27[a][1], y), qz = quad1(kHex27[a][2], z);
      N[a] = qx * qy * qz;
      G[a][0] = dquad1(kHex27[a][0], x) * qy * qz;
      G[a][1] = qx * dquad1(kHex27[a][1], y) * qz;
      G[a][2] = qx * qy * dquad1(kHex27[a][2], z);
    }
  } else if (type == ORC_CELL_HEX20) {
    for (int a = 0; a < 20; ++a) {
      const int *l = kHex27[a];
      double f[3] = {1 + l[0] * x, 1 + l[1] * y, 1 + l[2] * z};
      double q[3] = {x, y, z};
      if (a < 8) {
        double s = l[0] * x + l[1] * y + l[2] * z - 2;
        N[a] = f[0] * f[1] * f[2] * s / 8;
        for (int d = 0; d < 3; ++d) {
          double others = f[(d + 1) % 3] * f[(d + 2) % 3];
          G[a][d] = l[d] * others * (s + f[d]) / 8;
        }
      } else {
        int m = l[0] == 0 ? 0 : (l[1] == 0 ? 1 : 2); /* the midpoint's axis */
        double bub = 1 - q[m] * q[m];
        double o1 = f[(m + 1) % 3], o2 = f[(m + 2) % 3];
        N[a] = bub * o1 * o2 / 4;
        G[a][m] = -2 * q[m] * o1 * o2 / 4;
        G[a][(m + 1) % 3] = bub * l[(m + 1) % 3] * o2 / 4;
        G[a][(m + 2) % 3] = bub * o1 * l[(m + 2) % 3] / 4;
      }
    }
  } else {
    double L[4] = {x, y, z, 1 - x - y - z};
    double dL[4][3] = {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}, {-1, -1, -1}};
    int quad = type == ORC_CELL_TET10;
    for (int a = 0; a < 4; ++a) {
      N[a] = quad ? L[a] * (2 * L[a] - 1) : L[a];
      for (int d = 0; d < 3; ++d) G[a][d] = quad ? (4 * L[a] - 1) * dL[a][d] : dL[a][d];
    }
    if (quad)
      for (int e = 0; e < 6; ++e) {
        int i = kTetEdge[e][0], j = kTetEdge[e][1];
        N[4 + e] = 4 * L[i] * L[j];
        for (int d = 0; d < 3; ++d) G[4 + e][d] = 4 * (dL[i][d] * L[j] + L[i] * dL[j][d]);
      }
  }
}

void orc_map_point(int type, const double *xn, const double *loc, double *x, double *jac) {
  double N[27], G[27][3];
  int n = orc_type_nodes(type);
  shapes(type, loc, N, G);
  for (int d = 0; d < 3; ++d) x[d] = 0;
  for (int e = 0; e < 9; ++e) jac[e] = 0;
  for (int a = 0; a < n; ++a)
    for (int d = 0; d < 3; ++d) {
      x[d] += N[a] * xn[a * 3 + d];
      for (int r = 0; r < 3; ++r) jac[r * 3 + d] += G[a][r] * xn[a * 3 + d];
    }
}
