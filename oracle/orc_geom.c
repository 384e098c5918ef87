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
 * Wedge15 (coordinate/wedge.hpp:234-449) in its nodal serendipity form:
 * corners L (1 + zz_a)(2L + zz_a - 2) / 2, triangle mid-edges
 * 2 L_i L_j (1 + zz_a), vertical mid-edges L (1 - z^2); Wedge18
 * (wedge.hpp:456-690) the quadratic triangle times the quadratic Lagrange
 * polynomials in z.  Pyra13 / Pyra14 (pyramid.hpp:219-560) span the Pyra5
 * functions and the new nodes' functions (base mid-edges
 * b_x b_y (1 - z)^2 / 4 with b = 1 - t^2 on the node's zero axis and
 * (1 + t t_a) / 2 on the other, lateral mid-edges
 * (1 + xx_a)(1 + yy_a)(1 - z^2) / 4, the base centre
 * (1 - x^2)(1 - y^2)(1 - z) / 2); the nodal functions come from inverting
 * the generalised Vandermonde matrix of that span at the nodes.
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
/* Wedge18 / Pyramid14 local coordinates (wedge.hpp:656-676,
 * pyramid.hpp:545-556); the lower orders are prefixes */
static const double kWedge18[18][3] = {
    {1, 0, -1}, {0, 1, -1}, {0, 0, -1}, {1, 0, 1}, {0, 1, 1}, {0, 0, 1},
    {0.5, 0.5, -1}, {0, 0.5, -1}, {0.5, 0, -1}, {1, 0, 0}, {0, 1, 0}, {0, 0, 0},
    {0.5, 0.5, 1}, {0, 0.5, 1}, {0.5, 0, 1}, {0.5, 0.5, 0}, {0, 0.5, 0}, {0.5, 0, 0}};
static const double kPyra14[14][3] = {
    {-1, -1, -1}, {1, -1, -1}, {1, 1, -1}, {-1, 1, -1}, {0, 0, 1}, {0, -1, -1}, {1, 0, -1},
    {0, 1, -1}, {-1, 0, -1}, {-1, -1, 0}, {1, -1, 0}, {1, 1, 0}, {-1, 1, 0}, {0, 0, -1}};

/* 0 hexahedron, 1 tetrahedron, 2 wedge, 3 pyramid */
static int family(int type) {
  switch (type) {
    case ORC_CELL_TET4: case ORC_CELL_TET10: return 1;
    case ORC_CELL_WEDGE6: case ORC_CELL_WEDGE15: case ORC_CELL_WEDGE18: return 2;
    case ORC_CELL_PYRA5: case ORC_CELL_PYRA13: case ORC_CELL_PYRA14: return 3;
    default: return 0;
  }
}
int orc_type_is_wedge(int type) { return family(type) == 2; }
int orc_type_is_pyramid(int type) { return family(type) == 3; }

int orc_type_nodes(int type) {
  switch (type) {
    case ORC_CELL_HEX8: return 8;
    case ORC_CELL_TET4: return 4;
    case ORC_CELL_HEX27: return 27;
    case ORC_CELL_TET10: return 10;
    case ORC_CELL_HEX20: return 20;
    case ORC_CELL_WEDGE6: return 6;
    case ORC_CELL_PYRA5: return 5;
    case ORC_CELL_WEDGE15: return 15;
    case ORC_CELL_WEDGE18: return 18;
    case ORC_CELL_PYRA13: return 13;
    case ORC_CELL_PYRA14: return 14;
    default: return 0;
  }
}

int orc_type_faces(int type) {
  if (orc_type_is_tet(type)) return 4;
  return family(type) >= 2 ? 5 : 6;
}

int orc_type_face_corners(int type, int side, int *v) {
  static const int hex[6][4] = {{0, 3, 2, 1}, {0, 1, 5, 4}, {1, 2, 6, 5},
                                {2, 3, 7, 6}, {0, 4, 7, 3}, {4, 5, 6, 7}};
  static const int tet[4][4] = {{0, 2, 1, -1}, {0, 1, 3, -1}, {0, 3, 2, -1}, {1, 2, 3, -1}};
  static const int wedge[5][4] = {{0, 2, 1, -1}, {3, 4, 5, -1}, {0, 1, 4, 3}, {1, 2, 5, 4}, {0, 3, 5, 2}};
  static const int pyra[5][4] = {{0, 3, 2, 1}, {0, 1, 4, -1}, {1, 2, 4, -1}, {2, 3, 4, -1}, {3, 0, 4, -1}};
  const int *row = orc_type_is_tet(type) ? tet[side]
                   : family(type) == 2 ? wedge[side]
                   : family(type) == 3 ? pyra[side]
                                             : hex[side];
  int n = row[3] < 0 ? 3 : 4;
  for (int i = 0; i < n; ++i) v[i] = row[i];
  return n;
}

void orc_type_center(int type, double *loc) {
  if (orc_type_is_tet(type)) {
    loc[0] = loc[1] = loc[2] = 0.25;
  } else if (family(type) == 2) {
    loc[0] = loc[1] = 1.0 / 3;
    loc[2] = 0;
  } else if (family(type) == 3) {
    loc[0] = loc[1] = 0;
    loc[2] = -0.5;
  } else {
    loc[0] = loc[1] = loc[2] = 0;
  }
}

int orc_type_is_tet(int type) { return type == ORC_CELL_TET4 || type == ORC_CELL_TET10; }

void orc_local_of_node(int type, int a, double *loc) {
  if (family(type) == 2) {
    for (int e = 0; e < 3; ++e) loc[e] = kWedge18[a][e];
  } else if (family(type) == 3) {
    for (int e = 0; e < 3; ++e) loc[e] = kPyra14[a][e];
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

/* The span of the Pyra13 (n = 13) / Pyra14 (n = 14) functions: the Pyra5
 * shapes, then one function per new node (header comment). */
static void pyra_span(int n, const double *p, double *f, double (*g)[3]) {
  const double x = p[0], y = p[1], z = p[2];
  for (int a = 0; a < 4; ++a) {
    double fx = 1 + kPyra14[a][0] * x, fy = 1 + kPyra14[a][1] * y, fz = 1 - z;
    f[a] = fx * fy * fz / 8;
    g[a][0] = kPyra14[a][0] * fy * fz / 8;
    g[a][1] = kPyra14[a][1] * fx * fz / 8;
    g[a][2] = -fx * fy / 8;
  }
  f[4] = (1 + z) / 2;
  g[4][0] = g[4][1] = 0;
  g[4][2] = 0.5;
  for (int a = 5; a < 9; ++a) {
    double ax = kPyra14[a][0], ay = kPyra14[a][1];
    double bx = ax == 0 ? 1 - x * x : (1 + ax * x) / 2, dbx = ax == 0 ? -2 * x : ax / 2;
    double by = ay == 0 ? 1 - y * y : (1 + ay * y) / 2, dby = ay == 0 ? -2 * y : ay / 2;
    double w = (1 - z) * (1 - z) / 4, dw = -(1 - z) / 2;
    f[a] = bx * by * w;
    g[a][0] = dbx * by * w;
    g[a][1] = bx * dby * w;
    g[a][2] = bx * by * dw;
  }
  for (int a = 9; a < 13; ++a) {
    double ax = kPyra14[a][0], ay = kPyra14[a][1];
    double fx = 1 + ax * x, fy = 1 + ay * y, w = (1 - z * z) / 4;
    f[a] = fx * fy * w;
    g[a][0] = ax * fy * w;
    g[a][1] = ay * fx * w;
    g[a][2] = fx * fy * (-z / 2);
  }
  if (n == 14) {
    double bx = 1 - x * x, by = 1 - y * y;
    f[13] = bx * by * (1 - z) / 2;
    g[13][0] = -2 * x * by * (1 - z) / 2;
    g[13][1] = -2 * y * bx * (1 - z) / 2;
    g[13][2] = -bx * by / 2;
  }
}

/* Nodal Pyra13 / Pyra14 functions: N_a = sum_k f_k C[k][a] with C the
 * inverse of V[i][k] = f_k(node i) (Gauss-Jordan, partial pivoting). */
static void pyra_nodal(int n, const double *p, double *N, double (*G)[3]) {
  double A[14][28], f[14], g[14][3];
  for (int i = 0; i < n; ++i) {
    pyra_span(n, kPyra14[i], f, g);
    for (int k = 0; k < n; ++k) {
      A[i][k] = f[k];
      A[i][n + k] = i == k;
    }
  }
  for (int col = 0; col < n; ++col) {
    int piv = col;
    for (int r = col + 1; r < n; ++r)
      if (fabs(A[r][col]) > fabs(A[piv][col])) piv = r;
    for (int k = 0; k < 2 * n; ++k) {
      double t = A[col][k];
      A[col][k] = A[piv][k];
      A[piv][k] = t;
    }
    double d = A[col][col];
    for (int k = 0; k < 2 * n; ++k) A[col][k] /= d;
    for (int r = 0; r < n; ++r) {
      if (r == col || A[r][col] == 0) continue;
      double m = A[r][col];
      for (int k = 0; k < 2 * n; ++k) A[r][k] -= m * A[col][k];
    }
  }
  pyra_span(n, p, f, g);
  for (int a = 0; a < n; ++a) {
    N[a] = G[a][0] = G[a][1] = G[a][2] = 0;
    for (int k = 0; k < n; ++k) {
      double c = A[k][n + a];
      N[a] += f[k] * c;
      for (int d = 0; d < 3; ++d) G[a][d] += g[k][d] * c;
    }
  }
}

static void shapes(int type, const double *p, double *N, double (*G)[3]) {
  const double x = p[0], y = p[1], z = p[2];
  if (type == ORC_CELL_PYRA13 || type == ORC_CELL_PYRA14) {
    pyra_nodal(orc_type_nodes(type), p, N, G);
    return;
  }
  if (type == ORC_CELL_WEDGE15 || type == ORC_CELL_WEDGE18) {
    const double L[3] = {x, y, 1 - x - y};
    const double dL[3][2] = {{1, 0}, {0, 1}, {-1, -1}};
    for (int a = 0; a < orc_type_nodes(type); ++a) {
      const double za = kWedge18[a][2];
      /* the node's triangle position: a corner i (L_i = 1) or the mid-edge
       * of corners i, j */
      int i = -1, j = -1;
      for (int k = 0; k < 3; ++k) {
        double lk = k == 0 ? kWedge18[a][0] : k == 1 ? kWedge18[a][1] : 1 - kWedge18[a][0] - kWedge18[a][1];
        if (lk == 1) i = k;
        if (lk == 0.5) { if (i < 0) i = k; else j = k; }
      }
      double t, dt[2], bz, dbz;
      if (j < 0) {
        double li = L[i];
        if (type == ORC_CELL_WEDGE15 && za != 0) { /* serendipity corner */
          N[a] = li * (1 + za * z) * (2 * li + za * z - 2) / 2;
          double dli = (1 + za * z) * (4 * li + za * z - 2) / 2;
          G[a][0] = dli * dL[i][0];
          G[a][1] = dli * dL[i][1];
          G[a][2] = li * za * (2 * li + 2 * za * z - 1) / 2;
          continue;
        }
        t = type == ORC_CELL_WEDGE15 ? li : li * (2 * li - 1);
        for (int r = 0; r < 2; ++r) dt[r] = (type == ORC_CELL_WEDGE15 ? 1 : 4 * li - 1) * dL[i][r];
      } else {
        t = 4 * L[i] * L[j];
        for (int r = 0; r < 2; ++r) dt[r] = 4 * (dL[i][r] * L[j] + L[i] * dL[j][r]);
      }
      if (type == ORC_CELL_WEDGE15) { /* linear in z between levels, 1 - z^2 at 0 */
        bz = za == 0 ? 1 - z * z : (1 + za * z) / 2;
        dbz = za == 0 ? -2 * z : za / 2;
      } else {
        bz = quad1((int)za, z);
        dbz = dquad1((int)za, z);
      }
      N[a] = t * bz;
      G[a][0] = dt[0] * bz;
      G[a][1] = dt[1] * bz;
      G[a][2] = t * dbz;
    }
    return;
  }
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

/* Pyramid13::faces_ and SortNodesOnFace (coordinate/pyramid.hpp:240-260,
 * 399-408): base {0, 3, 2, 1, 8, 7, 6, 5 (, 13)}, lateral triangles with
 * corners (i, i + 1, apex) then their mid-edges. */
int orc_pyramid_face_nodes(int type, int side, int *v) {
  static const int base[9] = {0, 3, 2, 1, 8, 7, 6, 5, 13};
  if (side == 0) {
    int n = type == ORC_CELL_PYRA14 ? 9 : 8;
    for (int k = 0; k < n; ++k) v[k] = base[k];
    return n;
  }
  int i = side - 1, j = side % 4;
  v[0] = i; v[1] = j; v[2] = 4;
  v[3] = 5 + i;      /* base mid-edge of (i, j) */
  v[4] = 9 + j;      /* lateral mid-edge of (j, apex) */
  v[5] = 9 + i;      /* lateral mid-edge of (apex, i) */
  return 6;
}

/* Triangle6 (coordinate/triangle.hpp:206-210) with barycentric
 * (s, t, 1 - s - t); Quadrangle8 / 9 (coordinate/quadrangle.hpp:260-265,
 * 375-380). */
void orc_face_map(int n, const double *xf, double s, double t, double *x, double *ts, double *tt) {
  double N[9], Ds[9], Dt[9];
  if (n == 6) {
    const double L[3] = {s, t, 1 - s - t};
    const double dL[3][2] = {{1, 0}, {0, 1}, {-1, -1}};
    for (int i = 0; i < 3; ++i) {
      N[i] = L[i] * (2 * L[i] - 1);
      Ds[i] = (4 * L[i] - 1) * dL[i][0];
      Dt[i] = (4 * L[i] - 1) * dL[i][1];
      int j = (i + 1) % 3;
      N[3 + i] = 4 * L[i] * L[j];
      Ds[3 + i] = 4 * (dL[i][0] * L[j] + L[i] * dL[j][0]);
      Dt[3 + i] = 4 * (dL[i][1] * L[j] + L[i] * dL[j][1]);
    }
  } else {
    static const int q[9][2] = {{-1, -1}, {1, -1}, {1, 1}, {-1, 1}, {0, -1}, {1, 0}, {0, 1}, {-1, 0}, {0, 0}};
    for (int a = 0; a < n; ++a) {
      int qs = q[a][0], qt = q[a][1];
      if (n == 9) {
        N[a] = quad1(qs, s) * quad1(qt, t);
        Ds[a] = dquad1(qs, s) * quad1(qt, t);
        Dt[a] = quad1(qs, s) * dquad1(qt, t);
      } else if (qs != 0 && qt != 0) {
        double fs = (1 + qs * s) / 4, ft = 1 + qt * t, e = qs * s + qt * t - 1;
        N[a] = fs * ft * e;
        Ds[a] = qs / 4.0 * ft * e + fs * ft * qs;
        Dt[a] = fs * qt * e + fs * ft * qt;
      } else if (qs == 0) {
        N[a] = (1 - s * s) * (1 + qt * t) / 2;
        Ds[a] = -s * (1 + qt * t);
        Dt[a] = (1 - s * s) * qt / 2;
      } else {
        N[a] = (1 + qs * s) * (1 - t * t) / 2;
        Ds[a] = qs * (1 - t * t) / 2;
        Dt[a] = -t * (1 + qs * s);
      }
    }
  }
  for (int d = 0; d < 3; ++d) x[d] = ts[d] = tt[d] = 0;
  for (int a = 0; a < n; ++a)
    for (int d = 0; d < 3; ++d) {
      x[d] += N[a] * xf[a * 3 + d];
      ts[d] += Ds[a] * xf[a * 3 + d];
      tt[d] += Dt[a] * xf[a * 3 + d];
    }
}
