/* ORACLE internals shared between orc_dg.c and orc_weno.c (test
 * infrastructure only). */
#ifndef MCFD_ORACLE_ORC_INTERNAL_H_
#define MCFD_ORACLE_ORC_INTERNAL_H_

#include <stdint.h>

#include "orc.h"

#define ORC_MAXQ 6

/* Mesh of the nodal schemes (built by orc_mesh_create, orc_dg.c). */
struct orc_mesh {
  int p, q, n, qf; /* degree, line points, nodes per cell, points per face */
  int64_t n_cells, n_faces;
  double xq[ORC_MAXQ], wq[ORC_MAXQ], d[ORC_MAXQ * ORC_MAXQ];
  /* per cell */
  double *node_xyz;   /* [cells][N][3] */
  double *node_w;     /* [cells][N]  global weights */
  double *grad;       /* [cells][N][3][N]  basis global gradients */
  double *length;     /* [cells] */
  double *cell_center; /* [cells][3] Hex8 LocalToGlobal(0, 0, 0) */
  double *corners;    /* [cells][27][3] node coordinates (the type's first n) */
  int32_t *type;      /* [cells] ORC_CELL_HEX8 / HEX27 / HEX20 */
  double *jdi;        /* [cells][N][9] det(J) J^-1 (GetJacobianAssociated) */
  double *detj;       /* [cells][N] det(J) */
  int32_t *face_sides; /* [faces][2] local face index in holder / sharer */
  int scheme;          /* ORC_SCHEME_DGSEM or ORC_SCHEME_FR */
  /* per face */
  int64_t *face_cells; /* [faces][2] */
  int32_t *face_group; /* [faces] */
  double *face_shift;  /* [faces][3] periodic shift (zeros when absent) */
  double *face_xyz;    /* [faces][QF][3] */
  double *face_w;      /* [faces][QF] */
  double *face_frame;  /* [faces][QF][9] */
  int16_t *map_h, *map_s; /* [faces][QF] */
};

/* Mesh of the modal scheme (built by orc_modal_create, orc_modal.c). */
struct orc_modal {
  int p, m;
  int64_t n_cells, n_faces;
  int64_t *vp_off;     /* [cells + 1] volume point offsets */
  double *vx, *vw;     /* [points][3] global coordinates, [points] global weights */
  double *center;      /* [cells][3] */
  double *s;           /* [cells][M][M] */
  double *length;      /* [cells] */
  int64_t *fp_off;     /* [faces + 1] */
  double *fx, *fw, *ff; /* face points: coordinates, weights, frames [9] */
  int64_t *face_cells;
  int32_t *face_group;
  double *face_shift;
  double *corners;     /* [cells][8][3] (Tet4: first 4) */
  int32_t *type;       /* [cells] ORC_CELL_* */
};

/* Lagrange derivative of the FR correction at the right end, g_R'(1)
 * (basis/vincent.hpp:30-32, 73-89). */
double orc_fr_g_prime(int p);
/* Lagrange second derivatives on the line points x [q]: d2[a * q + i] = l_i''(x_a). */
void orc_lagrange_second(int q, const double *x, double *d2);

int orc_mesh_degree(const orc_mesh *m);
int64_t orc_mesh_cells(const orc_mesh *m);
int64_t orc_mesh_faces(const orc_mesh *m);
const int64_t *orc_mesh_face_cells(const orc_mesh *m);
const double *orc_mesh_face_shift(const orc_mesh *m);
/* Hex8 LocalToGlobal(0, 0, 0) of every cell, [cells][3]. */
void orc_cell_centers(const orc_mesh *m, double *center);

/* Taylor monomials about a centre (basis/taylor.hpp:198-218), t [M] at the
 * offset d = x - centre; gradients g [3][M]. */
void orc_taylor_values(int M, const double *d, double *t);
void orc_taylor_grad(int M, const double *d, double *g);
/* OrthoNormalize (integrator/function.hpp:139-172). */
void orc_orthonormalize(int M, int nq, const double *T, const double *W, double *S);

/* RungeKutta<order>::Update (temporal/rk.hpp:16-49) over any residual; the
 * hook runs after every SetSolutionColumn. */
typedef int (*orc_residual_fn)(void *ctx, double t, const double *u, double *r);
typedef void (*orc_set_hook)(void *ctx, double *u);
int orc_rk_generic(orc_residual_fn fn, void *ctx, int64_t L, int order, double t,
                   double dt, double *u, orc_set_hook hook, void *hook_ctx);

/* Cell maps (orc_geom.c): node count of a type, whether it is a
 * tetrahedron, the local coordinates of node a, and x(loc) with
 * jac[r * 3 + d] = d x_d / d loc_r for the type's nodes xn [n][3]. */
int orc_type_nodes(int type);
int orc_type_is_tet(int type);
int orc_type_is_wedge(int type);
int orc_type_is_pyramid(int type);
/* nodes of a quadratic pyramid's face in its face map's order; the point and
 * tangents of a Triangle6 (n = 6) / Quadrangle8 (8) / Quadrangle9 (9) map */
int orc_pyramid_face_nodes(int type, int side, int *v);
void orc_face_map(int n, const double *xf, double s, double t, double *x, double *ts, double *tt);
void orc_local_of_node(int type, int a, double *loc);
void orc_map_point(int type, const double *xn, const double *loc, double *x, double *jac);
/* local faces of a type (4, 5 or 6), the corners of local face `side` in v
 * (the return value: 3 or 4), and the type's local centre (BuildCenter). */
int orc_type_faces(int type);
int orc_type_face_corners(int type, int side, int *v);
void orc_type_center(int type, double *loc);

#endif /* MCFD_ORACLE_ORC_INTERNAL_H_ */
