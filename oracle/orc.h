/*
 * CPU restatement of miniCFD's DG/DGSEM residual + SSP-RK path (the ORACLE).
 *
 * This is TEST INFRASTRUCTURE.  It is the parity checker for the GPU library
 * and the timed CPU baseline.  Only tests/, __graft_entry__.smoke() and the
 * cpu_baseline / reference legs of bench.py load it.  The product library
 * never links, loads or calls it.
 *
 * Every routine restates one reference routine (file:line in the reference
 * project pvcStillInGradSchool/pvcRiemannSolvers) in plain C, keeping the
 * reference's operation order where that order is observable:
 *   gas conversions          include/mini/riemann/euler/types.hpp:186-334
 *   Exact / HLLC / AUSM      include/mini/riemann/euler/{exact,hllc,ausm}.hpp
 *   Roe / Lax-Friedrichs     python/riemann.py:405-476 (1D), restated in 3D
 *   rotated wrapper + BCs    include/mini/riemann/rotated/euler.hpp:42-345
 *   GLL rule                 include/mini/integrator/lobatto.hpp:37-83
 *   Lagrange line basis      include/mini/basis/lagrange.hpp:53-142
 *   Hex8 map / face table    include/mini/coordinate/hexahedron.hpp:353-490
 *   face frames              include/mini/coordinate/face.hpp:54-62
 *   quadrature points        include/mini/integrator/element.hpp:102-115
 *   DGSEM residual           include/mini/spatial/dg/lobatto.hpp:58-302
 *   residual orchestration   include/mini/spatial/fem.hpp:248-307
 *   time step                include/mini/spatial/fem.hpp:417-435
 *   SSP-RK1/2/3              include/mini/temporal/rk.hpp:16-49, ode.hpp:121-133
 */
#ifndef MCFD_ORACLE_ORC_H_
#define MCFD_ORACLE_ORC_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define ORC_K 5

/* Riemann solver kinds (same numbering as the product's mcfd.h). */
enum { ORC_EXACT = 0, ORC_HLLC = 1, ORC_AUSM = 2, ORC_ROE = 3, ORC_RUSANOV = 4 };

/* Boundary kinds (same numbering as the product's mcfd.h). */
enum {
  ORC_BC_NONE = 0,
  ORC_BC_INVISCID_WALL = 1,
  ORC_BC_SUPERSONIC_INLET = 2,
  ORC_BC_SUPERSONIC_OUTLET = 3,
  ORC_BC_SUBSONIC_INLET = 4,
  ORC_BC_SUBSONIC_OUTLET = 5,
  ORC_BC_SMART = 6,
  ORC_BC_NO_SLIP_WALL = 7 /* viscous fr::Lobatto only (spatial/fr/lobatto.hpp:298-317) */
};

/* Given-state programs for boundaries that need an exterior value: the
 * std::function<Value(Global, double)> of spatial/fem.hpp:196-222 for the
 * demos' functions. */
enum { ORC_STATE_CONSTANT = 0, ORC_STATE_MOVING_SPLIT = 1, ORC_STATE_OBLIQUE_SPLIT = 2,
       ORC_STATE_TABLE = 3 };

/* One boundary group: kind, and the given value program
 * value(x, t) = (x[axis] - speed * t) < position ? a : b         (MOVING_SPLIT)
 * value(x, t) = (normal . x - speed * t) < position ? a : b      (OBLIQUE_SPLIT)
 * value(x, t) = table[point] (the function sampled at every face
 *               point of the mesh, [face points][K], by global face-point
 *               index)                                             (TABLE)
 * value(x, t) = a                                                  (CONSTANT)   */
typedef struct {
  int kind;
  int program;
  int axis;
  double position, speed;
  double a[ORC_K], b[ORC_K];
  double normal[3];
  const double *table;
} orc_bc;

/* ---- point functions (used by the golden-vector tests) ---- */
void orc_cons_to_prim(const double *cons, double *prim);
void orc_prim_to_cons(const double *prim, double *cons);
void orc_flux_matrix(const double *cons, double *mat15); /* row-major 5x3 */
double orc_max_speed(const double *cons);
/* 1D (normal-frame) upwind flux from primitive (rho, u, v, w, p) pairs. */
void orc_flux_1d(int kind, const double *prim_l, const double *prim_r,
                 double *flux);
/* Rotated flux: frame = {normal, tangent, bitangent} row-major 3x3. */
void orc_flux_rotated(int kind, const double *frame, const double *cons_l,
                      const double *cons_r, double *flux);
void orc_flux_boundary(int riemann, int bc_kind, const double *frame,
                       const double *cons_in, const double *given,
                       double *flux);

/* ---- mesh + DGSEM ---- */
typedef struct orc_mesh orc_mesh;

/* The mesh description shared with the product (see include/mcfd.h).
 * cell_nodes: stride entries per cell (0: 8), CGNS order; cell_type NULL
 * for all Hex8, else ORC_CELL_HEX8 / HEX27 / HEX20 (the Hex27 / Hex20 maps of
 * coordinate/hexahedron.hpp give curved cells); faces: holder, sharer (-1 on a
 * boundary), the local face index on each side, the boundary group (-1 for
 * interior faces) and an optional periodic shift such that
 * x(sharer side) + shift = x(holder side). */
orc_mesh *orc_mesh_create(int64_t n_nodes, const double *xyz, int64_t n_cells,
                          const int64_t *cell_nodes, const int32_t *cell_type,
                          int32_t stride, int64_t n_faces,
                          const int64_t *face_cells, const int32_t *face_sides,
                          const int32_t *face_group, const double *face_shift,
                          int degree);
void orc_mesh_destroy(orc_mesh *m);
int64_t orc_column_size(const orc_mesh *m);
int orc_nodes_per_cell(const orc_mesh *m);
/* Node matching tables (reference dg/lobatto.hpp:58-78): int16 per face point;
 * sharer entries of boundary faces are -1. */
int orc_face_node_maps(const orc_mesh *m, int16_t *holder, int16_t *sharer);
/* Per node global coordinates [n_cells][N][3] and global weights [n_cells][N]. */
int orc_node_geometry(const orc_mesh *m, double *xyz, double *weights);
/* Per face point global coordinates / weights / frames. */
int orc_face_geometry(const orc_mesh *m, double *xyz, double *weights,
                      double *frames);
double orc_cell_length(const orc_mesh *m, int64_t i_cell);

void orc_set_threads(int n);
int orc_get_threads(void);

/* Spatial scheme of a mesh's residual: dg::Lobatto (default) or fr::Lobatto
 * with Huynh's g2 correction (spatial/fr/lobatto.hpp). */
enum { ORC_SCHEME_DGSEM = 0, ORC_SCHEME_FR = 1 };
void orc_mesh_set_scheme(orc_mesh *m, int scheme);

/* GetResidualColumn of dg::Lobatto (lumped mass divide included) or of
 * fr::Lobatto (divided by det J), by the mesh's scheme. */
int orc_dgsem_residual(const orc_mesh *m, int riemann, int n_bc,
                       const orc_bc *bcs, double t, const double *u, double *r);
/* FiniteElement::GetTimeStep with an explicit CFL number (cfl <= 0 selects
 * the reference table cfl_[rk_order][p]). */
double orc_time_step(const orc_mesh *m, const double *u, double dt_guess,
                     int rk_order, double cfl);
/* RungeKutta<order>::Update over the DGSEM system, in place on u. */
int orc_rk_update(const orc_mesh *m, int riemann, int n_bc, const orc_bc *bcs,
                  int order, double t, double dt, double *u);

/* RungeKutta<order>::Update on the linear system du/dt = A u (temporal
 * test physics, reference ode.hpp:55-85); A row-major n x n. */
int orc_rk_update_linear(int order, int64_t n, const double *a, double t,
                         double dt, double *u);

/* ---- WENO limiter on DGSEM cells (orc_weno.c) ---- */
/* LAZY: weno::Lazy on every cell; DETECT_LAZY: Lazy reconstruction of the
 * cells the weno::Eigen jump detector flags; EIGEN: weno::Eigen (jump
 * detector + characteristic-wise reconstruction, limiter/weno.hpp:196-348). */
enum { ORC_LIMITER_NONE = 0, ORC_LIMITER_LAZY = 1, ORC_LIMITER_DETECT_LAZY = 2, ORC_LIMITER_EIGEN = 3,
       /* tests only: the characteristic reconstruction on every cell */
       ORC_LIMITER_EIGEN_ALL = 4 };
/* EigenMatrices (riemann/euler/eigen.hpp:27-56) of a conservative state in
 * the frame {nu, mu, pi} (rows of frame9); L, R row-major 5x5. */
void orc_eigen_matrices(const double *cons, const double *frame9, double *L, double *R);
typedef struct orc_limiter orc_limiter;
orc_limiter *orc_limiter_create(const orc_mesh *m);
void orc_limiter_destroy(orc_limiter *l);
int orc_modal_count(int p);
int orc_limiter_modal_count(const orc_limiter *l);
/* modal coefficients [cells][K][M] of a nodal column */
void orc_limiter_modal(const orc_limiter *l, const double *u, double *modal);
/* limiter::Reconstruct in place; returns the number of reconstructed cells */
int64_t orc_limit(const orc_limiter *l, int mode, double w0, double eps,
                  double *u);
/* GetSmoothness (weno.hpp:78-95) of modal coeff cm [K][M] on cell c */
void orc_limiter_smoothness(const orc_limiter *l, int64_t c, const double *cm,
                            double *beta);
/* jump-detector flags [cells]; returns the troubled count */
int64_t orc_limiter_troubled(const orc_limiter *l, const double *u,
                             char *flags);
/* The limiter on the modal scheme's cells (WithLimiter<dg::General> over
 * Projection); orc_limit then works on the modal column [cells][M][K]. */
typedef struct orc_modal orc_modal;
orc_limiter *orc_modal_limiter_create(const orc_modal *m);
/* RungeKutta<order>::Update on WithLimiter<dg::Lobatto>: the limiter runs
 * after every SetSolutionColumn (spatial/with_limiter.hpp:56-59). */
int orc_rk_update_limited(const orc_mesh *m, int riemann, int n_bc,
                          const orc_bc *bcs, int order, double t, double dt,
                          double *u, const orc_limiter *l, int mode, double w0,
                          double eps);

/* ---- modal DG: dg::General over Projection on Hex8 / Tet4 (orc_modal.c) ---- */
enum { ORC_CELL_HEX8 = 0, ORC_CELL_TET4 = 1, ORC_CELL_HEX27 = 2, ORC_CELL_TET10 = 3,
       ORC_CELL_HEX20 = 4, ORC_CELL_WEDGE6 = 5, ORC_CELL_PYRA5 = 6, ORC_CELL_WEDGE15 = 7,
       ORC_CELL_WEDGE18 = 8, ORC_CELL_PYRA13 = 9, ORC_CELL_PYRA14 = 10 };
/* Same mesh description as orc_mesh_create plus cell types (NULL: all Hex8);
 * a Tet4 cell uses the first 4 of its 8 cell_nodes entries (CGNS order) and
 * local faces 0..3 of Tetrahedron4::faces_.  Column layout per cell: [M][K]. */
orc_modal *orc_modal_create(int64_t n_nodes, const double *xyz, int64_t n_cells,
                            const int64_t *cell_nodes, const int32_t *cell_type,
                            int32_t stride, int64_t n_faces, const int64_t *face_cells,
                            const int32_t *face_sides, const int32_t *face_group,
                            const double *face_shift, int degree);
void orc_modal_destroy(orc_modal *m);
int64_t orc_modal_column_size(const orc_modal *m);
int orc_modal_basis_count(const orc_modal *m);
/* volume quadrature points of all cells, cell by cell in integrator order */
int64_t orc_modal_point_count(const orc_modal *m);
int orc_modal_points(const orc_modal *m, double *xyz, double *weights);
int64_t orc_modal_face_point_count(const orc_modal *m);
int orc_modal_face_points(const orc_modal *m, double *xyz, double *weights,
                          double *frames);
double orc_modal_cell_length(const orc_modal *m, int64_t c);
/* solution values [points][K] at the volume points */
int orc_modal_values(const orc_modal *m, const double *u, double *values);
/* Approximate from values [points][K] at the volume points */
int orc_modal_project(const orc_modal *m, const double *values, double *u);
int orc_modal_residual(const orc_modal *m, int riemann, int n_bc,
                       const orc_bc *bcs, double t, const double *u, double *r);
double orc_modal_time_step(const orc_modal *m, const double *u, double dt_guess,
                           int rk_order, double cfl);
int orc_modal_rk_update(const orc_modal *m, int riemann, int n_bc,
                        const orc_bc *bcs, int order, double t, double dt,
                        double *u);
/* RungeKutta<order>::Update on WithLimiter<dg::General>: the limiter runs
 * after every SetSolutionColumn (spatial/with_limiter.hpp:56-59). */
int orc_modal_rk_update_limited(const orc_modal *m, int riemann, int n_bc,
                                const orc_bc *bcs, int order, double t, double dt,
                                double *u, const orc_limiter *l, int mode, double w0,
                                double eps);

/* ---- output sampling, Writer<Part>::Prepare (mesh/vtk.hpp:428-493) ---- */
/* nodal mesh: every cell at the 27 VTK Hexahedron27 locals; xyz
 * [cells][27][3], values [cells][27][K] of the GLL Lagrange interpolant */
int orc_vtk_sample(const orc_mesh *m, const double *u, double *xyz, double *values);
/* modal mesh: Hex8 -> Hexahedron27 (type 29), Tet4 -> Tetrahedron10 (type
 * 24), cell by cell; returns the number of points */
int64_t orc_modal_vtk_sample(const orc_modal *m, const double *u, double *xyz,
                             double *values, uint8_t *types);

/* ---- energy-based artificial viscosity on fr::Lobatto (orc_visc.c) ----
 * EnergyBasedViscosity<Part, ConvectionDiffusion<rotated::Euler<...>,
 * Direct<Isotropic>>> with WithViscosity<fr::Lobatto> (spatial/viscosity.hpp,
 * spatial/with_viscosity.hpp, riemann/diffusive/direct.hpp), Hex8 cells.
 * The mesh must use ORC_SCHEME_FR.  Creating the object builds the damping
 * matrices the way BuildDampingMatrices does (viscosity.hpp:299-384). */
typedef struct orc_visc orc_visc;
orc_visc *orc_visc_create(const orc_mesh *m, double beta0, double beta1, double time_scale);
void orc_visc_destroy(orc_visc *v);
/* damping matrices [cells][N][N] (row-major) */
const double *orc_visc_damping(const orc_visc *v);
/* IntegrateJumpOnFaces (viscosity.hpp:446-475): [cells][K] */
void orc_visc_jumps(const orc_visc *v, const double *u, double *jumps);
/* UpdateProperties: GetViscosityValues (viscosity.hpp:477-544) of the
 * solution u; nu [cells][K]; *min_dt = GetMinimumTimeStep() */
void orc_visc_properties(const orc_visc *v, const double *u, double *nu, double *min_dt);
/* GetResidualColumn of fr::Lobatto over the viscous Riemann object with
 * given cell viscosities nu [cells][K] (fr/general.hpp:249-515). */
int orc_visc_residual(const orc_visc *v, int riemann, int n_bc, const orc_bc *bcs,
                      double t, const double *u, const double *nu, double *r);
/* WithViscosity::GetTimeStep (with_viscosity.hpp:67-71) after
 * UpdateProperties on u: min(2 cfl min_dt, dt_guess); cfl <= 0 selects the
 * table. */
double orc_visc_time_step(const orc_visc *v, const double *u, double dt_guess, int rk_order,
                          double cfl);
/* RungeKutta<order>::Update on WithViscosity<fr::Lobatto>: every residual
 * uses the viscosities of its own input (SetSolutionColumn runs
 * UpdateProperties, with_viscosity.hpp:56-59). */
int orc_visc_rk_update(const orc_visc *v, int riemann, int n_bc, const orc_bc *bcs, int order,
                       double t, double dt, double *u);
/* Global value, gradient [3][K] and Hessian [6][K] (XX XY XZ YY YZ ZZ) at
 * node q of cell c (Hexahedron::GetGlobalValueGradientHessian, kLocal =
 * false, polynomial/hexahedron.hpp:586-595). */
void orc_visc_node_derivatives(const orc_visc *v, const double *u, int64_t c, int q,
                               double *grad, double *hess);
/* Initial limiters of the viscous demos: limiter::average::Reconstruct and
 * limiter::majority::Reconstruct (limiter/average.hpp:11-28,
 * limiter/majority.hpp:14-42), in place.  Returns the number of cells that
 * have a component without a strict majority value (left unchanged). */
enum { ORC_INIT_AVERAGE = 1, ORC_INIT_MAJORITY = 2 };
int64_t orc_initial_limiter(const orc_mesh *m, int kind, double *u);

#ifdef __cplusplus
}
#endif
#endif /* MCFD_ORACLE_ORC_H_ */
