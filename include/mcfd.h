/*
 * mcfd.h -- C ABI of the GB300-native DG/DGSEM residual and SSP Runge-Kutta
 * update for the 3D Euler equations (miniCFD's mini::spatial / mini::temporal
 * hot path), for sm_103a.
 *
 * Every entry point takes plain pointers and sizes and returns an int status
 * (MCFD_OK == 0).  One handle owns the device copy of one mesh and its
 * solution column; it is used by one host thread at a time, and calls on one
 * handle are ordered on the handle's CUDA stream.
 *
 * Column layout (identical to the reference so Set/GetSolutionColumn are a
 * drop-in): for cell c (in mesh order), node q (i*Q*Q + j*Q + k, i outer) and
 * component k (rho, rho*u, rho*v, rho*w, rho*E):
 *     column[c * 5 * N + q * 5 + k],   N = (p + 1)^3   (DGSEM)
 * which is the memcpy of the per-cell Eigen K x N column-major coefficient
 * block in the reference (include/mini/polynomial/expansion.hpp:83-90) placed
 * at Part::GetCellDataOffset (include/mini/mesh/part.hpp:784-797).
 *
 * Reference interfaces replaced (pvcStillInGradSchool/pvcRiemannSolvers):
 *   include/mini/temporal/ode.hpp:17-48     System<Scalar> virtual quartet
 *   include/mini/temporal/ode.hpp:92-133    Solver / Euler
 *   include/mini/temporal/rk.hpp:10-57      RungeKutta<1|2|3>
 *   include/mini/spatial/fem.hpp:196-258    BC registration, Set/Get columns
 *   include/mini/spatial/fem.hpp:417-435    GetTimeStep
 *   include/mini/spatial/dg/lobatto.hpp     dg::Lobatto (DGSEM) residual
 *   include/mini/riemann/rotated/euler.hpp  rotated Riemann/BC fluxes
 *   include/mini/spatial/with_limiter.hpp   limiter after SetSolutionColumn
 */
#ifndef MCFD_H_
#define MCFD_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define MCFD_ABI_VERSION 2
#define MCFD_K 5

/* Status codes. */
enum mcfd_status {
  MCFD_OK = 0,
  MCFD_ERR_ARGUMENT = 1,      /* bad argument or size mismatch */
  MCFD_ERR_MESH = 2,          /* inconsistent mesh (index or face matching) */
  MCFD_ERR_CUDA = 3,          /* CUDA runtime error (message in last_error) */
  MCFD_ERR_STATE = 4,         /* non-finite value produced by a kernel */
  MCFD_ERR_NOT_CONVERGED = 5, /* Exact solver hit its iteration cap */
  MCFD_ERR_UNSUPPORTED = 6,   /* option combination not built */
  MCFD_ERR_NO_DEVICE = 7,     /* no CUDA device / wrong architecture */
  MCFD_ERR_IO = 8             /* file cannot be written / read / verified */
};

/* Riemann solvers.  Exact / HLLC / AUSM follow
 * include/mini/riemann/euler/{exact,hllc,ausm}.hpp; Roe and Rusanov follow the
 * reference's 1D prototype python/riemann.py:405-476 extended to 3D. */
enum mcfd_riemann {
  MCFD_EXACT = 0,
  MCFD_HLLC = 1,
  MCFD_AUSM = 2,
  MCFD_ROE = 3,
  MCFD_RUSANOV = 4
};

/* Boundary kinds (include/mini/spatial/fem.hpp:196-222 registry,
 * include/mini/riemann/rotated/euler.hpp:144-318 fluxes). */
enum mcfd_bc_kind {
  MCFD_BC_NONE = 0,
  MCFD_BC_INVISCID_WALL = 1,     /* SetInviscidWall */
  MCFD_BC_SUPERSONIC_INLET = 2,  /* SetSupersonicInlet(value) */
  MCFD_BC_SUPERSONIC_OUTLET = 3, /* SetSupersonicOutlet */
  MCFD_BC_SUBSONIC_INLET = 4,    /* SetSubsonicInlet(p0, cos x/y/z, T0) */
  MCFD_BC_SUBSONIC_OUTLET = 5,   /* SetSubsonicOutlet(value[4] = p) */
  MCFD_BC_SMART = 6,             /* SetSmartBoundary(value) */
  MCFD_BC_NO_SLIP_WALL = 7       /* SetNoSlipWall (fem.hpp:213-219); MCFD_FR only: with
                                    the artificial viscosity the wall flux minus
                                    nu n . grad(u) (fr/general.hpp:460-476), without
                                    it no correction (:455-459) */
};

/* The reference passes a std::function<Value(Global, double t)> per boundary
 * name (spatial/fem.hpp:196-222).  The ABI carries that function as a small
 * program evaluated on the device at every boundary face point and stage
 * time:
 *   CONSTANT:       value = a
 *   MOVING_SPLIT:   value = (x[axis] - speed * t) < position ? a : b
 *                   (the moving-shock boundaries of demo/euler/riemann2d.cpp)
 *   OBLIQUE_SPLIT:  value = (normal . x - speed * t) < position ? a : b
 *                   (the oblique moving shock of demo/euler/double_mach.cpp:
 *                   normal = (tan 60, -1, 0), speed = tan 60 * u_x,
 *                   position = tan 60 * x_gap, a = post-shock, b = pre-shock)
 *   TABLE:          a value per face point of the group, set by
 *                   mcfd_set_bc_table: any function of the position alone,
 *                   sampled once by the caller at mcfd_bc_points (e.g. the
 *                   right boundary of demo/euler/shu_osher.cpp, whose state
 *                   is the initial sine profile)
 * a and b are conservative states, or for SUBSONIC_INLET the tuple
 * (p_total, cos_x, cos_y, cos_z, T_total), as in the reference. */
enum mcfd_state_program {
  MCFD_STATE_CONSTANT = 0,
  MCFD_STATE_MOVING_SPLIT = 1,
  MCFD_STATE_OBLIQUE_SPLIT = 2,
  MCFD_STATE_TABLE = 3
};

typedef struct mcfd_bc_state {
  int32_t kind;    /* enum mcfd_bc_kind */
  int32_t program; /* enum mcfd_state_program */
  int32_t axis;    /* 0, 1, 2 (MOVING_SPLIT only) */
  int32_t reserved;
  double position;
  double speed;
  double a[MCFD_K];
  double b[MCFD_K];
  double normal[3]; /* OBLIQUE_SPLIT only (need not be a unit vector) */
} mcfd_bc_state;

/* Element types and their maps (coordinate/hexahedron.hpp Hexahedron8 /
 * Hexahedron20 / Hexahedron27, coordinate/tetrahedron.hpp Tetrahedron4 /
 * Tetrahedron10), nodes in CGNS order.  The quadratic types give curved
 * cells and faces; the hexahedra run every scheme, the tetrahedra the MODAL
 * scheme; the WENO limiter takes every cell type on the MODAL scheme and
 * Hex8 cells on the nodal schemes. */
enum mcfd_cell_type {
  MCFD_HEX8 = 0,
  MCFD_TET4 = 1,
  MCFD_HEX27 = 2,
  MCFD_TET10 = 3,
  MCFD_HEX20 = 4,
  MCFD_WEDGE6 = 5, /* coordinate/wedge.hpp Wedge6 (modal scheme): local (a, b, z), c = 1 - a - b */
  MCFD_PYRA5 = 6,  /* coordinate/pyramid.hpp Pyramid5 (modal scheme): collapsed local cube */
  MCFD_WEDGE15 = 7, /* coordinate/wedge.hpp Wedge15 (modal scheme), CGNS PENTA_15 node order */
  MCFD_WEDGE18 = 8, /* coordinate/wedge.hpp Wedge18 (modal scheme), CGNS PENTA_18 node order */
  MCFD_PYRA13 = 9,  /* coordinate/pyramid.hpp Pyramid13 (modal scheme), CGNS PYRA_13 node order */
  MCFD_PYRA14 = 10  /* coordinate/pyramid.hpp Pyramid14 (modal scheme), CGNS PYRA_14 node order */
};

/* Unstructured mesh, the input that replaces mesh::part::Part
 * (include/mini/mesh/part.hpp:97-291):
 *   xyz          [n_nodes][3] node coordinates
 *   cell_nodes   [n_cells][cell_node_stride] node ids in CGNS order; a cell
 *                uses the first 4 / 8 / 10 / 20 / 27 slots of its type (the
 *                rest are ignored)
 *   cell_type    [n_cells] enum mcfd_cell_type, or NULL for all Hex8.
 *   face_cells   [n_faces][2] holder, sharer (-1 on a boundary).  The face
 *                normal points from the holder to the sharer (outward on a
 *                boundary), as in part.hpp:1518-1538.
 *   face_sides   [n_faces][2] local face index in the holder and sharer:
 *                Hex8 0..5 in the order of coordinate/hexahedron.hpp:378-389,
 *                Tet4 0..3 in the order of Tetrahedron4::faces_
 *                (coordinate/tetrahedron.hpp:141-147)
 *   face_group   [n_faces] boundary group id (>= 0) or -1 for interior faces
 *   face_shift   [n_faces][3] or NULL: periodic translation such that
 *                x(sharer side) + shift = x(holder side).  The reference has
 *                no periodic boundary; a periodic face here is an ordinary
 *                interior face whose sharer is found through this shift. */
typedef struct mcfd_mesh_desc {
  int64_t n_nodes;
  const double *xyz;
  int64_t n_cells;
  const int64_t *cell_nodes;
  const int32_t *cell_type;
  int64_t n_faces;
  const int64_t *face_cells;
  const int32_t *face_sides;
  const int32_t *face_group;
  const double *face_shift;
  int32_t cell_node_stride; /* slots per cell in cell_nodes; 0 means 8 */
} mcfd_mesh_desc;

/* Spatial schemes:
 *   DGSEM: dg::Lobatto, weak form with lumped mass (spatial/dg/lobatto.hpp)
 *          on GLL-collocated hexahedra
 *   FR:    fr::Lobatto, flux reconstruction with Huynh's g2 correction
 *          (spatial/fr/general.hpp, spatial/fr/lobatto.hpp, basis/vincent.hpp);
 *          its time step is twice the DGSEM one (fr/lobatto.hpp:220-222)
 *   MODAL: dg::General over polynomial::Projection (spatial/dg/general.hpp,
 *          polynomial/projection.hpp) on every cell type: per-cell
 *          orthonormal Taylor basis, column block [M][K] per cell with
 *          M = (p+1)(p+2)(p+3)/6.  Quadrature: Hex8 Gauss-Legendre (p+1)^3,
 *          Quad4 faces (p+1)^2; Tet4 14 points (p <= 2) or 24 points (p = 3),
 *          Tri3 faces 6 points (p <= 2) or 12 points (p = 3)
 *          (integrator/{legendre,tetrahedron,triangle}.hpp).  FP64 or mixed
 *          (FP32 contractions, FP64 face states / Riemann / RK); any
 *          limiter (WithLimiter<dg::General>, demo/euler/sourceless.hpp). */
enum mcfd_scheme { MCFD_DGSEM = 0, MCFD_FR = 1, MCFD_MODAL = 2 };
enum mcfd_precision { MCFD_FP64 = 0, MCFD_MIXED = 1 };

/* Limiter applied after every solution update (spatial/with_limiter.hpp:56-65):
 *   LAZY:        weno::Lazy on every cell (limiter/weno.hpp:97-195)
 *   DETECT_LAZY: weno::Lazy reconstruction on the cells that the jump
 *                detector of weno::Eigen::IsNotSmooth flags
 *                (limiter/weno.hpp:230-258)
 * The modal basis is the per-cell orthonormalised Taylor basis of
 * polynomial::Extrapolation (polynomial/extrapolation.hpp). */
enum mcfd_limiter {
  MCFD_LIMITER_NONE = 0,
  MCFD_LIMITER_LAZY = 1,
  MCFD_LIMITER_DETECT_LAZY = 2,
  MCFD_LIMITER_EIGEN = 3   /* weno::Eigen: the jump detector, then the
                              characteristic-wise reconstruction in each
                              adjacent face's frame, averaged with the
                              neighbours' volumes (limiter/weno.hpp:259-348) */
};

typedef struct mcfd_options {
  int32_t degree;    /* polynomial degree p (1..3) */
  int32_t scheme;    /* enum mcfd_scheme */
  int32_t riemann;   /* enum mcfd_riemann */
  int32_t precision; /* enum mcfd_precision */
  double cfl;        /* <= 0: the reference table fem.hpp:26-37 */
  int32_t device;    /* CUDA device ordinal */
  int32_t limiter;   /* enum mcfd_limiter */
  double weno_w0;    /* linear weight of a neighbour; <= 0 selects 0.001 */
  double weno_eps;   /* smoothness offset; <= 0 selects 1e-6 */
  int32_t contraction; /* enum mcfd_contraction (mixed form) */
  int32_t shock_cells_fp64; /* mixed form with a WENO limiter on a nodal scheme:
                               n = 1 or 2 runs the cells that the last limiter
                               pass flagged, and n layers of face neighbours,
                               through the FP64 cell update (with FP64 face
                               fluxes and nodal-to-modal products);
                               the other cells stay mixed; 0 = off */
  int32_t reserved[2];
} mcfd_options;

/* Where the mixed form's DGSEM differentiation runs: the FP32 SIMT pipes
 * (default), or the tensor cores as TF32x3 compensated products with FP32
 * accumulation (mma.sync m16n8k8; DGSEM, p = 3, mixed form only). */
enum mcfd_contraction { MCFD_CONTRACTION_SIMT = 0, MCFD_CONTRACTION_TENSOR = 1 };

typedef struct mcfd_handle mcfd_handle;

/* Library identification. */
int mcfd_abi_version(void);

/* Builds the device-resident mesh and geometry.  Replaces the construction
 * of spatial::FiniteElement / dg::Lobatto (fem.hpp:95-115, lobatto.hpp:113-125):
 * Riemann frames per face point and face-point to cell-node matching. */
int mcfd_create(const mcfd_mesh_desc *mesh, const mcfd_options *options,
                mcfd_handle **out);
int mcfd_destroy(mcfd_handle *h);

/* Length of the solution column (Part::GetCellDataSize, part.hpp:793-797). */
int64_t mcfd_column_size(const mcfd_handle *h);

/* Boundary registration for one face group (fem.hpp:196-222). */
int mcfd_set_bc(mcfd_handle *h, int32_t group, const mcfd_bc_state *state);

/* Face points of boundary group `group` in the order a TABLE program takes
 * its values: the group's faces in mesh order, each face's quadrature points
 * in order.  xyz [n][3] host memory. */
int mcfd_bc_point_count(const mcfd_handle *h, int32_t group, int64_t *n);
int mcfd_bc_points(const mcfd_handle *h, int32_t group, double *xyz, int64_t n);
/* The values [n][5] of a group registered with program MCFD_STATE_TABLE, at
 * mcfd_bc_points (host memory, copied to the device; call after
 * mcfd_set_bc).  Until set, such a group's value is its state a. */
int mcfd_set_bc_table(mcfd_handle *h, int32_t group, const double *values, int64_t n);

/* System<Scalar> quartet (ode.hpp:17-48): host columns of length n. */
int mcfd_set_time(mcfd_handle *h, double t);
int mcfd_set_solution(mcfd_handle *h, const double *column, int64_t n);
int mcfd_get_solution(mcfd_handle *h, double *column, int64_t n);
/* GetResidualColumn of dg::Lobatto incl. the lumped mass divide
 * (fem.hpp:248-258, lobatto.hpp:143-158). */
int mcfd_residual(mcfd_handle *h, double *residual, int64_t n);

/* Same three calls on caller-owned device memory (no host copies). */
int mcfd_set_solution_device(mcfd_handle *h, const double *d_column, int64_t n);
int mcfd_get_solution_device(mcfd_handle *h, double *d_column, int64_t n);
int mcfd_residual_device(mcfd_handle *h, double *d_residual, int64_t n);

/* Residual that allocates nothing.  No counterpart in the reference.
 *
 * For callers that cannot call cudaMalloc while they run: a host program that
 * hands all device memory to its own pool at start-up and forbids further
 * allocations, or a time-critical loop where the implicit device
 * synchronisation of cudaMalloc/cudaFree is not acceptable.  The caller
 * passes the input column d_u and the output d_residual (device pointers,
 * length n = mcfd_column_size); the face-flux scratch is a fixed 16 MiB
 * device array inside the library (2,097,152 doubles, i.e. meshes with at
 * most 419,430 face points; larger meshes are rejected with
 * MCFD_ERR_ARGUMENT).  Every GPU that loads the library holds that array
 * until the process exits.  The first call on a device looks up the array's
 * device address (cudaGetSymbolAddress) and should come before any stream
 * capture.  All calls share the array and it keeps the last call's contents;
 * every scratch entry is written before it is read within a call, so nothing
 * needs clearing, but calls that overlap on the GPU (other threads or
 * streams) race on it.  Results equal mcfd_residual_device. */
int mcfd_residual_device_noalloc(mcfd_handle *h, const double *d_u,
                                 double *d_residual, int64_t n);

/* FiniteElement::GetTimeStep(dt_guess, rk_order) (fem.hpp:417-435). */
int mcfd_time_step(mcfd_handle *h, double dt_guess, int32_t rk_order,
                   double *dt);

/* RungeKutta<order>::Update(system, t, dt) (rk.hpp:16-49), fused on device. */
int mcfd_rk_step(mcfd_handle *h, double t, double dt, int32_t order);

/* The driver loop of demo/euler/sourceless.cpp:187-215 without I/O:
 * n_steps x { dt = GetTimeStep(dt_guess, order); Update(t, dt); t += dt },
 * with dt and t kept on the device (no host round trip per step).  *t is the
 * start time on entry and the end time on return. */
int mcfd_advance(mcfd_handle *h, int32_t n_steps, double dt_guess,
                 int32_t rk_order, double *t);

/* Streamed stepping: a sequence of jobs, each "load a column from host memory
 * at time t, mcfd_advance n_steps, store the result to host memory", where
 * the upload of job k+1 and the download of job k-1 overlap job k's compute
 * (two device staging slots, one copy stream per direction; each job's graph
 * steps its input slot straight into its output slot).  The loop of
 * demo/euler/sourceless.cpp:187-215 with SetSolutionColumn / GetSolutionColumn
 * around every step, pipelined.  mcfd_stream_step only enqueues: host_in must
 * stay unchanged and host_out unread until mcfd_stream_end returns.  Use
 * page-locked host memory for the copies to be asynchronous.  Each job's
 * result equals mcfd_set_solution(host_in) + mcfd_advance(n_steps, t) +
 * mcfd_get_solution(host_out); the handle's own solution is not touched.
 * mcfd_stream_end waits for every job and reports the first kernel status
 * (non-finite value, Exact-solver cap).  The staging (4 columns) is
 * allocated by the first mcfd_stream_begin and kept until mcfd_destroy. */
int mcfd_stream_begin(mcfd_handle *h);
int mcfd_stream_step(mcfd_handle *h, const double *host_in, double *host_out,
                     int64_t n, double t, int32_t n_steps, double dt_guess,
                     int32_t rk_order);
int mcfd_stream_end(mcfd_handle *h);

/* ---- mesh ingest ----
 * Face connectivity from cells alone, as Part::BuildLocalFaces /
 * BuildBoundaryFaces (mesh/part.hpp:932-1019, 1456-1545) derive it: (cell,
 * local face) slots are keyed by their sorted corner ids (cell_nodes with
 * cell_node_stride slots per cell, 0 meaning 8); equal keys pair into
 * interior faces with the lower cell id as holder (the shuffler's
 * [i_cell_small, i_cell_large] adjacency, mesh/shuffler.hpp:399-421).  Free
 * slots are boundary faces: bface_nodes [n_bfaces][4] (a triangle's 4th entry
 * is -1) with bface_group give their groups (free slots not listed get -1);
 * periodic_groups [n_periodic][2] = (a, b) with periodic_shift [n_periodic][3]
 * such that x(face of b) + shift = x(face of a) joins the two groups face by
 * face (matched by centroid) into interior faces.  Output arrays in
 * mcfd_mesh_desc form with capacity cap >= mcfd_face_slot_count(); order:
 * interior and periodic faces by (holder, holder side), then boundary faces
 * by (group, holder, side), ungrouped ones last.  MCFD_ERR_MESH with the
 * reason in mcfd_build_error() for a face shared by three cells, a boundary
 * element that is not a free face, or an unmatched periodic face. */
int64_t mcfd_face_slot_count(int64_t n_cells, const int32_t *cell_type);
int mcfd_build_faces(int64_t n_nodes, const double *xyz, int64_t n_cells,
                     const int64_t *cell_nodes, const int32_t *cell_type,
                     int32_t cell_node_stride, int64_t n_bfaces, const int64_t *bface_nodes,
                     const int32_t *bface_group, int32_t n_periodic,
                     const int32_t *periodic_groups, const double *periodic_shift,
                     int64_t cap, int64_t *face_cells, int32_t *face_sides,
                     int32_t *face_group, double *face_shift, int64_t *n_faces);
const char *mcfd_build_error(void);
/* The same faces, index for index, with the keying and pairing of the face
 * slots on GPU `device` (hash table + prefix sums); the free slots (O(n^(2/3)))
 * are grouped and ordered on the host as above.  Needs n_nodes < 2^32;
 * MCFD_ERR_CUDA for device errors. */
int mcfd_build_faces_gpu(int32_t device, int64_t n_nodes, const double *xyz,
                         int64_t n_cells, const int64_t *cell_nodes,
                         const int32_t *cell_type, int32_t cell_node_stride,
                         int64_t n_bfaces, const int64_t *bface_nodes,
                         const int32_t *bface_group, int32_t n_periodic,
                         const int32_t *periodic_groups, const double *periodic_shift,
                         int64_t cap, int64_t *face_cells, int32_t *face_sides,
                         int32_t *face_group, double *face_shift, int64_t *n_faces);
/* Legacy VTK unstructured grid reader (ASCII or BINARY; CELLS in the classic
 * or the version-5 OFFSETS / CONNECTIVITY layout): hexahedra (12) and
 * tetrahedra (10) become cells in mcfd_mesh_desc form (VTK and CGNS share
 * their corner order), quads (9) and triangles (5) boundary elements whose
 * group is the integral CELL_DATA array named group_array (NULL: the first
 * single-component one; 0 without any).  Feed the result to
 * mcfd_build_faces.  MCFD_ERR_IO with the reason in mcfd_vtk_error(). */
typedef struct mcfd_vtk_mesh mcfd_vtk_mesh;
int mcfd_vtk_read(const char *path, const char *group_array, mcfd_vtk_mesh **out);
int mcfd_vtk_mesh_sizes(const mcfd_vtk_mesh *m, int64_t *n_nodes, int64_t *n_cells,
                        int64_t *n_bfaces);
/* Slots per cell of cell_nodes: 8, or up to 27 when the file holds quadratic
 * cells (VTK 25 / 29 hexahedra, 24 tetrahedra, 26 / 32 wedges, 27
 * pyramids), which are read into CGNS node order (MCFD_HEX20 / HEX27 /
 * TET10 / WEDGE15 / WEDGE18 / PYRA13). */
int mcfd_vtk_mesh_stride(const mcfd_vtk_mesh *m, int32_t *stride);
/* xyz [n_nodes][3], cell_nodes [n_cells][stride] (unused slots -1),
 * cell_type [n_cells], bface_nodes [n_bfaces][4] (triangles end in -1),
 * bface_group. */
int mcfd_vtk_mesh_arrays(const mcfd_vtk_mesh *m, double *xyz, int64_t *cell_nodes,
                         int32_t *cell_type, int64_t *bface_nodes, int32_t *bface_group);
void mcfd_vtk_mesh_destroy(mcfd_vtk_mesh *m);
const char *mcfd_vtk_error(void);
/* order[k] = the point (cell centroid) at position k along a 3D Hilbert
 * curve through the points' bounding cube (21 bits per axis; Skilling 2004).
 * Renumbering cells in this order (in place of the reference's METIS
 * shuffle, mesh/shuffler.hpp) keeps face neighbours close in memory. */
int mcfd_hilbert_order(int64_t n, const double *points, int64_t *order);

/* ---- output and restart ----
 * Writer<Part>::WriteSolutions (mesh/vtk.hpp:526-669): every cell is written
 * as a disconnected VTK element, Hex8 cells as Hexahedron27 (type 29) and
 * Tet4 cells as Tetrahedron10 (type 24), carrying the conservative variables
 * (Density, MomentumX/Y/Z, EnergyStagnationDensity) at the element's VTK
 * nodes (Writer::Prepare, vtk.hpp:428-493: LocalToGlobalAndValue at the VTK
 * local coordinates).  Points are cell by cell, 27 or 10 per cell. */
int mcfd_vtk_point_count(const mcfd_handle *h, int64_t *n_points);
/* xyz [n_points][3], values [n_points][5], types [n_cells] (host memory). */
int mcfd_vtk_sample(mcfd_handle *h, double *xyz, double *values, uint8_t *types,
                    int64_t n_points);
/* <directory>/<soln_name>.pvtu and <directory>/<soln_name>/0.vtu in the
 * reference's layout: values ASCII at the stream's default 6 significant
 * digits, points base64 (binary = 0, as the reference); binary = 1 writes
 * values, offsets and types base64 as well (full precision).  The
 * directories are created as needed. */
int mcfd_write_vtu(mcfd_handle *h, const char *directory, const char *soln_name,
                   int32_t binary);
/* The writer alone, on host arrays as mcfd_vtk_sample returns them (types
 * 29 or 24); needs no device. */
int mcfd_write_vtu_arrays(const char *directory, const char *soln_name,
                          int64_t n_points, const double *xyz,
                          const double *values, int64_t n_cells,
                          const uint8_t *types, int32_t binary);
/* Base64 of the VTK binary arrays (mesh/vtk.hpp:21-91 EncodeBase64): writes
 * the text and a terminating NUL to out (capacity cap) and its length to
 * *written; out = NULL only queries the length. */
int mcfd_base64_encode(const uint8_t *data, int64_t n, char *out, int64_t cap,
                       int64_t *written);

/* Part::GatherSolutions / ScatterSolutions (mesh/part.hpp:380-395,
 * 1053-1069): the DataOnCells fields, field-major [F][n_cells] with
 * F = column / n_cells and field i of cell c = value i of the cell's column
 * block (device pointers, n = column size).  Scatter replaces the solution
 * without running the limiter, as ScatterFields sets the coefficients. */
int mcfd_gather_fields(mcfd_handle *h, double *d_fields, int64_t n);
int mcfd_scatter_fields(mcfd_handle *h, const double *d_fields, int64_t n);
/* Part::WriteSolutions / ReadSolutions (mesh/part.hpp:1070-1208) with a
 * binary file in place of CGNS: a header (magic "MCFDRST", version 1,
 * scheme, degree, F, n_cells, t, 64-bit FNV-1a checksum of the payload over
 * 8-byte words) and the DataOnCells fields.  Reading checks the header
 * against the handle and the checksum, scatters the fields and returns t. */
int mcfd_write_restart(mcfd_handle *h, const char *path, double t);
int mcfd_read_restart(mcfd_handle *h, const char *path, double *t);

/* limiter::Reconstruct(part, limiter) (limiter/reconstruct.hpp:21-54) on the
 * current solution with the handle's limiter (no-op when none is set).
 * *troubled (may be NULL) receives the number of reconstructed cells. */
int mcfd_limit(mcfd_handle *h, int64_t *troubled);

/* Energy-based artificial viscosity, the shock capturing of the reference's
 * viscous demos: WithViscosity<fr::Lobatto<Part, EnergyBasedViscosity<Part,
 * ConvectionDiffusion<Riemann, Direct<Isotropic>>>>> (spatial/viscosity.hpp:
 * 35-602, spatial/with_viscosity.hpp:20-72, riemann/diffusive/direct.hpp).
 * Replaces Direct::SetBetaValues(ddg_beta0, ddg_beta1),
 * EnergyBasedViscosity::SetTimeScale(time_scale) and the construction of
 * WithViscosity (demo/euler/sourceless.cpp:117-121).  From then on every
 * residual, stage and time step of the handle uses the viscosities of its
 * own input state (SetSolutionColumn runs UpdateProperties) and
 * mcfd_time_step returns min(2 cfl min_dt, dt_guess).  Needs MCFD_FR, the
 * plain FP64 form, no limiter, no cases and Hex8 cells
 * (MCFD_ERR_UNSUPPORTED otherwise). */
int mcfd_set_viscosity(mcfd_handle *h, double ddg_beta0, double ddg_beta1, double time_scale);

/* The viscosity of every cell and component, [cells][5], of the current
 * solution (GetPropertyOnCell(cell, 0), the demos' CellViscosity fields). */
int mcfd_get_viscosity(mcfd_handle *h, double *nu, int64_t n);

/* Initial limiters of the viscous demos on the current solution of a nodal
 * handle (sourceless.cpp:146-153): MCFD_INIT_AVERAGE sets every node to the
 * cell average (limiter/average.hpp:11-28); MCFD_INIT_MAJORITY sets every
 * node to the value a strict majority of the cell's nodes hold, per
 * component (limiter/majority.hpp:14-42; no-op for p < 2).  A cell with a
 * component without such a value stays unchanged and the call returns
 * MCFD_ERR_STATE after treating the others. */
enum mcfd_initial_limiter_kind { MCFD_INIT_AVERAGE = 1, MCFD_INIT_MAJORITY = 2 };
int mcfd_initial_limiter(mcfd_handle *h, int32_t kind);

/* Cells reconstructed by limiter passes since the last call (reset on read). */
int mcfd_troubled_cells(mcfd_handle *h, int64_t *count);

/* Use a caller-provided cudaStream_t (NULL = the handle's own stream). */
int mcfd_set_stream(mcfd_handle *h, void *cuda_stream);
int mcfd_synchronize(mcfd_handle *h);

/* Face-point to cell-node maps (lobatto.hpp:54-78 i_node_on_holder_ /
 * i_node_on_sharer_), [n_faces][(p+1)^2] each; sharer entries of boundary
 * faces are -1.  For indexing parity checks. */
int mcfd_face_node_maps(const mcfd_handle *h, int16_t *holder, int16_t *sharer);

/* Kernel launches issued by this handle since creation. */
int64_t mcfd_launch_count(const mcfd_handle *h);

/* Instrumentation (the reference times with MPI_Wtime in
 * demo/euler/sourceless.cpp:94-215): average device time in milliseconds of
 * one launch of each kernel of an SSP-RK3 stage, measured with CUDA events on
 * the handle's stream over `reps` launches on the current solution (which is
 * left unchanged).  out_ms[0] = dt reduction, [1] = face fluxes,
 * [2] = cell update (volume + lift + mass + stage), [3] = whole RK3 step. */
int mcfd_kernel_times(mcfd_handle *h, int32_t reps, double *out_ms);

/* Approximate (spatial/fem.hpp:147-154 -> Projection::Approximate,
 * polynomial/projection.hpp:28-42) of the MODAL scheme, split so that the
 * initial-value function runs on the caller's side:
 *   mcfd_point_count   number of volume quadrature points (all cells, cell by
 *                      cell in integrator order)
 *   mcfd_points        their global coordinates [n][3]
 *   mcfd_project       sets the solution to the projection of the values
 *                      [n][K] given at those points (coeff = sum_q f_q psi w_q)
 * Nodal schemes return MCFD_ERR_UNSUPPORTED (their Approximate is the value
 * at each node, i.e. mcfd_set_solution). */
int64_t mcfd_point_count(const mcfd_handle *h);
int mcfd_points(const mcfd_handle *h, double *xyz, int64_t n);
int mcfd_project(mcfd_handle *h, const double *values, int64_t n);

/* Batching (no reference counterpart: in the reference every case is its own
 * run of the demo/euler/sourceless.cpp:187-215 loop).
 *
 * mcfd_set_cases splits one handle's mesh into independent cases: cells
 * [case_offsets[k], case_offsets[k+1]) form case k (n_cases <= 1024, no face
 * may join two cases; a disjoint union of meshes qualifies).  From then on
 * every case takes its own time step (GetTimeStep over its own cells) and
 * keeps its own time, starting at 0: mcfd_advance steps all cases at once and
 * returns the smallest case time, mcfd_rk_step applies the given (t, dt) to
 * every case, boundary values are evaluated at each case's own time, and
 * mcfd_time_step reports the smallest case step.
 * mcfd_case_times copies the case times (and, when dt is not NULL, the last
 * steps) to the host. */
int mcfd_set_cases(mcfd_handle *h, int32_t n_cases, const int64_t *case_offsets);
int mcfd_case_times(mcfd_handle *h, double *t, double *dt, int32_t n);

/* An ensemble steps several handles (e.g. one per scheme and degree) with one
 * CUDA graph per step: the replay forks to every member's stream, runs its dt
 * reduction and RK stages, and joins, so members run concurrently.  Members
 * share one device, stay owned by the caller, and must outlive the ensemble;
 * reconfiguring a member (cases, limiter, stream) after the first advance is
 * not allowed. */
typedef struct mcfd_ensemble mcfd_ensemble;
int mcfd_ensemble_create(mcfd_handle *const *handles, int32_t n, mcfd_ensemble **out);
int mcfd_ensemble_advance(mcfd_ensemble *e, int32_t n_steps, double dt_guess, int32_t rk_order);
int mcfd_ensemble_destroy(mcfd_ensemble *e);
/* Replays go to the caller's stream from now on (the ensemble's own stream is
 * released); the caller keeps ownership of the stream. */
int mcfd_ensemble_set_stream(mcfd_ensemble *e, void *cuda_stream);
const char *mcfd_ensemble_last_error(const mcfd_ensemble *e);
/* Streamed ensemble stepping: each job loads every member's column from
 * host_in[i], runs n_steps ensemble steps and stores the columns to
 * host_out[i]; the uploads of job k+1 and the downloads of job k-1 overlap
 * job k (staging of two columns per member and direction, allocated by the
 * first begin and kept until mcfd_ensemble_destroy).  As mcfd_stream_*: the
 * host arrays stay untouched until mcfd_ensemble_stream_end, which waits and
 * reports the first member status.  Member times continue from job to job,
 * as with set-solution + mcfd_ensemble_advance. */
int mcfd_ensemble_stream_begin(mcfd_ensemble *e);
int mcfd_ensemble_stream_step(mcfd_ensemble *e, const double *const *host_in,
                              double *const *host_out, int32_t n_steps,
                              double dt_guess, int32_t rk_order);
int mcfd_ensemble_stream_end(mcfd_ensemble *e);

/* Launch-shape autotuner (no reference counterpart).  Times the candidate
 * launch shapes of this handle's kernels on its own mesh and current solution
 * (face-flux and dt-reduction block sizes 128 / 256 / 512; persistent limiter
 * grid of 4 / 8 / 16 / 32 blocks per SM), keeps the fastest and re-captures
 * the step graph on the next mcfd_advance.  With cache_path, the choice is
 * first looked up in that file (one JSON object per line, keyed by scheme,
 * degree, precision, solver, limiter and cell-count bucket) and otherwise
 * appended to it.  choice (NULL or [4]): face block, dt block, limiter blocks
 * per SM, 1 when taken from the cache.  Tune members before building an
 * ensemble from them. */
int mcfd_autotune(mcfd_handle *h, const char *cache_path, int32_t *choice);

/* ---- device probes (for verification; no handle) ----
 * mcfd_probe_flux evaluates, on GPU `device`, the flux that a face kernel
 * computes at one face point, for n points given on caller-owned device
 * memory: d_left [n][5] the holder's conservative state, d_right [n][5] the
 * sharer's state (bc_kind == MCFD_BC_NONE: an interior face, the rotated
 * solver's GetFluxUpwind, riemann/rotated/euler.hpp:153-159) or the given
 * boundary value (bc_kind = MCFD_BC_INVISCID_WALL .. MCFD_BC_SMART: the
 * boundary fluxes of rotated/euler.hpp:144-318), d_normal [n][3] unit
 * normals, d_flux [n][5] the flux through the normal (face weight 1).  The
 * same device code and template instance as the face kernels of `precision`
 * (MCFD_MIXED: the seeded square roots of the mixed form), including the
 * conservative-input fast paths and their primitive fallbacks.  *status
 * (may be NULL) receives the device status bits (2: the Exact solver hit
 * its iteration cap, also returned as MCFD_ERR_NOT_CONVERGED).  Restores the
 * caller's current device. */
int mcfd_probe_flux(int32_t device, int32_t riemann, int32_t precision,
                    int32_t bc_kind, int64_t n, const double *d_left,
                    const double *d_right, const double *d_normal,
                    double *d_flux, uint32_t *status);
/* mcfd_probe_numerics applies one operation elementwise to n device values:
 * the arithmetic that the kernels use in place of CUDA's operators on their
 * FP64-bound paths, and CUDA's own operators for comparison. */
enum mcfd_probe_op {
  MCFD_PROBE_RCP = 0,             /* double -> double: Newton reciprocal 1/x, x > 0 */
  MCFD_PROBE_RCP_SIGNED = 1,      /* double -> double: Newton reciprocal of either sign */
  MCFD_PROBE_SQRT_SEEDED = 2,     /* double -> double: FP32-seeded square root, x >= 0 */
  MCFD_PROBE_F64_TO_F32 = 3,      /* double -> float: integer-pipe rounding conversion */
  MCFD_PROBE_F32_TO_F64 = 4,      /* float -> double: integer-pipe widening */
  MCFD_PROBE_CUDA_RCP = 5,        /* double -> double: 1.0 / x */
  MCFD_PROBE_CUDA_SQRT = 6,       /* double -> double: sqrt(x) */
  MCFD_PROBE_CUDA_F64_TO_F32 = 7, /* double -> float: __double2float_rn */
  MCFD_PROBE_CUDA_F32_TO_F64 = 8, /* float -> double: (double)f */
  MCFD_PROBE_RCP1 = 9,            /* double -> double: one-step Newton reciprocal, x > 0
                                     (the mixed form's node traces) */
  /* the Exact solver's powers for gamma = 1.4, from FP32-seeded inverse roots
     refined by Newton steps (pow outside x in [2^-120, 2^120]) */
  MCFD_PROBE_ROOT7 = 10,          /* double -> double: x^((gamma-1)/(2 gamma)) = x^(1/7) */
  MCFD_PROBE_ROOT7_OVER_X = 11,   /* double -> double: x^(1/7) / x */
  MCFD_PROBE_POW_NEG_GAMMA = 12,  /* double -> double: x^(-gamma) */
  MCFD_PROBE_CUDA_POW_ROOT7 = 13, /* double -> double: pow(x, (gamma-1)/(2 gamma)) */
  MCFD_PROBE_CUDA_POW_NEG_GAMMA = 14 /* double -> double: 1 / pow(x, gamma) */
};
int mcfd_probe_numerics(int32_t device, int32_t op, int64_t n, const void *d_in,
                        void *d_out);

/* Message describing the last failure on this handle (or of mcfd_create when
 * h is NULL).  Valid until the next call on the handle. */
const char *mcfd_last_error(const mcfd_handle *h);

#ifdef __cplusplus
}
#endif
#endif /* MCFD_H_ */
