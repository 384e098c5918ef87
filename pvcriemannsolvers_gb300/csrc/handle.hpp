// Internal state of one mcfd handle: device-resident mesh tables, geometry,
// solution buffers and launch parameters.  Shared by the C-ABI layer
// (api.cpp) and the kernel launchers (dgsem.cu).
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <string>
#include <vector>

struct mcfd_mesh_desc;

namespace mcfd {

// Makes `device` current for a scope and restores the caller's device.
struct DeviceGuard {
  int prev = -1;
  explicit DeviceGuard(int device) {
    if (cudaGetDevice(&prev) != cudaSuccess) prev = -1;
    cudaSetDevice(device);
  }
  ~DeviceGuard() {
    if (prev >= 0) cudaSetDevice(prev);
  }
  DeviceGuard(const DeviceGuard &) = delete;
  DeviceGuard &operator=(const DeviceGuard &) = delete;
};

// An NVTX range for the lifetime of a scope (the C-ABI calls open one named
// after the call), so that a timeline tool shows the host phases around the
// kernels and graph replays; a function-pointer test when no tool is attached.
#if defined(__has_include)
#if __has_include(<nvtx3/nvToolsExt.h>)
#include <nvtx3/nvToolsExt.h>
#define MCFD_HAVE_NVTX 1
#endif
#endif
struct NvtxRange {
#ifdef MCFD_HAVE_NVTX
  explicit NvtxRange(const char *name) { nvtxRangePushA(name); }
  ~NvtxRange() { nvtxRangePop(); }
#else
  explicit NvtxRange(const char *) {}
#endif
  NvtxRange(const NvtxRange &) = delete;
  NvtxRange &operator=(const NvtxRange &) = delete;
};

// Device-side scalars of the time loop.  t and dt live on the device so a
// whole step (dt reduction + 3 stages) runs without a host round trip.
struct DevState {
  double t;               // current time (start of the step)
  double dt;              // current step size
  double dt_guess;        // upper bound passed by the caller
  double cfl;             // CFL number used by the dt kernels
  unsigned long long max_rate_bits;  // max over cells of max_speed / length (bits of a positive double)
  unsigned int status;    // StatusBits
  unsigned int pad;
  unsigned long long min_dt_bits;  // viscosity: min over cells of the stable step (bits of a positive double)
};

// One boundary group on the device (mirror of mcfd_bc_state).
struct BcDev {
  int kind, program, axis, pad;
  double position, speed;
  double a[5], b[5];
  double normal[3];      // OBLIQUE_SPLIT
  const double *table;   // TABLE: [group points][5] (device), or null
};

#ifdef __CUDACC__
// The given value of boundary group bc at face point (x, y, z) and time t;
// row = the point's index within its group (TABLE programs), or -1.
__device__ __forceinline__ void boundary_given(const BcDev &bc, double x, double y, double z,
                                               double t, int32_t row, double *g) {
  const double *src = bc.a;
  if (bc.program == 1) {
    const double pos[3] = {x, y, z};
    if ((pos[bc.axis] - bc.speed * t) >= bc.position) src = bc.b;
  } else if (bc.program == 2) {
    if ((bc.normal[0] * x + bc.normal[1] * y + bc.normal[2] * z - bc.speed * t) >= bc.position) src = bc.b;
  } else if (bc.program == 3 && bc.table && row >= 0) {
    src = bc.table + (int64_t)row * 5;
  }
#pragma unroll
  for (int k = 0; k < 5; ++k) g[k] = src[k];
}

// Warp maximum of non-negative, non-NaN doubles given as bit patterns, which
// order like the values as unsigned integers: shuffles and integer compares,
// no FP64 max (the FP64 unit bounds these kernels).
__device__ __forceinline__ unsigned long long warp_max_bits(unsigned long long b) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const unsigned long long other = __shfl_xor_sync(0xffffffffu, b, o);
    b = other > b ? other : b;
  }
  return b;
}

// The block's maximum of such bit patterns into *word (the handle's rate) or
// case_word[key] (the case of every thread, when the block is one case),
// with one atomic per block: every warp's atomic on one address serialised
// in L2 and bounded the time-step passes.  A block that spans cases (case
// boundaries) takes one atomic per warp, or per lane where a warp spans them
// too.  Every thread of the block calls this (it synchronises the block).
__device__ __forceinline__ void block_max_bits(unsigned long long b, int key, unsigned long long *word,
                                               unsigned long long *case_word) {
  __shared__ unsigned long long s_max[32];
  __shared__ int s_key;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (threadIdx.x == 0) s_key = key;
  __syncthreads();
  const int key0 = s_key;
  if (case_word && !__syncthreads_and(key == key0)) {
    const int wkey = __shfl_sync(0xffffffffu, key, 0);
    if (__all_sync(0xffffffffu, key == wkey)) {
      const unsigned long long m = warp_max_bits(b);
      if (lane == 0 && wkey >= 0 && m > 0) atomicMax(&case_word[wkey], m);
    } else if (key >= 0 && b > 0) {
      atomicMax(&case_word[key], b);
    }
    return;
  }
  const unsigned long long m = warp_max_bits(b);
  if (lane == 0) s_max[warp] = m;
  __syncthreads();
  if (warp == 0) {
    const unsigned long long v = warp_max_bits(lane < (int)(blockDim.x >> 5) ? s_max[lane] : 0ull);
    if (lane == 0 && v > 0) {
      if (!case_word) atomicMax(word, v);
      else if (key0 >= 0) atomicMax(&case_word[key0], v);
    }
  }
}
#endif

// Stage combinations of RungeKutta<1|2|3> (temporal/rk.hpp:16-49):
//   kStageEuler:    u + R dt                          (Euler::NextSolution)
//   kStageRk2Last:  ((u + R dt) + u0) * 0.5
//   kStageRk3Mid:   (u0 * 3 + (u + R dt)) / 4
//   kStageRk3Last:  ((u + R dt) * 2 + u0) / 3
//   kStageResidual: R                                 (GetResidualColumn)
enum Stage {
  kStageEuler = 0,
  kStageRk2Last = 1,
  kStageRk3Mid = 2,
  kStageRk3Last = 3,
  kStageResidual = 4,
};

// The same combinations expanded as cu u + c0 u0 + cd (R dt): the kernels
// fold cd into the increment's scale and take the rest as two FMAs per value
// (three FP64 operations where the nested form takes four; equal to it up to
// rounding).
template <int STAGE>
struct StageCoef {
  static constexpr double cu = STAGE == kStageRk2Last ? 0.5
                               : STAGE == kStageRk3Mid ? 0.25
                               : STAGE == kStageRk3Last ? 2.0 / 3.0 : 1.0;
  static constexpr double c0 = STAGE == kStageRk2Last ? 0.5
                               : STAGE == kStageRk3Mid ? 0.75
                               : STAGE == kStageRk3Last ? 1.0 / 3.0 : 0.0;
  static constexpr double cd = cu;
};

struct Mesh {
  int p = 0, q = 0, n = 0, qf = 0;  // degree, line points, nodes/cell, points/face
  int64_t n_cells = 0, n_faces = 0, n_points = 0, column = 0;
  int n_groups = 0;
  // device arrays
  double *cell_geo = nullptr;       // [cells][N][10]: w*J^-1 (3x3 row-major), 1/w
  float *cell_geo32 = nullptr;      // [cells][N][10]: FP32 w*J^-1, 1/w (mixed form only); with
                                    // geo32_affine [cells][10]: adj(J), 1/det(J)
  float *node_w32 = nullptr;        // [2][N] with geo32_affine: w_q, 1/w_q (DGSEM) or 1, 1 (FR)
  bool geo32_affine = false;        // every cell affine: the FP32 metric terms stored per cell
  double *cell_rate = nullptr;      // [cells] 1 / length  (length = cbrt(V)/2)
  float *cell_rate32 = nullptr;     // [cells] FP32 copy (mixed form's time step)
  int32_t *cell_flux = nullptr;     // [cells][6][QF] flux slot: >=0 subtract, <0 add (~slot), INT32_MIN none
  int2 *face_cells = nullptr;       // [faces] holder, sharer
  int32_t *face_group = nullptr;    // [faces]
  double4 *face_geo = nullptr;      // [points] unit normal, weight
  double4 *face_nh = nullptr;       // [points] (w/2) n, w/2: Rusanov handles' face kernel
  double *face_xyz = nullptr;       // [points][3]
  short2 *face_map = nullptr;       // [points] holder node, sharer node
  double *dmat = nullptr;           // [Q][Q] D[a][i] = l_i'(x_a)
  BcDev *bcs = nullptr;             // [n_groups]
  // output sampling (mcfd_vtk_sample): cell corners and types
  double *corners = nullptr;        // [cells][8][3] corner coordinates (Tet4: first 4)
  uint8_t *cell_type = nullptr;     // [cells] 0 Hex8, 1 Tet4
  std::vector<uint8_t> host_types;  // [cells] 0 hexahedron, 1 tetrahedron, 2 wedge, 3 pyramid
  std::vector<uint8_t> host_cell_type;  // [cells] enum mcfd_cell_type
  bool curved = false;              // output points come from the host maps (quadratic, wedge or pyramid cells)
  std::vector<double> host_nodes;   // [cells][27][3] all nodes (curved meshes only)
  double xq[4] = {0, 0, 0, 0};      // GLL abscissae of the nodal schemes
  // host copies for parity queries
  std::vector<int16_t> map_h, map_s;
  std::vector<BcDev> host_bcs;
  // TABLE boundary programs: per face point its row in its group's table
  // (-1 elsewhere), allocated with the first table; per group the table
  int32_t *bc_row = nullptr;          // [points] (device)
  std::vector<int32_t> host_bc_row;   // [points]
  std::vector<double *> bc_tables;    // [n_groups] device tables (owned)
  double *node_w = nullptr;         // [cells][N] global weights (initial limiters; built on first use)
  std::vector<double> host_corners;  // [cells][8][3] (as uploaded to corners)
  std::vector<double> host_shift;    // [faces][3] periodic shifts (empty: none)
  std::vector<int8_t> host_face_sides;  // [faces][2] local face on the holder / sharer side
};

// Energy-based artificial viscosity on fr::Lobatto (spatial/viscosity.hpp,
// spatial/with_viscosity.hpp, riemann/diffusive/direct.hpp), Hex8 cells.
// Per stage a properties kernel turns the stage input into one viscosity per
// cell and component; the face and cell kernels then add the viscous fluxes
// where it is not zero.
struct Visc {
  bool on = false;
  double beta0 = 2.0, beta1 = 1.0 / 12, time_scale = 1.0;
  double *nu = nullptr;     // [cells][K] viscosity of the last properties pass
  double *side = nullptr;   // [points][2 sides][6]: m = J^-T n, q (Hessian chain-rule term)
  double *pt = nullptr;     // [points][4]: beta0 / d, beta1 d, w h_holder, w h_sharer
  double *cell = nullptr;   // [cells][2]: length, length^(p + 4)
  double *d2 = nullptr;     // [Q][Q] second derivatives l_i''(x_a)
  double *wloc = nullptr;   // [N] local GLL weights of the nodes
  // work list of the damping-rate pass (cells whose jump reaches the
  // reference square): count, cells, kViscRateData doubles per entry
  unsigned *rate_count = nullptr;
  int32_t *rate_cell = nullptr;
  double *rate_data = nullptr;
  int rate_blocks = 1;  // persistent grid of the damping-rate kernel
};
constexpr int kViscRateData = 8;  // wave speed, 5 jump integrals, flags, pad

// Device tables of the WENO limiter (built when a limiter is requested).
// M = (p+1)(p+2)(p+3)/6 modal basis functions per cell.
struct Limiter {
  int kind = 0;              // mcfd_limiter
  int m = 0;                 // modal basis size
  double w0 = 0.001, eps = 1e-6;
  double *psi = nullptr;     // [cells][N][M] orthonormal basis at the cell's nodes
  double *mn = nullptr;      // [cells][N][M] w_n psi_m(x_n) (modal_to_nodal)
  float *mn32 = nullptr;     // FP32 copy of mn (mixed form)
  double *proj = nullptr;    // [cells][6][M][M] neighbour -> own basis projection
  double *beta = nullptr;    // [cells][M][M] smoothness quadratic form
  double *eval = nullptr;    // [cells][7][M] basis values at this cell's centre:
                             //   slots 0..5 neighbour bases, slot 6 own basis
  double *s00 = nullptr;     // [cells] S(0,0) of the own basis
  double *divisor = nullptr; // [cells] volume^((p+1)/6) * n_adj (jump detector)
  int32_t *adj = nullptr;    // [cells][6] neighbour cells (-1 = none), face order
  double *frame = nullptr;   // [cells][6][9] frame of the shared face at its first
                             //   point: normal, tangent, bitangent (weno::Eigen)
  double *volume = nullptr;  // [cells] cell volume (weno::Eigen face weights)
  double *modal = nullptr;   // [cells][K][M] scratch: modal coefficients
  int32_t *list = nullptr;   // [cells] troubled cells of the current pass
  unsigned *list_count = nullptr;
  // mixed form with shock_fp64: per cell the last pass's flag, per block of
  // the cell kernel (CellCfg cells) whether it holds a flagged cell or a
  // face neighbour of one (those blocks take the FP64 cell update)
  uint8_t *cell_hot = nullptr;   // [cells]
  uint8_t *cell_hot2 = nullptr;  // [cells] after the first dilation (two layers)
  uint8_t *block_hot = nullptr;  // [cell-kernel blocks]
  int64_t n_blocks = 0;
  unsigned long long *troubled = nullptr;  // counter of reconstructed cells
};

// Modal DG tables (dg::General over Projection, Hex8 and Tet4 cells).
// Cell c's basis is psi = S_c T(x - centre_c) with T the M Taylor monomials;
// kernels work with the Taylor coefficients a = S^T u of the stage input and
// accumulate the residual against T, then apply S once per cell.
struct Modal {
  int m = 0;                        // basis size M
  int64_t n_vol = 0, n_fpts = 0;    // volume / face quadrature points
  double4 *center = nullptr;        // [cells] centre, 1 / length
  double *s = nullptr;              // [cells][M (M + 1) / 2] packed rows of S
  int32_t *vol_off = nullptr;       // [cells + 1]
  double4 *vol = nullptr;           // [volume points] x - centre, global weight
  int32_t *cell_faces = nullptr;    // [cells][6] 2 face + (1 on the sharer side), -1 none
  int32_t *face_off = nullptr;      // [faces + 1]
  int32_t *point_face = nullptr;    // [face points] face id
  double4 *fpt = nullptr;           // [face points] x, global weight
  double4 *fnrm = nullptr;          // [face points] unit normal (holder -> sharer)
  double4 *fshift = nullptr;        // [faces] periodic shift: sharer sees x - shift
  double *taylor = nullptr;         // [cells][M][K] Taylor coefficients of a stage input
  double *values = nullptr;         // [volume points][K] scratch of mcfd_project
  // mixed form: FP32 copies for the contractions
  float *s32 = nullptr;             // [cells][M (M + 1) / 2]
  float4 *vol32 = nullptr;          // [volume points] x - centre, global weight
  float4 *foff32 = nullptr;         // [face points][2] x - centre (holder), x - shift - centre (sharer)
  float *taylor32 = nullptr;        // [cells][M][K]
  std::vector<double> host_points;  // [volume points][3] global coordinates
  // kept by build_modal_mesh for build_modal_limiter when a limiter is set,
  // then released: per point weights, per cell centre, full S and volume,
  // per cell point offsets, per face the frame at its first point
  bool keep_host = false;
  std::vector<double> host_weights, host_center, host_s, host_volume, host_frame0;
  std::vector<int32_t> host_vol_off;
};

// Independent cases inside one handle (an ensemble member: disjoint meshes
// concatenated).  Cells [offsets[k], offsets[k+1]) form case k; no face
// joins two cases.  Every case has its own time step (the minimum over its
// cells) and its own time.
struct Cases {
  int n = 0;
  int32_t *cell_case = nullptr;        // [cells] case id
  double *t = nullptr;                 // [n] time of each case
  double *dt = nullptr;                // [n] current step of each case
  unsigned long long *rate = nullptr;  // [n] max of max_speed / length (bits)
  std::vector<int64_t> offsets;        // [n + 1] host copy
};

// Case fields of the kernel argument blocks (all null without cases).
struct CaseView {
  const int32_t *cell_case;
  const double *t;
  const double *dt;
};

struct Buffers {
  double *u = nullptr;     // current solution
  double *u1 = nullptr;    // stage buffers
  double *u2 = nullptr;
  double *res = nullptr;   // residual output
  double *flux = nullptr;  // [points][5] face flux scratch
  // [cells][N][3] 1/rho, p, sound speed of one stage state (Rusanov, nodal
  // schemes without a limiter): written by the cell kernel that produces the
  // state, read by the next face kernel instead of recomputing per face point
  double *trace = nullptr;
  DevState *state = nullptr;
  // FP64 nodal forms: the FP32 upper bound of each dt block's largest rate
  // (one word per 128 nodes), from the first pass of the two-pass dt
  unsigned *dt_hi = nullptr;
};

struct Options {
  int riemann = 4;
  int precision = 0;
  int scheme = 0;     // 0 dg::Lobatto (DGSEM), 1 fr::Lobatto (Huynh g2), 2 dg::General (modal)
  double cfl = 0;
  double fr_g1 = 0;   // g_R'(1) of the FR correction function
  int tensor_contraction = 0;  // mixed DGSEM p = 3: differentiation on the tensor cores
  int shock_fp64 = 0;  // mixed + limiter: flagged cells and 1 or 2 neighbour layers in FP64
};

}  // namespace mcfd

namespace mcfd {
// Streamed stepping (mcfd_stream_*): double-buffered device staging of the
// host columns and one copy stream per direction, so that the uploads and
// downloads of neighbouring jobs overlap the current job's compute.  Job k
// uses staging slot b = k & 1; its graph steps in[b] into out[b] directly
// (first stage reads in[b], last stage writes out[b]), so no device copy of
// the column is made.
struct Streamer {
  bool on = false;
  double *in[2] = {nullptr, nullptr}, *out[2] = {nullptr, nullptr};
  cudaGraphExec_t graph[2] = {nullptr, nullptr};
  int graph_order[2] = {0, 0}, graph_steps[2] = {0, 0}, graph_kernels[2] = {0, 0};
  cudaStream_t copy_in = nullptr, copy_out = nullptr;
  cudaEvent_t in_ready[2] = {nullptr, nullptr}, in_free[2] = {nullptr, nullptr};
  cudaEvent_t out_ready[2] = {nullptr, nullptr}, out_free[2] = {nullptr, nullptr};
  int64_t k = 0;
};

// Launch shapes chosen by mcfd_autotune (defaults until it runs).
struct Tune {
  int face_block = 256;            // threads per block of the face kernels
  int dt_block = 256;              // threads per block of the dt reductions
  int limiter_blocks_per_sm = 16;  // persistent reconstruction grid width
  bool tuned = false;
};
}  // namespace mcfd

struct mcfd_handle {
  int device = 0;
  mcfd::Tune tune;
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  mcfd::Options opt;
  mcfd::Mesh mesh;
  mcfd::Buffers buf;
  mcfd::Limiter lim;
  mcfd::Modal modal;
  mcfd::Cases cases;
  mcfd::Visc visc;
  double t_host = 0;
  int64_t launches = 0;
  bool use_trace = false;            // see Buffers::trace
  const double *trace_for = nullptr; // the buffer whose trace buf.trace holds
  std::string err;
  // CUDA graph of one SSP-RK3 step (dt + 3 stages), built on first use
  cudaGraphExec_t step_graph = nullptr;
  int step_graph_order = 0;
  int step_graph_kernels = 0;
  mcfd::Streamer streamer;
};

namespace mcfd {

// Drop every captured step graph (launch shapes, cases or pointers changed).
inline void drop_graphs(mcfd_handle *h) {
  if (h->step_graph) { cudaGraphExecDestroy(h->step_graph); h->step_graph = nullptr; }
  for (int b = 0; b < 2; ++b)
    if (h->streamer.graph[b]) { cudaGraphExecDestroy(h->streamer.graph[b]); h->streamer.graph[b] = nullptr; }
}

// Kernel launchers (dgsem.cu).  Each returns the number of kernels launched.
int launch_set_state(mcfd_handle *h, double t, double dt, double dt_guess,
                     double cfl, int reset_rate);
// dt guess and CFL of the next steps with the device time left as it is.
int launch_set_bounds(mcfd_handle *h, double dt_guess, double cfl);
// props_fresh: the viscosity properties of u were just computed by launch_dt
int launch_face_flux(mcfd_handle *h, const double *u, double stage_c, bool props_fresh = false);
int launch_cell_update(mcfd_handle *h, int stage, const double *u_in,
                       const double *u0, double *u_out, int advance_time);
int launch_dt(mcfd_handle *h, const double *u);
// Trace of a state buffer (Buffers::trace), when the handle uses one.
int launch_trace(mcfd_handle *h, const double *u);
// A host-side or limiter write to `u` makes its trace stale.
inline void invalidate_trace(mcfd_handle *h, const double *u) {
  if (h->trace_for == u) h->trace_for = nullptr;
}
// dt finalisation after a max-rate reduction (handle word or per case).
int launch_dt_finalize(mcfd_handle *h);
// Output (output.cu): column <-> DataOnCells fields ([F][cells], F values
// per cell) and the VTK sample points of every cell (Hex27 / Tet10 locals),
// written at xyz / values + off[cell] (3 and K doubles per point).
int launch_fields_transpose(mcfd_handle *h, const double *src, double *dst, int to_fields);
int launch_vtk_sample(mcfd_handle *h, const double *u, const int64_t *off, double *xyz,
                      double *values);
int launch_modal_vtk_sample(mcfd_handle *h, const double *u, const int64_t *off, double *xyz,
                            double *values);
// One RK step's stages from u_in to u_out (both default to buf.u);
// after_dt: launch_dt(u_in) ran right before (its viscosity properties are
// the first stage's).
int launch_rk_stage_sequence(mcfd_handle *h, int order, const double *u_in = nullptr,
                             double *u_out = nullptr, bool after_dt = false);
// WENO limiter pass on a solution buffer, in place (weno.cu).
int launch_limiter(mcfd_handle *h, double *u);

// Cases (dgsem.cu): per-case time advance after the last stage, and the
// per-case stage time / step set by mcfd_rk_step.
int launch_advance_cases(mcfd_handle *h);
int launch_set_cases(mcfd_handle *h, double t, double dt);
inline CaseView case_view(const mcfd_handle *h) {
  if (h->cases.n == 0) return CaseView{nullptr, nullptr, nullptr};
  return CaseView{h->cases.cell_case, h->cases.t, h->cases.dt};
}

// Modal DG (modal.cu): the same stage interface as the nodal launchers.
constexpr int kSchemeModal = 2;
int launch_modal_face_flux(mcfd_handle *h, const double *u, double stage_c);
int launch_modal_cell_update(mcfd_handle *h, int stage, const double *u_in,
                             const double *u0, double *u_out, int advance_time);
int launch_modal_dt(mcfd_handle *h, const double *u);
// Projection::Approximate from values [volume points][K] in modal.values.
int launch_modal_project(mcfd_handle *h, double *u);
// Host set-up of the modal tables (modal_setup.cpp); returns an mcfd status.
int build_modal_mesh(mcfd_handle *h, const ::mcfd_mesh_desc *d, int degree);
// The WENO limiter tables of the modal scheme from the cells' own bases and
// volume quadratures (after build_modal_mesh with modal.keep_host set).
int build_modal_limiter(mcfd_handle *h, const ::mcfd_mesh_desc *d, int kind, double w0, double eps);

// Artificial viscosity (viscosity.cu / visc_setup.cpp).  The properties
// pass writes Visc::nu and Visc::trace from the state u; with dt_mode it also
// folds every cell's stable step into DevState::min_dt_bits, and
// launch_visc_dt turns that into the step (with_viscosity.hpp:67-71).
int build_viscosity(mcfd_handle *h, double beta0, double beta1, double time_scale);
void release_viscosity(mcfd_handle *h);
int launch_visc_properties(mcfd_handle *h, const double *u, int dt_mode);
// resident blocks per SM of the damping-rate kernel for Q nodes per direction
// (its persistent grid; queried once at set-up, outside any stream capture)
int visc_rate_blocks_per_sm(int q);
int launch_visc_face_flux(mcfd_handle *h, const double *u);
int launch_visc_dt_finalize(mcfd_handle *h);
// Initial limiters of the viscous demos (limiter/average.hpp,
// limiter/majority.hpp), in place; majority counts the cells without one.
int launch_initial_limiter(mcfd_handle *h, int kind, double *u, unsigned long long *missing);

// Residual whose face-flux scratch is a fixed file-scope device array
// (mcfd_residual_device_noalloc).  Capacity in doubles: 2 Mi = 16 MiB, i.e.
// at most 419,430 face points (5 doubles each).
constexpr int64_t kStaticFluxCapacity = 2 * 1024 * 1024;
int static_flux_scratch(int device, double **ptr, std::string *err);
int launch_residual_static_scratch(mcfd_handle *h, const double *d_u,
                                   double *d_r, double *scratch);

}  // namespace mcfd
