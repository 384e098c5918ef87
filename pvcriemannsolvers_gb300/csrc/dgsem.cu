// DGSEM (dg::Lobatto, kLocal = false) residual and SSP-RK stages on sm_103a,
// plain FP64 form.
//
// Per RK stage two kernels run over device-resident data:
//   face_flux_kernel   one thread per face point: gathers the holder and
//                      sharer node states, evaluates the rotated Riemann (or
//                      boundary) flux in the global frame, scales it by the
//                      face weight and writes it to a face-point flux buffer.
//                      (spatial/dg/lobatto.hpp:171-302)
//   cell_update_kernel one thread per cell node: contravariant volume flux
//                      F * (w J^-1) to shared memory, sum-factorised GLL
//                      differentiation (equal to the reference's dense
//                      F * J^-1 grad(phi) product, lobatto.hpp:161-170),
//                      gather of the <= 3 face fluxes this node lifts
//                      (atomic-free, deterministic), lumped mass divide
//                      (lobatto.hpp:143-158) and the RK stage combination
//                      (temporal/rk.hpp:16-49), written in one pass.
// The time step (spatial/fem.hpp:417-435) is a max-reduction of
// max_speed / length over all nodes plus a one-thread finalisation; dt and t
// stay in device memory.
#include <cuda_runtime.h>

#include <climits>
#include <cstdint>
#include <mutex>
#include <string>

#include "euler.cuh"
#include "handle.hpp"

namespace mcfd {
namespace {

template <int Q>
struct CellCfg {
  static constexpr int kN = Q * Q * Q;
  static constexpr int kCells = (Q == 4) ? 4 : (Q == 3 ? 9 : 32);
  static constexpr int kThreads = kCells * kN;
};

struct FaceArgs {
  const double *u;
  const int2 *face_cells;
  const int32_t *face_group;
  const double4 *face_geo;
  const double *face_xyz;
  const short2 *face_map;
  const BcDev *bcs;
  double *flux;
  DevState *state;
  double stage_c;
  int64_t n_points;
  int n_groups;
  int fr;  // flux reconstruction: mark faces without a boundary condition
  CaseView cs;
  const double *trace;  // node traces of u (Rusanov), or null
  int f32_out;          // mixed form: the flux buffer holds FP32 values
  int visc;             // artificial viscosity: no-slip walls take the wall flux
  const int32_t *bc_row;  // [points] row in the group's boundary table, or null
  const double4 *face_nh; // [points] (w/2) n, w/2 (Rusanov handles), or null
};

// FR: a boundary face point without a registered boundary gets no correction
// (the reference skips such faces); the face kernel marks its flux with this
// exact NaN bit pattern (kNoFluxBits32 in an FP32 flux buffer: the FP32
// conversion canonicalises every other NaN) and the FR lift skips exactly
// that pattern, so a NaN from a degenerate state still reaches the residual.
constexpr unsigned long long kNoFluxBits = 0x7ff8dead0000beefull;
constexpr unsigned kNoFluxBits32 = 0x7fbeef01u;

// Face-point flux store: FP64, or FP32 for the mixed form's FP32 lift (one
// conversion per face point instead of one per lifting cell).
__device__ __forceinline__ void store_flux(double *flux, int f32_out, int64_t gid,
                                           const double *v) {
  if (f32_out) {
    float *d = reinterpret_cast<float *>(flux) + gid * kK;
#pragma unroll
    for (int k = 0; k < kK; ++k) d[k] = f64_to_f32(v[k]);
    if (bits64(v[0]) == kNoFluxBits) d[0] = __uint_as_float(kNoFluxBits32);
  } else {
    double *d = flux + gid * kK;
#pragma unroll
    for (int k = 0; k < kK; ++k) d[k] = v[k];
  }
}


struct CellArgs {
  const double *u_in;
  const double *u0;
  double *u_out;
  const double *cell_geo;
  const int32_t *cell_flux;
  const double *flux;
  const double *dmat;
  DevState *state;
  int64_t n_cells;
  int advance_time;
  int fr;     // 0: dg::Lobatto (weak form), 1: fr::Lobatto (Huynh g2)
  double g1;  // FR: g_R'(1) of the Huynh g2 correction
  CaseView cs;
  double *trace;  // write the node traces of u_out here (surface nodes), or null
  const double *nu;  // artificial viscosity [cells][K] (VISC variant), else null
  int trace_roe;     // the traces' third entry is sqrt(rho) (Roe), else the sound speed
  // FP64 shock cells (mixed form): the blocks flagged in block_hot take the
  // FP64 kernel, the others the mixed one; hot_mode 1 skips flagged blocks,
  // 2 skips the others.  flux64: the face fluxes are stored in FP64.
  const uint8_t *block_hot;
  int hot_mode;
  int flux64;
};

// Whether this block of a cell kernel sits out under the FP64 shock-cell split.
__device__ __forceinline__ bool skip_block(const CellArgs &a) {
  if (!a.block_hot) return false;
  const bool hot = a.block_hot[blockIdx.x] != 0;
  return a.hot_mode == 1 ? hot : !hot;
}

// Step of the case that owns cell c (the handle's step without cases).
__device__ __forceinline__ double cell_dt(const CaseView &cs, const DevState *state, int64_t c) {
  return cs.dt ? cs.dt[cs.cell_case[c]] : state->dt;
}

// Stage time t + stage_c dt of the case that owns cell c.
__device__ __forceinline__ double stage_time(const CaseView &cs, const DevState *state,
                                             int64_t c, double stage_c) {
  if (cs.t) {
    const int k = cs.cell_case[c];
    return cs.t[k] + stage_c * cs.dt[k];
  }
  return state->t + stage_c * state->dt;
}

// FR: axis and orientation of each local hex face (fr/lobatto.hpp:81-152)
// sides 0..5 -> axes 2, 1, 0, 1, 0, 2 (one nibble per side, side 0 lowest)
__device__ __forceinline__ int fr_dir(int side) { return (0x201012 >> (4 * side)) & 0xf; }
__device__ __forceinline__ double fr_sign(int side) {
  return ((0x2c >> side) & 1) ? 1.0 : -1.0;  // + for faces 2, 3, 5
}


// FAST_SQRT (the mixed form): the Rusanov wave speed's square root from an
// FP32 seed and one FP64 Newton step (sqrt_seeded, relative error ~1e-13).
template <int Q, int R, bool FAST_SQRT>
__global__ void __launch_bounds__(512) face_flux_kernel(FaceArgs a) {
  constexpr int QF = Q * Q, KN = kK * Q * Q * Q;
  int64_t gid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (gid >= a.n_points) return;
  int64_t f = gid / QF;
  int2 cells = a.face_cells[f];
  short2 map = a.face_map[gid];
  const double *uh = a.u + (int64_t)cells.x * KN + map.x * kK;
  double ch[kK];
#pragma unroll
  for (int k = 0; k < kK; ++k) ch[k] = uh[k];
  double out[kK];
  bool not_converged = false, no_flux = false;
  if (cells.y >= 0) {
    const double *us = a.u + (int64_t)cells.y * KN + map.y * kK;
    double cs[kK];
#pragma unroll
    for (int k = 0; k < kK; ++k) cs[k] = us[k];
    // Rusanov with traces and precomputed half-weighted normals: neither the
    // unit normal nor the weight is loaded
    if constexpr (R == kRusanov) {
      if (a.trace && a.face_nh) {
        const double *th = a.trace + ((int64_t)cells.x * (Q * Q * Q) + map.x) * 3;
        const double *ts = a.trace + ((int64_t)cells.y * (Q * Q * Q) + map.y) * 3;
        const double trh[3] = {th[0], th[1], th[2]}, trs[3] = {ts[0], ts[1], ts[2]};
        const double4 h4 = a.face_nh[gid];
        const double nh[3] = {h4.x, h4.y, h4.z};
        if (rusanov_traced_nh(ch, trh, cs, trs, nh, h4.w, out)) {
          store_flux(a.flux, a.f32_out, gid, out);
          return;
        }
      }
    }
    const double4 g = a.face_geo[gid];
    const double n[3] = {g.x, g.y, g.z};
    if constexpr (R == kRusanov || R == kRoe || R == kHllc) {
      if (a.trace) {
        // both sides' node traces: 1/rho, p and the sound speed (Roe: sqrt(rho))
        const double *th = a.trace + ((int64_t)cells.x * (Q * Q * Q) + map.x) * 3;
        const double *ts = a.trace + ((int64_t)cells.y * (Q * Q * Q) + map.y) * 3;
        const double trh[3] = {th[0], th[1], th[2]}, trs[3] = {ts[0], ts[1], ts[2]};
        bool done = true;
        if constexpr (R == kRusanov) {
          flux_rusanov_traced_weighted(ch, trh, cs, trs, n, g.w, out);
        } else if constexpr (R == kRoe) {
          done = flux_roe_traced_weighted<FAST_SQRT>(ch, trh, cs, trs, n, g.w, out);
        } else {
          done = flux_hllc_traced_weighted<FAST_SQRT>(ch, trh, cs, trs, n, g.w, out);
        }
        if (done) {
          store_flux(a.flux, a.f32_out, gid, out);
          return;
        }
      }
    }
    // already multiplied by the face weight
    interior_flux_weighted<R, FAST_SQRT>(ch, cs, n, g.w, out, &not_converged);
    if (not_converged) atomicOr(&a.state->status, (unsigned)kStatusNotConverged);
    store_flux(a.flux, a.f32_out, gid, out);
    return;
  }
  const double4 g = a.face_geo[gid];
  const double n[3] = {g.x, g.y, g.z};
  {
    Prim l = cons_to_prim(ch[0], ch[1], ch[2], ch[3], ch[4]);
    int grp = a.face_group[f];
    if (grp >= 0 && grp < a.n_groups && a.bcs[grp].kind != kBcNone &&
        (a.bcs[grp].kind != kBcNoSlipWall || a.visc)) {
      const BcDev &bc = a.bcs[grp];
      double t = stage_time(a.cs, a.state, cells.x, a.stage_c);
      double given[kK];
      const double *xp = a.face_xyz + gid * 3;
      boundary_given(bc, xp[0], xp[1], xp[2], t, a.bc_row ? a.bc_row[gid] : -1, given);
      // a no-slip wall's convective part is the inviscid wall flux
      flux_boundary<R>(bc.kind == kBcNoSlipWall ? (int)kBcInviscidWall : bc.kind, l, given, n, out,
                       &not_converged);
    } else {
#pragma unroll
      for (int k = 0; k < kK; ++k) out[k] = 0;
      no_flux = a.fr != 0;
    }
  }
  if (not_converged) atomicOr(&a.state->status, (unsigned)kStatusNotConverged);
#pragma unroll
  for (int k = 0; k < kK; ++k) out[k] *= g.w;
  if (no_flux) out[0] = __longlong_as_double((long long)kNoFluxBits);
  store_flux(a.flux, a.f32_out, gid, out);
}

// VISC: fr::Lobatto with the energy-based artificial viscosity: the volume
// flux carries -nu_k grad(u_k) (spatial/fem.hpp:393-403), so every node also
// needs its gradient, from the cell's states staged in shared memory.
template <int Q, int STAGE, bool VISC = false>
__global__ void __launch_bounds__(CellCfg<Q>::kThreads)
cell_update_kernel(CellArgs a) {
  constexpr int N = Q * Q * Q, QF = Q * Q, KN = kK * N;
  constexpr int CPB = CellCfg<Q>::kCells;
  if (skip_block(a)) return;
  __shared__ double s_ft[CPB][15][N];
  __shared__ double s_d[Q * Q];
  __shared__ double s_u[VISC ? CPB : 1][VISC ? KN : 1];
  const int tid = threadIdx.x;
  if (tid < Q * Q) s_d[tid] = a.dmat[tid];
  const int lc = tid / N, q = tid - lc * N;
  const int64_t c = (int64_t)blockIdx.x * CPB + lc;
  const bool active = c < a.n_cells;
  double uq[kK];
  if (active) {
    const double *up = a.u_in + c * KN + q * kK;
#pragma unroll
    for (int k = 0; k < kK; ++k) uq[k] = up[k];
    if constexpr (VISC) {
#pragma unroll
      for (int k = 0; k < kK; ++k) s_u[lc][q * kK + k] = uq[k];
    }
  }
  if constexpr (VISC) __syncthreads();
  if (active) {
    const double *geo = a.cell_geo + (c * N + q) * 10;
    double A[9];
#pragma unroll
    for (int e = 0; e < 9; ++e) A[e] = geo[e];
    Prim w = cons_to_prim(uq[0], uq[1], uq[2], uq[3], uq[4]);
    // Contravariant flux Ft[:, e] = sum_d F[:, d] A[d][e], F = GetFluxMatrix
    // (types.hpp:322-333).  With V_e = sum_d u_d A[d][e] (u = primitive
    // velocity) and m the conservative momentum:
    //   Ft[0][e] = m . A[:, e], Ft[1+x][e] = m_x V_e + p A[x][e],
    //   Ft[4][e] = (E + p) V_e.
    // For a converted state (rho > 0) the mass row equals rho V_e; clamped
    // (all-zero primitives) and rho == 0 (unconverted) states take the
    // general form (a branch, not a select: the common path issues one
    // multiplication per direction).
    double ft[15], vel[3];
#pragma unroll
    for (int e = 0; e < 3; ++e) vel[e] = w.u * A[0 * 3 + e] + w.v * A[1 * 3 + e] + w.w * A[2 * 3 + e];
    if (ne_zero(w.rho)) {
#pragma unroll
      for (int e = 0; e < 3; ++e) ft[0 * 3 + e] = w.rho * vel[e];
    } else {
#pragma unroll
      for (int e = 0; e < 3; ++e)
        ft[0 * 3 + e] = uq[1] * A[0 * 3 + e] + uq[2] * A[1 * 3 + e] + uq[3] * A[2 * 3 + e];
    }
#pragma unroll
    for (int e = 0; e < 3; ++e) {
      const double ve = vel[e];
      ft[1 * 3 + e] = uq[1] * ve + w.p * A[0 * 3 + e];
      ft[2 * 3 + e] = uq[2] * ve + w.p * A[1 * 3 + e];
      ft[3 * 3 + e] = uq[3] * ve + w.p * A[2 * 3 + e];
      ft[4 * 3 + e] = (uq[4] + w.p) * ve;
    }
    const double *nu = VISC ? a.nu + c * kK : nullptr;
    if (VISC && (nu[0] != 0 || nu[1] != 0 || nu[2] != 0 || nu[3] != 0 || nu[4] != 0)) {
      // -nu_k grad(u_k), grad = det(J)^-1 adj(J) g_local, in contravariant form
      const int i = q / QF, j = (q / Q) % Q, l = q % Q;
      const double inv_det = geo[9];
#pragma unroll
      for (int r = 0; r < kK; ++r) {
        double g0 = 0, g1 = 0, g2 = 0;
#pragma unroll
        for (int m = 0; m < Q; ++m) {
          g0 += s_d[i * Q + m] * s_u[lc][((m * Q + j) * Q + l) * kK + r];
          g1 += s_d[j * Q + m] * s_u[lc][((i * Q + m) * Q + l) * kK + r];
          g2 += s_d[l * Q + m] * s_u[lc][((i * Q + j) * Q + m) * kK + r];
        }
        double gu[3];
#pragma unroll
        for (int d = 0; d < 3; ++d)
          gu[d] = inv_det * (A[d * 3 + 0] * g0 + A[d * 3 + 1] * g1 + A[d * 3 + 2] * g2);
        const double nr = nu[r];
#pragma unroll
        for (int e = 0; e < 3; ++e)
          ft[r * 3 + e] -= nr * (gu[0] * A[0 * 3 + e] + gu[1] * A[1 * 3 + e] + gu[2] * A[2 * 3 + e]);
      }
    }
#pragma unroll
    for (int r = 0; r < 15; ++r) s_ft[lc][r][q] = ft[r];
  }
  __syncthreads();
  if (!active) return;
  const int i = q / QF, j = (q / Q) % Q, k = q % Q;
  double res[kK];
  if (!a.fr) {
    // weak form: sum_q Ft_q . grad(phi_n)(x_q)
#pragma unroll
    for (int r = 0; r < kK; ++r) {
      double s = 0;
#pragma unroll
      for (int m = 0; m < Q; ++m) {
        s += s_ft[lc][r * 3 + 0][(m * Q + j) * Q + k] * s_d[m * Q + i];
        s += s_ft[lc][r * 3 + 1][(i * Q + m) * Q + k] * s_d[m * Q + j];
        s += s_ft[lc][r * 3 + 2][(i * Q + j) * Q + m] * s_d[m * Q + k];
      }
      res[r] = s;
    }
  } else {
    // FR: minus the divergence of the interpolated contravariant flux at the
    // node (fr/general.hpp:271-288)
#pragma unroll
    for (int r = 0; r < kK; ++r) {
      double s = 0;
#pragma unroll
      for (int m = 0; m < Q; ++m) {
        s -= s_ft[lc][r * 3 + 0][(m * Q + j) * Q + k] * s_d[i * Q + m];
        s -= s_ft[lc][r * 3 + 1][(i * Q + m) * Q + k] * s_d[j * Q + m];
        s -= s_ft[lc][r * 3 + 2][(i * Q + j) * Q + m] * s_d[k * Q + m];
      }
      res[r] = s;
    }
  }
  // Surface terms.  DG: holder -= flux, sharer += flux (lobatto.hpp:184-189).
  // FR: -= g'(1) (F_out |n| - sigma Ft[:, dir]) at the node
  // (fr/lobatto.hpp:232-251, fr/general.hpp:296-315).
  const int32_t *cf = a.cell_flux + c * 6 * QF;
  auto lift = [&](int side, int t) {
    int32_t v = cf[side * QF + t];
    if (v == INT32_MIN) return;
    const double *fl = a.flux + (int64_t)(v >= 0 ? v : ~v) * kK;
    if (a.fr) {
      if (bits64(fl[0]) == kNoFluxBits) return;  // no boundary
      const int dir = fr_dir(side);
      const double sigma = fr_sign(side), out_sign = v >= 0 ? 1.0 : -1.0;
#pragma unroll
      for (int r = 0; r < kK; ++r)
        res[r] -= a.g1 * (out_sign * fl[r] - sigma * s_ft[lc][r * 3 + dir][q]);
      return;
    }
    // -fl or +fl as one FMA with a +-1 factor (exact, and no divergence
    // between holder and sharer lanes)
    const double sign = v >= 0 ? -1.0 : 1.0;
#pragma unroll
    for (int r = 0; r < kK; ++r) res[r] = fma(sign, fl[r], res[r]);
  };
  // A node touches at most one of the two faces normal to each axis, so the
  // six faces are visited as three axes (sides 0/5, 1/3, 4/2: the order of
  // the per-face form), and a warp issues three flux additions, not six.
  if (k == 0 || k == Q - 1) lift(k == 0 ? 0 : 5, i * Q + j);
  if (j == 0 || j == Q - 1) lift(j == 0 ? 1 : 3, i * Q + k);
  if (i == 0 || i == Q - 1) lift(i == 0 ? 4 : 2, j * Q + k);
  const double inv_w = a.cell_geo[(c * N + q) * 10 + 9];
  double *out = a.u_out + c * KN + q * kK;
  bool bad = false;
  if (STAGE == kStageResidual) {
#pragma unroll
    for (int r = 0; r < kK; ++r) {
      double v = res[r] * inv_w;
      bad |= !finite64(v);
      out[r] = v;
    }
  } else {
    using SC = StageCoef<STAGE>;
    const double scale = (SC::cd * cell_dt(a.cs, a.state, c)) * inv_w;
    double nv[kK];
#pragma unroll
    for (int r = 0; r < kK; ++r) {
      double v;
      if (STAGE == kStageEuler) {
        v = fma(res[r], scale, uq[r]);
      } else {
        v = fma(SC::c0, a.u0[c * KN + q * kK + r], fma(SC::cu, uq[r], res[r] * scale));
      }
      bad |= !finite64(v);
      out[r] = v;
      nv[r] = v;
    }
    const bool surface = i == 0 || i == Q - 1 || j == 0 || j == Q - 1 || k == 0 || k == Q - 1;
    if (a.trace && surface) {
      double tr[3];
      node_trace<false>(nv, tr, a.trace_roe != 0);
      double *dst = a.trace + (c * N + q) * 3;
      dst[0] = tr[0]; dst[1] = tr[1]; dst[2] = tr[2];
    }
  }
  if (bad) atomicOr(&a.state->status, (unsigned)kStatusNonFinite);
  if (a.advance_time && !a.cs.dt && blockIdx.x == 0 && tid == 0) a.state->t += a.state->dt;
}

// Mixed-precision form of cell_update_kernel.  In FP32: the volume flux and
// its contravariant transform (FP32 copy of w J^-1), the sum-factorised GLL
// differentiation, the lift of the (FP64-computed) face fluxes and the
// mass-scaled increment dt * R / w.  In FP64: the sign checks of density and
// energy (exact, on the bit patterns), the stage accumulation u + dt R and the
// RK combinations, and the node traces of the new state.  Conversions
// between the two formats run on the integer pipes, so a node issues 29-34
// FP64 instructions (two FMAs per value for the stage combination, about 17
// for its trace) instead of about 150 in the FP64 kernel.
// ---- tensor-core differentiation (TC variant of the mixed cell kernel, Q = 4)
// The DGSEM derivative along axis d applies the transposed 1D matrix D^T
// (4 x 4, shared by every cell) to the 4-point lines of each contravariant
// flux component: R_d[(p, i), n] = sum_m D[m][i] F_d[p][m][n], p one of the
// block's 20 (cell, component) pairs and n the 16 positions of the line
// across the other two axes.  Four pairs share one m16n8k8 product: A =
// diag(D^T, D^T, D^T, D^T) (16 x 16, two k-steps), B the four pairs' lines
// (16 x 8 per n-tile).  Operands are split as x = tf32(x) + tf32(x - tf32(x))
// and each product takes three TF32 MMAs (hi hi, hi lo, lo hi) with FP32
// accumulation, which keeps the FP32 SIMT path's accuracy.
__device__ __forceinline__ unsigned tf32_of(float x) {
  unsigned r;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
  return r;
}

__device__ __forceinline__ void split_tf32(float x, unsigned *hi, unsigned *lo) {
  *hi = tf32_of(x);
  *lo = tf32_of(x - __uint_as_float(*hi));
}

__device__ __forceinline__ void mma_tf32(float *c, const unsigned *a, unsigned b0, unsigned b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k8.row.col.f32.tf32.tf32.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};"
      : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

// s_ft [4 cells][15][64] -> s_res [4 cells][5][64] = sum over the three axes
// of the line derivatives (the weak-form volume term before the lift), for
// the block's 4 cells; every thread of the 256-thread block takes part.
__device__ __forceinline__ void tc_differentiate(const float (*s_ft)[15][64], const float *s_d,
                                                 float (*s_res)[kK][64]) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int gid = lane >> 2, tig = lane & 3;
  // A fragments of diag(D^T, ...) for both k-steps: element (row r, col kk)
  // of k-step s is D[m][i] when r / 4 == (8 s + kk) / 4, with i = r % 4,
  // m = kk % 4 (a0: (gid, tig), a1: (gid + 8, tig), a2: (gid, tig + 4),
  // a3: (gid + 8, tig + 4))
  unsigned ahi[2][4], alo[2][4];
#pragma unroll
  for (int st = 0; st < 2; ++st) {
#pragma unroll
    for (int e = 0; e < 4; ++e) {
      const int r = gid + ((e & 1) ? 8 : 0), kk = tig + ((e & 2) ? 4 : 0);
      const int col = st * 8 + kk;
      const float v = (r / 4 == col / 4) ? s_d[(col % 4) * 4 + (r % 4)] : 0.f;
      split_tf32(v, &ahi[st][e], &alo[st][e]);
    }
  }
  // one direction at a time: each output element is written by one lane
#pragma unroll 1
  for (int d = 0; d < 3; ++d) {
#pragma unroll 1
    for (int item = warp; item < 10; item += 8) {
      const int g = item >> 1, t = item & 1;  // pair group (4 pairs), n-tile
      float c[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
      for (int st = 0; st < 2; ++st) {
        // B (8 x 8): row kk = (pair pb, m), col n; b0: (tig, gid), b1: (tig + 4, gid)
        unsigned bhi[2], blo[2];
#pragma unroll
        for (int e = 0; e < 2; ++e) {
          const int kk = tig + 4 * e;
          const int pb = st * 2 + kk / 4, m = kk % 4;
          const int pr = g * 4 + pb, cell = pr / kK, comp = pr % kK;
          const int col = t * 8 + gid, hi = col / 4, lo = col % 4;
          int node;
          if (d == 0) node = (m * 4 + hi) * 4 + lo;        // (m, j, k)
          else if (d == 1) node = (hi * 4 + m) * 4 + lo;   // (i, m, k)
          else node = (hi * 4 + lo) * 4 + m;               // (i, j, m)
          split_tf32(s_ft[cell][comp * 3 + d][node], &bhi[e], &blo[e]);
        }
        mma_tf32(c, alo[st], bhi[0], bhi[1]);
        mma_tf32(c, ahi[st], blo[0], blo[1]);
        mma_tf32(c, ahi[st], bhi[0], bhi[1]);
      }
      // C (16 x 8): c0, c1 at (gid, 2 tig + 0/1), c2, c3 at (gid + 8, ...)
#pragma unroll
      for (int e = 0; e < 4; ++e) {
        const int r = gid + ((e & 2) ? 8 : 0), n = t * 8 + 2 * tig + (e & 1);
        const int pr = g * 4 + r / 4, cell = pr / kK, comp = pr % kK, i = r % 4;
        const int hi = n / 4, lo = n % 4;
        int node;
        if (d == 0) node = (i * 4 + hi) * 4 + lo;
        else if (d == 1) node = (hi * 4 + i) * 4 + lo;
        else node = (hi * 4 + lo) * 4 + i;
        if (d == 0) s_res[cell][comp][node] = c[e];
        else s_res[cell][comp][node] += c[e];
      }
    }
    __syncthreads();
  }
}

// TC (Q = 4, dg::Lobatto only): the differentiation on the tensor cores
// (tc_differentiate), everything else as the SIMT form.
// Resident blocks per SM the compiler is held to: p = 3 SIMT eight (32
// registers; 1.6 % faster per launch than its unconstrained 48 registers on
// the 64^3 case); the other instances at the register counts they take
// unconstrained (p = 2 and the tensor form 48, p = 1 40), since a looser
// bound lets the compiler trade occupancy for registers (90 at p = 2, and
// 66 % slower).
template <int Q, bool TC>
constexpr int mixed_cell_min_blocks() {
  return Q == 4 ? (TC ? 5 : 8) : (Q == 3 ? 5 : 6);
}

template <int Q, int STAGE, bool TC = false>
__global__ void __launch_bounds__(CellCfg<Q>::kThreads, mixed_cell_min_blocks<Q, TC>())
cell_update_mixed_kernel(CellArgs a, const float *__restrict__ geo32,
                         const float *__restrict__ node_w32) {
  constexpr int N = Q * Q * Q, QF = Q * Q, KN = kK * N;
  constexpr int CPB = CellCfg<Q>::kCells;
  static_assert(!TC || (Q == 4 && CPB == 4), "the tensor-core form is built for Q = 4");
  if (skip_block(a)) return;
  __shared__ float s_ft[CPB][15][N];
  __shared__ float s_res[TC ? CPB : 1][kK][TC ? N : 1];
  __shared__ float s_d[Q * Q];
  const int tid = threadIdx.x;
  if (tid < Q * Q) s_d[tid] = f64_to_f32(a.dmat[tid]);
  const int lc = tid / N, q = tid - lc * N;
  const int64_t c = (int64_t)blockIdx.x * CPB + lc;
  const bool active = c < a.n_cells;
  double uq[kK];
  float inv_w = 0.f;
  if (active) {
    const double *up = a.u_in + c * KN + q * kK;
#pragma unroll
    for (int k = 0; k < kK; ++k) uq[k] = up[k];
    // metric terms: per node, or (every cell affine) adj(J) and 1/det(J) of
    // the cell scaled by the node's weight
    float A[9];
    if (node_w32) {
      const float *g = geo32 + c * 10;
      const float wn = node_w32[q];
#pragma unroll
      for (int e = 0; e < 9; ++e) A[e] = wn * g[e];
      inv_w = node_w32[N + q] * g[9];
    } else {
      const float *g = geo32 + (c * N + q) * 10;
#pragma unroll
      for (int e = 0; e < 9; ++e) A[e] = g[e];
      inv_w = g[9];
    }
    const float r = f64_to_f32(uq[0]), mx = f64_to_f32(uq[1]), my = f64_to_f32(uq[2]),
                mz = f64_to_f32(uq[3]), en = f64_to_f32(uq[4]);
    // ConservativeToPrimitive with its clamp; rho < 0 and E < 0 are decided
    // on the FP64 values, p < 0 in FP32.
    float pr = r, u = mx, v = my, w = mz, p = en;
    if (negative64(uq[0]) || negative64(uq[4])) {
      pr = u = v = w = p = 0.f;
    } else if (nonzero64(uq[0])) {
      float inv = 1.0f / r;
      u = mx * inv; v = my * inv; w = mz * inv;
      p = (en - r * (0.5f * (u * u + v * v + w * w))) * (float)kGm1;
      if (p < 0.f) pr = u = v = w = p = 0.f;
    }
    const bool converted = pr != 0.f;
    float ft[15];
#pragma unroll
    for (int e = 0; e < 3; ++e) {
      float ve = u * A[0 * 3 + e] + v * A[1 * 3 + e] + w * A[2 * 3 + e];
      ft[0 * 3 + e] = converted ? pr * ve
                                : mx * A[0 * 3 + e] + my * A[1 * 3 + e] + mz * A[2 * 3 + e];
      ft[1 * 3 + e] = mx * ve + p * A[0 * 3 + e];
      ft[2 * 3 + e] = my * ve + p * A[1 * 3 + e];
      ft[3 * 3 + e] = mz * ve + p * A[2 * 3 + e];
      ft[4 * 3 + e] = (en + p) * ve;
    }
#pragma unroll
    for (int rr = 0; rr < 15; ++rr) s_ft[lc][rr][q] = ft[rr];
  } else if constexpr (TC) {
#pragma unroll
    for (int rr = 0; rr < 15; ++rr) s_ft[lc][rr][q] = 0.f;
  }
  __syncthreads();
  float res[kK];
  if constexpr (TC) {
    tc_differentiate(s_ft, s_d, s_res);
    if (!active) return;
#pragma unroll
    for (int rr = 0; rr < kK; ++rr) res[rr] = s_res[lc][rr][q];
  }
  if (!active) return;
  const int i = q / QF, j = (q / Q) % Q, k = q % Q;
  if constexpr (TC) {
  } else if (!a.fr) {
#pragma unroll
    for (int rr = 0; rr < kK; ++rr) {
      float s = 0.f;
#pragma unroll
      for (int m = 0; m < Q; ++m) {
        s = fmaf(s_ft[lc][rr * 3 + 0][(m * Q + j) * Q + k], s_d[m * Q + i], s);
        s = fmaf(s_ft[lc][rr * 3 + 1][(i * Q + m) * Q + k], s_d[m * Q + j], s);
        s = fmaf(s_ft[lc][rr * 3 + 2][(i * Q + j) * Q + m], s_d[m * Q + k], s);
      }
      res[rr] = s;
    }
  } else {
#pragma unroll
    for (int rr = 0; rr < kK; ++rr) {
      float s = 0.f;
#pragma unroll
      for (int m = 0; m < Q; ++m) {
        s = fmaf(-s_ft[lc][rr * 3 + 0][(m * Q + j) * Q + k], s_d[i * Q + m], s);
        s = fmaf(-s_ft[lc][rr * 3 + 1][(i * Q + m) * Q + k], s_d[j * Q + m], s);
        s = fmaf(-s_ft[lc][rr * 3 + 2][(i * Q + j) * Q + m], s_d[k * Q + m], s);
      }
      res[rr] = s;
    }
  }
  const int32_t *cf = a.cell_flux + c * 6 * QF;
  const float g1 = a.fr ? f64_to_f32(a.g1) : 0.f;
  auto lift = [&](int side, int t) {
    int32_t vv = cf[side * QF + t];
    if (vv == INT32_MIN) return;
    // FP32 face fluxes (the face kernel converts once per face point), or
    // FP64 ones converted here (FP64 shock cells: one flux buffer format)
    const int64_t slot = (int64_t)(vv >= 0 ? vv : ~vv) * kK;
    float fl[kK];
    bool no_flux;
    if (a.flux64) {
      const double *fd = a.flux + slot;
#pragma unroll
      for (int rr = 0; rr < kK; ++rr) fl[rr] = f64_to_f32(fd[rr]);
      no_flux = bits64(fd[0]) == kNoFluxBits;
    } else {
      const float *fs = reinterpret_cast<const float *>(a.flux) + slot;
#pragma unroll
      for (int rr = 0; rr < kK; ++rr) fl[rr] = fs[rr];
      no_flux = __float_as_uint(fl[0]) == kNoFluxBits32;
    }
    if (a.fr) {
      if (no_flux) return;  // no boundary
      const int dir = fr_dir(side);
      const float sigma = fr_sign(side) > 0 ? 1.f : -1.f, out_sign = vv >= 0 ? 1.f : -1.f;
#pragma unroll
      for (int rr = 0; rr < kK; ++rr)
        res[rr] -= g1 * (out_sign * fl[rr] - sigma * s_ft[lc][rr * 3 + dir][q]);
      return;
    }
    const float sign = vv >= 0 ? -1.f : 1.f;
#pragma unroll
    for (int rr = 0; rr < kK; ++rr) res[rr] = fmaf(sign, fl[rr], res[rr]);
  };
  // three axes, at most one face each (the per-face order: sides 0/5, 1/3, 4/2)
  if (k == 0 || k == Q - 1) lift(k == 0 ? 0 : 5, i * Q + j);
  if (j == 0 || j == Q - 1) lift(j == 0 ? 1 : 3, i * Q + k);
  if (i == 0 || i == Q - 1) lift(i == 0 ? 4 : 2, j * Q + k);
  double *out = a.u_out + c * KN + q * kK;
  bool bad = false;
  if (STAGE == kStageResidual) {
#pragma unroll
    for (int rr = 0; rr < kK; ++rr) {
      double val = f32_to_f64(res[rr] * inv_w);
      bad |= !finite64(val);
      out[rr] = val;
    }
  } else {
    // the stage's increment weight folded into the FP32 scale (exact for
    // 1, 1/2 and 1/4; 2/3 rounds to FP32 like the increment itself)
    using SC = StageCoef<STAGE>;
    const float wdt = inv_w * f64_to_f32(cell_dt(a.cs, a.state, c)) * (float)SC::cd;
    double nv[kK];
#pragma unroll
    for (int rr = 0; rr < kK; ++rr) {
      const double d = f32_to_f64(res[rr] * wdt);
      double val;
      if (STAGE == kStageEuler) {
        val = uq[rr] + d;
      } else {
        val = fma(SC::c0, a.u0[c * KN + q * kK + rr], fma(SC::cu, uq[rr], d));
      }
      bad |= !finite64(val);
      out[rr] = val;
      nv[rr] = val;
    }
    const bool surface = i == 0 || i == Q - 1 || j == 0 || j == Q - 1 || k == 0 || k == Q - 1;
    if (a.trace && surface) {
      double tr[3];
      node_trace<true>(nv, tr, a.trace_roe != 0);
      double *dst = a.trace + (c * N + q) * 3;
      dst[0] = tr[0]; dst[1] = tr[1]; dst[2] = tr[2];
    }
  }
  if (bad) atomicOr(&a.state->status, (unsigned)kStatusNonFinite);
  if (a.advance_time && !a.cs.dt && blockIdx.x == 0 && tid == 0) a.state->t += a.state->dt;
}

// dt: max over nodes of max(1e-5, max_speed) / length, as the bit pattern of
// a positive double (monotone as an unsigned integer).
// Max of `rate` into the handle's word, or into the word of each lane's case.
// Cases are contiguous runs of cells, so almost every warp is uniform.
// (rates are >= 1e-5 / length, or 0 for idle lanes: never negative or NaN;
// FP32 rates of the mixed form are widened exactly first)
__device__ __forceinline__ void reduce_rate(double rate, int key, DevState *state,
                                            unsigned long long *case_rate) {
  block_max_bits(bits64(rate), key, &state->max_rate_bits, case_rate);
}

// FP64 -> FP32 by truncating the mantissa (|result| within 2^-23 below |x|),
// a third of f64_to_f32's integer work: for the mixed time step's wave-speed
// estimate.  Magnitudes below the normal FP32 range give a signed zero, above
// it (and infinities, NaN) a signed infinity.
__device__ __forceinline__ float f64_to_f32_trunc(double x) {
  const unsigned long long b = bits64(x);
  const unsigned hi = (unsigned)(b >> 32), lo = (unsigned)b;
  const unsigned e = (hi >> 20) & 0x7ffu;
  unsigned bits = ((e - 896u) << 23) | ((hi & 0xfffffu) << 3) | (lo >> 29);
  bits = e <= 896u ? 0u : bits;
  bits = e >= 1151u ? 0x7f800000u : bits;
  return __uint_as_float((hi & 0x80000000u) | bits);
}

template <int Q>
__global__ void __launch_bounds__(512)
dt_reduce_kernel(const double *u, const double *cell_rate, int64_t n_nodes,
                 DevState *state, const int32_t *cell_case,
                 unsigned long long *case_rate) {
  constexpr int N = Q * Q * Q;
  int64_t gid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  double rate = 0;
  if (gid < n_nodes) {
    const double *p = u + gid * kK;
    Prim w = cons_to_prim(p[0], p[1], p[2], p[3], p[4]);
    double c = sound_speed(w);
    double speed = c + sqrt(w.u * w.u + w.v * w.v + w.w * w.w);
    rate = fmax(speed, 1e-5) * cell_rate[gid / N];
  }
  reduce_rate(rate, (case_rate && gid < n_nodes) ? cell_case[gid / N] : -1, state, case_rate);
}

// ---- FP64 time step at FP32 cost: the exact FP64 maximum of the rates is
// found in two passes.  Pass 1 brackets every node's rate [lo, hi] in FP32
// interval arithmetic (directed roundings), reduces max(lo) into the handle's
// (or the case's) rate word and stores each block's max(hi).  Pass 2 reads
// that word as a threshold: a block whose max(hi) is below it returns at
// once, without reading the solution; in the other blocks a node forms the
// FP64 rate, with exactly dt_reduce_kernel's arithmetic, when its own hi is
// not below the threshold, and those rates reduce into the same word.  The
// node of the largest FP64 rate always passes (its hi is above its rate,
// which is above every lo), every value the word holds during pass 2 is at
// most that rate, and a node that fails the test has a rate below it, so the
// word ends at the same FP64 maximum as dt_reduce_kernel's.  Nodes whose
// bracket is uncertain (a value above the FP32 range, a density or energy the
// clamp might zero, a pressure that cancels to below 2^-20 of the energy)
// take hi = +inf and always pass.

// [lo, hi] in FP32 around a double: the magnitude truncated and, unless
// exact, the next float up; below the normal FP32 range [0, FLT_MIN] with the
// sign.  False above the FP32 range (and for infinities and NaN).
__device__ __forceinline__ bool f32_bracket(double x, float *lo, float *hi) {
  const unsigned long long b = bits64(x);
  const unsigned h = (unsigned)(b >> 32), l = (unsigned)b;
  const unsigned e = (h >> 20) & 0x7ffu;
  if (e >= 1151u) return false;
  float t = 0.f, tu = 0.f;
  if ((b << 1) == 0ull) {
  } else if (e <= 896u) {
    tu = __uint_as_float(0x00800000u);  // FLT_MIN
  } else {
    const unsigned mag = ((e - 896u) << 23) | ((h & 0xfffffu) << 3) | (l >> 29);
    t = __uint_as_float(mag);
    tu = (l & 0x1fffffffu) == 0u ? t : __uint_as_float(mag + 1u);
  }
  if (h & 0x80000000u) {
    *lo = -tu;
    *hi = -t;
  } else {
    *lo = t;
    *hi = tu;
  }
  return true;
}

// FP32 bounds of the FP64 rate max(|u| + c, 1e-5) * cell_rate of a node;
// false when the node must take the FP64 path.  The FP64 arithmetic (one
// Newton reciprocal, products, two square roots) stays within 2^-30 relative
// of the exact rate once the pressure does not cancel below 2^-20 of the
// energy, and the bounds are widened by 2^-20 relative on top of that.
__device__ __forceinline__ bool rate_bracket(const double *p, double cell_rate, float *lo, float *hi) {
  // the double constants gamma - 1 = 0.4, gamma = 1.4 and 1e-5 bracketed
  const float g1l = __uint_as_float(0x3ecccccc), g1h = __uint_as_float(0x3ecccccd);
  const float gl = __uint_as_float(0x3fb33333), gh = __uint_as_float(0x3fb33334);
  const float fl = __uint_as_float(0x3727c5ac), fh = __uint_as_float(0x3727c5ad);
  constexpr float kTol = 9.5367431640625e-7f;  // 2^-20
  float rl, rh, el, eh, crl, crh;
  if (!f32_bracket(p[0], &rl, &rh) || !f32_bracket(p[4], &el, &eh) || !f32_bracket(cell_rate, &crl, &crh))
    return false;
  if (!(rl > 0.f) || !(el >= 0.f) || !(crl > 0.f)) return false;
  float m2l = 0.f, m2h = 0.f;
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    float ml, mh;
    if (!f32_bracket(p[1 + d], &ml, &mh)) return false;
    const float al = ml >= 0.f ? ml : (mh <= 0.f ? -mh : 0.f);
    const float ah = fmaxf(-ml, mh);
    m2l = __fadd_rd(m2l, __fmul_rd(al, al));
    m2h = __fadd_ru(m2h, __fmul_ru(ah, ah));
  }
  const float irl = __frcp_rd(rh), irh = __frcp_ru(rl);  // bounds of 1 / rho
  const float kel = __fmul_rd(__fmul_rd(m2l, 0.5f), irl), keh = __fmul_ru(__fmul_ru(m2h, 0.5f), irh);
  const float pl = __fmul_rd(__fsub_rd(el, keh), g1l), ph = __fmul_ru(__fsub_ru(eh, kel), g1h);
  if (!(pl > __fmul_ru(__fadd_ru(eh, keh), kTol))) return false;
  const float c2l = __fmul_rd(__fmul_rd(gl, pl), irl), c2h = __fmul_ru(__fmul_ru(gh, ph), irh);
  const float ul = __fmul_rd(__fsqrt_rd(m2l), irl), uh = __fmul_ru(__fsqrt_ru(m2h), irh);
  const float sl = fmaxf(__fadd_rd(__fsqrt_rd(c2l), ul), fl);
  const float sh = fmaxf(__fadd_ru(__fsqrt_ru(c2h), uh), fh);
  *lo = __fmul_rd(__fmul_rd(sl, crl), 1.f - kTol);
  *hi = __fmul_ru(__fmul_ru(sh, crh), 1.f + kTol);
  return true;
}

template <int Q>
__global__ void __launch_bounds__(512)
dt_bound_kernel(const double *u, const double *cell_rate, int64_t n_nodes, DevState *state,
                const int32_t *cell_case, unsigned long long *case_rate, unsigned *block_hi) {
  constexpr int N = Q * Q * Q;
  __shared__ unsigned s_hi[16];
  const int64_t gid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  double lo64 = 0;
  unsigned hib = 0u;
  if (gid < n_nodes) {
    float lo, hi;
    if (rate_bracket(u + gid * kK, cell_rate[gid / N], &lo, &hi)) {
      lo64 = f32_to_f64(lo);
      hib = __float_as_uint(hi);
    } else {
      hib = 0x7f800000u;  // +inf
    }
  }
  // the block's max(hi): non-negative floats order as their bit patterns
  hib = __reduce_max_sync(0xffffffffu, hib);
  if ((threadIdx.x & 31) == 0) s_hi[threadIdx.x >> 5] = hib;
  reduce_rate(lo64, (case_rate && gid < n_nodes) ? cell_case[gid / N] : -1, state, case_rate);
  // reduce_rate's barrier orders the s_hi writes before this read
  if (threadIdx.x == 0) {
    unsigned m = 0u;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) m = max(m, s_hi[w]);
    block_hi[blockIdx.x] = m;
  }
}

template <int Q>
__global__ void __launch_bounds__(512)
dt_exact_kernel(const double *u, const double *cell_rate, int64_t n_nodes, DevState *state,
                const int32_t *cell_case, unsigned long long *case_rate, const unsigned *block_hi) {
  constexpr int N = Q * Q * Q;
  __shared__ int s_skip;
  const int64_t gid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const double bh = f32_to_f64(__uint_as_float(block_hi[blockIdx.x]));
  if (!case_rate) {
    // one decision for the block (the word may grow while its threads read it)
    if (threadIdx.x == 0)
      s_skip = bh < __longlong_as_double((long long)*(volatile const unsigned long long *)&state->max_rate_bits);
    __syncthreads();
    if (s_skip) return;
  }
  double rate = 0;
  int key = -1;
  if (gid < n_nodes) {
    if (case_rate) key = cell_case[gid / N];
    const unsigned long long *word = case_rate ? &case_rate[key] : &state->max_rate_bits;
    const double threshold = __longlong_as_double((long long)*(volatile const unsigned long long *)word);
    if (!(bh < threshold)) {
      const double *p = u + gid * kK;
      const double cr = cell_rate[gid / N];
      float lo, hi;
      if (!rate_bracket(p, cr, &lo, &hi) || !(f32_to_f64(hi) < threshold)) {
        Prim w = cons_to_prim(p[0], p[1], p[2], p[3], p[4]);
        double c = sound_speed(w);
        double speed = c + sqrt(w.u * w.u + w.v * w.v + w.w * w.w);
        rate = fmax(speed, 1e-5) * cr;
      }
    }
  }
  reduce_rate(rate, key, state, case_rate);
}

// Mixed-precision dt reduction: wave speeds and rates in FP32 (the FP32 copy
// of the cell rates), the state converted by mantissa truncation on the
// integer pipes (the hardware conversion issues on the FP64 unit, the
// bottleneck of this part), the maximum by integer reductions: no FP64
// instruction per node.
template <int Q>
__global__ void __launch_bounds__(512)
dt_reduce_mixed_kernel(const double *u, const float *cell_rate32, int64_t n_nodes,
                       DevState *state, const int32_t *cell_case,
                       unsigned long long *case_rate) {
  constexpr int N = Q * Q * Q;
  int64_t gid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  float rate = 0.f;
  if (gid < n_nodes) {
    const double *p = u + gid * kK;
    float r = f64_to_f32_trunc(p[0]), mx = f64_to_f32_trunc(p[1]), my = f64_to_f32_trunc(p[2]),
          mz = f64_to_f32_trunc(p[3]), en = f64_to_f32_trunc(p[4]);
    float speed = 0.f;
    if (r > 0.f && en >= 0.f) {
      float inv = 1.0f / r;
      float uu = (mx * mx + my * my + mz * mz) * inv * inv;
      float pp = (en - 0.5f * r * uu) * (float)kGm1;
      float c = pp > 0.f ? sqrtf((float)kGamma * pp * inv) : 0.f;
      speed = pp >= 0.f ? c + sqrtf(uu) : 0.f;
    } else if (r == 0.f && en >= 0.f) {
      speed = sqrtf(mx * mx + my * my + mz * mz);
    }
    rate = fmaxf(speed, 1e-5f) * cell_rate32[gid / N];
  }
  reduce_rate(f32_to_f64(rate), (case_rate && gid < n_nodes) ? cell_case[gid / N] : -1, state, case_rate);
}

__global__ void dt_finalize_kernel(DevState *state, int fr) {
  double max_rate = __longlong_as_double((long long)state->max_rate_bits);
  double min_dt = max_rate > 0 ? 1.0 / max_rate : 1.e+100;
  double dt = state->cfl * min_dt;
  dt = fmin(dt, state->dt_guess);
  // fr::Lobatto::GetTimeStep doubles the base step (fr/lobatto.hpp:220-222)
  if (fr) dt = fmin(state->dt_guess, 2.0 * dt);
  state->dt = dt;
  state->max_rate_bits = 0ull;
}

// Per-case finalisation (one block): dt_k from each case's maximum rate, the
// handle's dt = min over cases (what mcfd_time_step reports).
__global__ void dt_finalize_cases_kernel(DevState *state, unsigned long long *case_rate,
                                         double *case_dt, int n, int fr) {
  __shared__ double s_min[32];
  double local = 1.e+300;
  for (int k = threadIdx.x; k < n; k += blockDim.x) {
    const double max_rate = __longlong_as_double((long long)case_rate[k]);
    const double min_dt = max_rate > 0 ? 1.0 / max_rate : 1.e+100;
    double dt = fmin(state->cfl * min_dt, state->dt_guess);
    if (fr) dt = fmin(state->dt_guess, 2.0 * dt);
    case_dt[k] = dt;
    case_rate[k] = 0ull;
    local = fmin(local, dt);
  }
  for (int o = 16; o > 0; o >>= 1) local = fmin(local, __shfl_xor_sync(0xffffffffu, local, o));
  if ((threadIdx.x & 31) == 0) s_min[threadIdx.x >> 5] = local;
  __syncthreads();
  if (threadIdx.x == 0) {
    double m = s_min[0];
    for (int w = 1; w < (int)(blockDim.x >> 5); ++w) m = fmin(m, s_min[w]);
    state->dt = m;
  }
}

// After the last stage: t_k += dt_k; the handle's t = min over cases.
__global__ void advance_cases_kernel(DevState *state, double *case_t, const double *case_dt,
                                     int n) {
  __shared__ double s_min[32];
  double local = 1.e+300;
  for (int k = threadIdx.x; k < n; k += blockDim.x) {
    case_t[k] += case_dt[k];
    local = fmin(local, case_t[k]);
  }
  for (int o = 16; o > 0; o >>= 1) local = fmin(local, __shfl_xor_sync(0xffffffffu, local, o));
  if ((threadIdx.x & 31) == 0) s_min[threadIdx.x >> 5] = local;
  __syncthreads();
  if (threadIdx.x == 0) {
    double m = s_min[0];
    for (int w = 1; w < (int)(blockDim.x >> 5); ++w) m = fmin(m, s_min[w]);
    state->t = m;
  }
}

__global__ void set_cases_kernel(double *case_t, double *case_dt, int n, double t, double dt) {
  for (int k = threadIdx.x; k < n; k += blockDim.x) {
    case_t[k] = t;
    case_dt[k] = dt;
  }
}

// Node traces of a state (Buffers::trace), one thread per node.
template <bool FAST_SQRT>
__global__ void __launch_bounds__(256)
trace_kernel(const double *u, double *trace, int64_t n_nodes, int roe) {
  const int64_t gid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (gid >= n_nodes) return;
  double tr[3];
  node_trace<FAST_SQRT>(u + gid * kK, tr, roe != 0);
  trace[gid * 3 + 0] = tr[0];
  trace[gid * 3 + 1] = tr[1];
  trace[gid * 3 + 2] = tr[2];
}

__global__ void set_state_kernel(DevState *state, double t, double dt,
                                 double dt_guess, double cfl, int reset_rate) {
  state->t = t;
  state->dt = dt;
  state->dt_guess = dt_guess;
  state->cfl = cfl;
  if (reset_rate) state->max_rate_bits = 0ull;
}

template <int Q, int R>
void face_launch(mcfd_handle *h, const FaceArgs &fa) {
  const int bs = h->tune.face_block;
  int64_t blocks = (fa.n_points + bs - 1) / bs;
  if constexpr (R == kRusanov || R == kRoe || R == kHllc) {
    if (h->opt.precision == 1) {
      face_flux_kernel<Q, R, true><<<(unsigned)blocks, bs, 0, h->stream>>>(fa);
      return;
    }
  }
  face_flux_kernel<Q, R, false><<<(unsigned)blocks, bs, 0, h->stream>>>(fa);
}

template <int Q>
void face_dispatch_r(mcfd_handle *h, const FaceArgs &fa) {
  switch (h->opt.riemann) {
    case kExact: face_launch<Q, kExact>(h, fa); break;
    case kHllc: face_launch<Q, kHllc>(h, fa); break;
    case kAusm: face_launch<Q, kAusm>(h, fa); break;
    case kRoe: face_launch<Q, kRoe>(h, fa); break;
    default: face_launch<Q, kRusanov>(h, fa); break;
  }
}

template <int Q, int S>
void cell_launch(mcfd_handle *h, const CellArgs &ca) {
  constexpr int CPB = CellCfg<Q>::kCells;
  int64_t blocks = (ca.n_cells + CPB - 1) / CPB;
  if (ca.nu)
    cell_update_kernel<Q, S, true><<<(unsigned)blocks, CellCfg<Q>::kThreads, 0, h->stream>>>(ca);
  else
    cell_update_kernel<Q, S><<<(unsigned)blocks, CellCfg<Q>::kThreads, 0, h->stream>>>(ca);
}

template <int Q, int S>
void cell_launch_mixed(mcfd_handle *h, const CellArgs &ca) {
  constexpr int CPB = CellCfg<Q>::kCells;
  int64_t blocks = (ca.n_cells + CPB - 1) / CPB;
  const float *w32 = h->mesh.geo32_affine ? h->mesh.node_w32 : nullptr;
  if constexpr (Q == 4) {
    if (h->opt.tensor_contraction && !ca.fr) {
      cell_update_mixed_kernel<Q, S, true><<<(unsigned)blocks, CellCfg<Q>::kThreads, 0, h->stream>>>(
          ca, h->mesh.cell_geo32, w32);
      return;
    }
  }
  cell_update_mixed_kernel<Q, S><<<(unsigned)blocks, CellCfg<Q>::kThreads, 0, h->stream>>>(
      ca, h->mesh.cell_geo32, w32);
}

template <int Q>
void cell_dispatch_s(mcfd_handle *h, int stage, const CellArgs &ca) {
  if (h->opt.precision == 1) {
    switch (stage) {
      case kStageEuler: cell_launch_mixed<Q, kStageEuler>(h, ca); break;
      case kStageRk2Last: cell_launch_mixed<Q, kStageRk2Last>(h, ca); break;
      case kStageRk3Mid: cell_launch_mixed<Q, kStageRk3Mid>(h, ca); break;
      case kStageRk3Last: cell_launch_mixed<Q, kStageRk3Last>(h, ca); break;
      default: cell_launch_mixed<Q, kStageResidual>(h, ca); break;
    }
    return;
  }
  switch (stage) {
    case kStageEuler: cell_launch<Q, kStageEuler>(h, ca); break;
    case kStageRk2Last: cell_launch<Q, kStageRk2Last>(h, ca); break;
    case kStageRk3Mid: cell_launch<Q, kStageRk3Mid>(h, ca); break;
    case kStageRk3Last: cell_launch<Q, kStageRk3Last>(h, ca); break;
    default: cell_launch<Q, kStageResidual>(h, ca); break;
  }
}

}  // namespace

// Step bounds only (dt guess, CFL, rate reset), the device time kept.
__global__ void set_bounds_kernel(DevState *state, double dt_guess, double cfl) {
  state->dt_guess = dt_guess;
  state->cfl = cfl;
  state->max_rate_bits = 0ull;
}

int launch_set_bounds(mcfd_handle *h, double dt_guess, double cfl) {
  set_bounds_kernel<<<1, 1, 0, h->stream>>>(h->buf.state, dt_guess, cfl);
  return 1;
}

int launch_set_state(mcfd_handle *h, double t, double dt, double dt_guess,
                     double cfl, int reset_rate) {
  set_state_kernel<<<1, 1, 0, h->stream>>>(h->buf.state, t, dt, dt_guess, cfl,
                                           reset_rate);
  return 1;
}

int launch_face_flux(mcfd_handle *h, const double *u, double stage_c, bool props_fresh) {
  if (h->opt.scheme == kSchemeModal) return launch_modal_face_flux(h, u, stage_c);
  // viscosity: the properties of this stage input first (SetSolutionColumn
  // runs UpdateProperties, with_viscosity.hpp:56-59)
  int n = 0;
  if (h->visc.on && !props_fresh) n += launch_visc_properties(h, u, 0);
  const Mesh &m = h->mesh;
  FaceArgs fa{u, m.face_cells, m.face_group, m.face_geo, m.face_xyz,
              m.face_map, m.bcs, h->buf.flux, h->buf.state, stage_c,
              m.n_points, m.n_groups, h->opt.scheme == 1, case_view(h),
              (h->use_trace && h->trace_for == u) ? h->buf.trace : nullptr,
              h->opt.precision == 1 && !h->opt.shock_fp64, h->visc.on ? 1 : 0, m.bc_row, m.face_nh};
  if (m.n_points == 0) return n;
  switch (m.q) {
    case 2: face_dispatch_r<2>(h, fa); break;
    case 3: face_dispatch_r<3>(h, fa); break;
    default: face_dispatch_r<4>(h, fa); break;
  }
  ++n;
  if (h->visc.on) n += launch_visc_face_flux(h, u);
  return n;
}

int launch_cell_update(mcfd_handle *h, int stage, const double *u_in,
                       const double *u0, double *u_out, int advance_time) {
  if (h->opt.scheme == kSchemeModal)
    return launch_modal_cell_update(h, stage, u_in, u0, u_out, advance_time);
  const Mesh &m = h->mesh;
  double *trace = (h->use_trace && stage != kStageResidual) ? h->buf.trace : nullptr;
  CellArgs ca{u_in, u0, u_out, m.cell_geo, m.cell_flux, h->buf.flux, m.dmat,
              h->buf.state, m.n_cells, advance_time, h->opt.scheme == 1, h->opt.fr_g1,
              case_view(h), trace, h->visc.on ? h->visc.nu : nullptr, h->opt.riemann == kRoe};
  if (trace) h->trace_for = u_out;
  if (h->opt.shock_fp64 && h->opt.precision == 1 && h->lim.block_hot) {
    // the mixed kernel on the quiet blocks, the FP64 kernel on the blocks of
    // the last limiter pass's flagged cells and their neighbours; one FP64
    // flux buffer for both
    CellArgs mixed = ca, fp64 = ca;
    mixed.block_hot = fp64.block_hot = h->lim.block_hot;
    mixed.hot_mode = 1;
    fp64.hot_mode = 2;
    mixed.flux64 = fp64.flux64 = 1;
    h->opt.precision = 0;
    switch (m.q) {
      case 2: cell_dispatch_s<2>(h, stage, fp64); break;
      case 3: cell_dispatch_s<3>(h, stage, fp64); break;
      default: cell_dispatch_s<4>(h, stage, fp64); break;
    }
    h->opt.precision = 1;
    switch (m.q) {
      case 2: cell_dispatch_s<2>(h, stage, mixed); break;
      case 3: cell_dispatch_s<3>(h, stage, mixed); break;
      default: cell_dispatch_s<4>(h, stage, mixed); break;
    }
    return 2;
  }
  switch (m.q) {
    case 2: cell_dispatch_s<2>(h, stage, ca); break;
    case 3: cell_dispatch_s<3>(h, stage, ca); break;
    default: cell_dispatch_s<4>(h, stage, ca); break;
  }
  return 1;
}

// Finalisation of a dt reduction: the handle's word, or one word per case.
int launch_dt_finalize(mcfd_handle *h) {
  const int fr = h->opt.scheme == 1;
  if (h->cases.n) {
    dt_finalize_cases_kernel<<<1, 1024, 0, h->stream>>>(h->buf.state, h->cases.rate,
                                                      h->cases.dt, h->cases.n, fr);
  } else {
    dt_finalize_kernel<<<1, 1, 0, h->stream>>>(h->buf.state, fr);
  }
  return 1;
}

int launch_dt(mcfd_handle *h, const double *u) {
  if (h->opt.scheme == kSchemeModal) return launch_modal_dt(h, u);
  if (h->visc.on) return launch_visc_properties(h, u, 1) + launch_visc_dt_finalize(h);
  const Mesh &m = h->mesh;
  int64_t nodes = m.n_cells * m.n;
  const int bs = h->tune.dt_block;
  unsigned blocks = (unsigned)((nodes + bs - 1) / bs);
  const int32_t *cc = h->cases.cell_case;
  unsigned long long *cr = h->cases.n ? h->cases.rate : nullptr;
  // (with FP64 shock cells too: an FP64 time step measured no closer to the
  // FP64 form over 200 limited steps and costs 1.6 ms per four-quadrant step)
  if (h->opt.precision == 1) {
    switch (m.q) {
      case 2: dt_reduce_mixed_kernel<2><<<blocks, bs, 0, h->stream>>>(u, m.cell_rate32, nodes, h->buf.state, cc, cr); break;
      case 3: dt_reduce_mixed_kernel<3><<<blocks, bs, 0, h->stream>>>(u, m.cell_rate32, nodes, h->buf.state, cc, cr); break;
      default: dt_reduce_mixed_kernel<4><<<blocks, bs, 0, h->stream>>>(u, m.cell_rate32, nodes, h->buf.state, cc, cr); break;
    }
  } else {
    // the exact FP64 maximum in two passes (FP32 brackets, then FP64 only
    // for the nodes that can hold it); buf.dt_hi holds a word per block of
    // at least 128 threads
    unsigned *bh = h->buf.dt_hi;
    switch (m.q) {
      case 2:
        dt_bound_kernel<2><<<blocks, bs, 0, h->stream>>>(u, m.cell_rate, nodes, h->buf.state, cc, cr, bh);
        dt_exact_kernel<2><<<blocks, bs, 0, h->stream>>>(u, m.cell_rate, nodes, h->buf.state, cc, cr, bh);
        break;
      case 3:
        dt_bound_kernel<3><<<blocks, bs, 0, h->stream>>>(u, m.cell_rate, nodes, h->buf.state, cc, cr, bh);
        dt_exact_kernel<3><<<blocks, bs, 0, h->stream>>>(u, m.cell_rate, nodes, h->buf.state, cc, cr, bh);
        break;
      default:
        dt_bound_kernel<4><<<blocks, bs, 0, h->stream>>>(u, m.cell_rate, nodes, h->buf.state, cc, cr, bh);
        dt_exact_kernel<4><<<blocks, bs, 0, h->stream>>>(u, m.cell_rate, nodes, h->buf.state, cc, cr, bh);
        break;
    }
    return 2 + launch_dt_finalize(h);
  }
  return 1 + launch_dt_finalize(h);
}

int launch_trace(mcfd_handle *h, const double *u) {
  if (!h->use_trace) return 0;
  const int64_t nodes = h->mesh.n_cells * h->mesh.n;
  const unsigned blocks = (unsigned)((nodes + 255) / 256);
  const int roe = h->opt.riemann == kRoe;
  if (h->opt.precision == 1)
    trace_kernel<true><<<blocks, 256, 0, h->stream>>>(u, h->buf.trace, nodes, roe);
  else
    trace_kernel<false><<<blocks, 256, 0, h->stream>>>(u, h->buf.trace, nodes, roe);
  h->trace_for = u;
  return 1;
}

int launch_advance_cases(mcfd_handle *h) {
  if (!h->cases.n) return 0;
  advance_cases_kernel<<<1, 1024, 0, h->stream>>>(h->buf.state, h->cases.t, h->cases.dt, h->cases.n);
  return 1;
}

int launch_set_cases(mcfd_handle *h, double t, double dt) {
  if (!h->cases.n) return 0;
  set_cases_kernel<<<1, 1024, 0, h->stream>>>(h->cases.t, h->cases.dt, h->cases.n, t, dt);
  return 1;
}

// ---------------------------------------------------------------------------
// Residual for callers that cannot allocate device memory.
//
// The face-flux scratch of this variant is a fixed file-scope device array
// instead of the handle's allocated buffer.  Host code must not pass the
// symbol itself to a kernel (on the host it names a host-side stand-in), so
// the device address is fetched with cudaGetSymbolAddress once per device,
// with that device current, on the first call, and cached.
namespace {
__device__ __align__(256) double g_static_face_flux[kStaticFluxCapacity];

struct StaticScratchSlot {
  double *ptr = nullptr;
  bool ready = false;
};
constexpr int kMaxDevices = 64;
StaticScratchSlot g_static_slots[kMaxDevices];
std::mutex g_static_mutex;
}  // namespace

int static_flux_scratch(int device, double **ptr, std::string *err) {
  if (device < 0 || device >= kMaxDevices) {
    *err = "device ordinal out of range for the static scratch table";
    return 1;
  }
  std::lock_guard<std::mutex> lock(g_static_mutex);
  StaticScratchSlot &slot = g_static_slots[device];
  if (!slot.ready) {
    void *p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_static_face_flux);
    if (e != cudaSuccess) {
      *err = std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e);
      return 1;
    }
    slot.ptr = static_cast<double *>(p);
    slot.ready = true;
  }
  *ptr = slot.ptr;
  return 0;
}

int launch_residual_static_scratch(mcfd_handle *h, const double *d_u,
                                   double *d_r, double *scratch) {
  const Mesh &m = h->mesh;
  FaceArgs fa{d_u, m.face_cells, m.face_group, m.face_geo, m.face_xyz,
              m.face_map, m.bcs, scratch, h->buf.state, 0.0,
              m.n_points, m.n_groups, h->opt.scheme == 1, case_view(h), nullptr,
              h->opt.precision == 1, 0, m.bc_row, nullptr};
  CellArgs ca{d_u, nullptr, d_r, m.cell_geo, m.cell_flux, scratch, m.dmat,
              h->buf.state, m.n_cells, 0, h->opt.scheme == 1, h->opt.fr_g1, case_view(h), nullptr,
              nullptr, 0};
  int n = 0;
  if (m.n_points > 0) {
    switch (m.q) {
      case 2: face_dispatch_r<2>(h, fa); break;
      case 3: face_dispatch_r<3>(h, fa); break;
      default: face_dispatch_r<4>(h, fa); break;
    }
    ++n;
  }
  switch (m.q) {
    case 2: cell_dispatch_s<2>(h, kStageResidual, ca); break;
    case 3: cell_dispatch_s<3>(h, kStageResidual, ca); break;
    default: cell_dispatch_s<4>(h, kStageResidual, ca); break;
  }
  return n + 1;
}

// The stages of RungeKutta<order>::Update with the result left in buf.u.
// Stage times: t, t + dt, t + dt/2 (rk.hpp:34-42).  The last stage also
// advances the device time by dt.
int launch_rk_stage_sequence(mcfd_handle *h, int order, const double *u_in, double *u_out,
                             bool after_dt) {
  Buffers &b = h->buf;
  const double *u = u_in ? u_in : b.u;
  double *out = u_out ? u_out : b.u;
  int n = 0;
  // Each stage result is a SetSolutionColumn in the reference, which runs the
  // limiter when one is installed (spatial/with_limiter.hpp:56-59).
  if (order == 1) {
    n += launch_face_flux(h, u, 0.0, after_dt);
    n += launch_cell_update(h, kStageEuler, u, nullptr, out, 1);
    n += launch_limiter(h, out);
  } else if (order == 2) {
    n += launch_face_flux(h, u, 0.0, after_dt);
    n += launch_cell_update(h, kStageEuler, u, nullptr, b.u1, 0);
    n += launch_limiter(h, b.u1);
    n += launch_face_flux(h, b.u1, 1.0);
    n += launch_cell_update(h, kStageRk2Last, b.u1, u, out, 1);
    n += launch_limiter(h, out);
  } else {
    n += launch_face_flux(h, u, 0.0, after_dt);
    n += launch_cell_update(h, kStageEuler, u, nullptr, b.u1, 0);
    n += launch_limiter(h, b.u1);
    n += launch_face_flux(h, b.u1, 1.0);
    n += launch_cell_update(h, kStageRk3Mid, b.u1, u, b.u2, 0);
    n += launch_limiter(h, b.u2);
    n += launch_face_flux(h, b.u2, 0.5);
    n += launch_cell_update(h, kStageRk3Last, b.u2, u, out, 1);
    n += launch_limiter(h, out);
  }
  return n + launch_advance_cases(h);
}

}  // namespace mcfd
