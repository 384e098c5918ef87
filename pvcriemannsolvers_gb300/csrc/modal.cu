// Modal DG (dg::General over polynomial::Projection) on Hex8 and Tet4 cells,
// FP64, on sm_103a.
//
// The reference evaluates, at every quadrature point, the cell's orthonormal
// basis psi = S T(x - centre) (T the M Taylor monomials, S lower triangular)
// and its gradient, and adds F . grad(psi) w (volume, spatial/dg/general.hpp:
// 58-69) and -F^ w psi (faces, general.hpp:70-202) to the K x M block.  Here
// the same sums are reassociated through S:
//   u(x)   = sum_m c_m psi_m(x) = sum_j a_j T_j(x - centre),   a = S^T c
//   R_m    = sum_j S_mj Rt_j,   Rt_j = sum_q w F . grad T_j - sum_f w F^ T_j
// so a point costs one K x M contraction with the Taylor coefficients a and a
// sparse update of Rt (each monomial has at most three non-zero partials);
// S is applied once per cell.  Per RK stage three kernels run:
//   modal_taylor_kernel  a = S^T c of the stage input, one thread per
//                        (cell, pair of monomials j and M - 1 - j, component)
//   modal_face_kernel    one thread per face point: u on both sides from a,
//                        the rotated Riemann or boundary flux, times w
//   modal_cell_kernel    one thread per cell: volume quadrature, lift of its
//                        <= 6 faces' point fluxes (gathered, atomic-free),
//                        R = S Rt and the RK stage combination
// The time step follows fem.hpp:417-435 with the Projection quirk that
// GetValue(i) for i < M reads the value at quadrature point i.
#include <cuda_runtime.h>

#include <cstdint>

#include "euler.cuh"
#include "handle.hpp"
#include "vtk_locals.cuh"

namespace mcfd {
namespace {

// Cell-kernel storage: the Taylor coefficients sit in shared memory, one
// column of a [K M][block] array per thread (conflict-free, at most 25.6 KB
// per block); the K x M residual accumulators stay in registers.  At M = 20
// part of them spills to L1, which measured faster (25 ms against 40 ms per
// launch on the ensemble's p = 3 handle) than keeping them in shared memory.
template <int M>
struct ModalCfg {
  static constexpr int kBlock = M == 20 ? 32 : 64;
  static constexpr int kSmemBytes = kK * M * kBlock * 8;
};

// Taylor monomials at offset (x, y, z) in the reference's order
// (basis/taylor.hpp:198-218).
template <int M, class Real>
__device__ __forceinline__ void taylor_values(Real x, Real y, Real z, Real *t) {
  t[0] = Real(1);
  t[1] = x; t[2] = y; t[3] = z;
  if constexpr (M >= 10) {
    t[4] = x * x; t[5] = x * y; t[6] = x * z;
    t[7] = y * y; t[8] = y * z; t[9] = z * z;
  }
  if constexpr (M >= 20) {
    t[10] = x * t[4]; t[11] = x * t[5]; t[12] = x * t[6];
    t[13] = x * t[7]; t[14] = x * t[8]; t[15] = x * t[9];
    t[16] = y * t[7]; t[17] = y * t[8]; t[18] = y * t[9];
    t[19] = z * t[9];
  }
}

// rt[j] += gx dT_j/dx + gy dT_j/dy + gz dT_j/dz at offset (x, y, z), t the
// monomial values there (basis/taylor.hpp:387-472).
// `rt(j)` yields the accumulator of monomial j (registers or shared memory).
template <int M, class Real, class R>
__device__ __forceinline__ void add_gradient(const Real *t, Real gx, Real gy, Real gz,
                                             R &&rt) {
  rt(1) += gx;
  rt(2) += gy;
  rt(3) += gz;
  if constexpr (M >= 10) {
    const Real x = t[1], y = t[2], z = t[3];
    rt(4) += gx * (2 * x);
    rt(5) += gx * y + gy * x;
    rt(6) += gx * z + gz * x;
    rt(7) += gy * (2 * y);
    rt(8) += gy * z + gz * y;
    rt(9) += gz * (2 * z);
  }
  if constexpr (M >= 20) {
    const Real xx = t[4], xy = t[5], xz = t[6], yy = t[7], yz = t[8], zz = t[9];
    rt(10) += gx * (3 * xx);
    rt(11) += gx * (2 * xy) + gy * xx;
    rt(12) += gx * (2 * xz) + gz * xx;
    rt(13) += gx * yy + gy * (2 * xy);
    rt(14) += gx * yz + gy * xz + gz * xy;
    rt(15) += gx * zz + gz * (2 * xz);
    rt(16) += gy * (3 * yy);
    rt(17) += gy * (2 * yz) + gz * yy;
    rt(18) += gy * zz + gz * (2 * yz);
    rt(19) += gz * (3 * zz);
  }
}

// a[c][j][k] = sum_{m >= j} S[m][j] u[c][m][k].  A thread takes the rows j
// and M - 1 - j (M is even), M + 1 products in all: the same count on every
// lane (one row per thread gave lanes M - j products, and the FP64 pipe spent
// the longest row's slots on the whole warp).
template <int M>
__global__ void __launch_bounds__(256)
modal_taylor_kernel(const double *u, const double *s, double *a, int64_t n) {
  static_assert(M % 2 == 0, "paired rows need an even basis size");
  constexpr int KM = kK * M, KH = kK * (M / 2), NS = M * (M + 1) / 2;
  int64_t gid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (gid >= n) return;
  const int64_t c = gid / KH;
  const int r = (int)(gid - c * KH), j0 = r / kK, k = r - j0 * kK, j1 = M - 1 - j0;
  const double *uc = u + c * KM;
  const double *sc = s + c * NS;
  double acc0 = 0, acc1 = 0;
  for (int m = j0; m < M; ++m) acc0 += sc[m * (m + 1) / 2 + j0] * uc[m * kK + k];
  for (int m = j1; m < M; ++m) acc1 += sc[m * (m + 1) / 2 + j1] * uc[m * kK + k];
  a[c * KM + j0 * kK + k] = acc0;
  a[c * KM + j1 * kK + k] = acc1;
}

struct ModalFaceArgs {
  const double *taylor;
  const double4 *center;
  const int2 *face_cells;
  const int32_t *face_group;
  const int32_t *point_face;
  const double4 *fpt, *fnrm, *fshift;
  const BcDev *bcs;
  double *flux;
  DevState *state;
  double stage_c;
  int64_t n_points;
  int n_groups;
  CaseView cs;
  const int32_t *bc_row;  // [points] row in the group's boundary table, or null
};

template <int M, class Real>
__device__ __forceinline__ void eval_taylor(const Real *a, const Real *t, Real *u) {
#pragma unroll
  for (int k = 0; k < kK; ++k) {
    Real s = 0;
#pragma unroll
    for (int j = 0; j < M; ++j) s += a[j * kK + k] * t[j];
    u[k] = s;
  }
}

template <int M, int R>
__global__ void __launch_bounds__(512) modal_face_kernel(ModalFaceArgs a) {
  int64_t gid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (gid >= a.n_points) return;
  const int f = a.point_face[gid];
  const int2 cells = a.face_cells[f];
  const double4 x = a.fpt[gid];
  const double4 nv = a.fnrm[gid];
  const double n[3] = {nv.x, nv.y, nv.z};
  const double4 ch = a.center[cells.x];
  double t[M], uh[kK], out[kK];
  taylor_values<M>(x.x - ch.x, x.y - ch.y, x.z - ch.z, t);
  eval_taylor<M>(a.taylor + (int64_t)cells.x * M * kK, t, uh);
  bool not_converged = false;
  if (cells.y >= 0) {
    const double4 sh = a.fshift[f];
    const double4 cs = a.center[cells.y];
    double us[kK];
    taylor_values<M>((x.x - sh.x) - cs.x, (x.y - sh.y) - cs.y, (x.z - sh.z) - cs.z, t);
    eval_taylor<M>(a.taylor + (int64_t)cells.y * M * kK, t, us);
    // the point weight folded into the flux (Rusanov and Roe through the
    // half-weighted normal, the others by one multiplication)
    interior_flux_weighted<R, false>(uh, us, n, x.w, out, &not_converged);
  } else {
    Prim l = cons_to_prim(uh[0], uh[1], uh[2], uh[3], uh[4]);
    const int grp = a.face_group[f];
    if (grp >= 0 && grp < a.n_groups && a.bcs[grp].kind != kBcNone) {
      const BcDev &bc = a.bcs[grp];
      double given[kK];
      double t = a.state->t + a.stage_c * a.state->dt;
      if (a.cs.t) {
        const int k = a.cs.cell_case[cells.x];
        t = a.cs.t[k] + a.stage_c * a.cs.dt[k];
      }
      boundary_given(bc, x.x, x.y, x.z, t, a.bc_row ? a.bc_row[gid] : -1, given);
      flux_boundary<R>(bc.kind, l, given, n, out, &not_converged);
    } else {
#pragma unroll
      for (int k = 0; k < kK; ++k) out[k] = 0;
    }
#pragma unroll
    for (int k = 0; k < kK; ++k) out[k] *= x.w;
  }
  if (not_converged) atomicOr(&a.state->status, (unsigned)kStatusNotConverged);
  double *dst = a.flux + gid * kK;
#pragma unroll
  for (int k = 0; k < kK; ++k) dst[k] = out[k];
}

struct ModalCellArgs {
  const double *u_in, *u0;
  double *u_out;
  const double *taylor;
  const double *s;
  const double4 *center;
  const int32_t *vol_off;
  const double4 *vol;
  const int32_t *cell_faces;
  const int32_t *face_off;
  const double4 *fpt, *fshift;
  const double *flux;
  DevState *state;
  int64_t n_cells;
  int advance_time;
  CaseView cs;
};

template <int M, int STAGE>
__global__ void __launch_bounds__(ModalCfg<M>::kBlock) modal_cell_kernel(ModalCellArgs a) {
  constexpr int KM = kK * M, NS = M * (M + 1) / 2, kCellBlock = ModalCfg<M>::kBlock;
  extern __shared__ double s_dyn[];  // [KM][block] Taylor coefficients
  const int tid = threadIdx.x;
  const int64_t c = (int64_t)blockIdx.x * kCellBlock + tid;
  if (c >= a.n_cells) return;
  const double *ac = a.taylor + c * KM;
  double rt[kK][M];
  auto coef = [&](int i) -> double { return s_dyn[i * kCellBlock + tid]; };
  auto RT = [&](int k, int j) -> double & { return rt[k][j]; };
#pragma unroll
  for (int i = 0; i < KM; ++i) s_dyn[i * kCellBlock + tid] = ac[i];
#pragma unroll
  for (int k = 0; k < kK; ++k)
#pragma unroll
    for (int j = 0; j < M; ++j) RT(k, j) = 0;
  // volume: sum_q w F(u_q) . grad T(x_q)
  const int q0 = a.vol_off[c], q1 = a.vol_off[c + 1];
  for (int q = q0; q < q1; ++q) {
    const double4 g = a.vol[q];
    double t[M], u[kK];
    taylor_values<M>(g.x, g.y, g.z, t);
#pragma unroll
    for (int k = 0; k < kK; ++k) {
      double s = 0;
#pragma unroll
      for (int j = 0; j < M; ++j) s += coef(j * kK + k) * t[j];
      u[k] = s;
    }
    // GetFluxMatrix (types.hpp:322-333); mass row = momentum, which for a
    // converted state equals rho * velocity
    const Prim w = cons_to_prim(u[0], u[1], u[2], u[3], u[4]);
    const bool converted = w.rho != 0;
    const double vel[3] = {w.u, w.v, w.w};
    double f[kK][3];
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      f[0][d] = converted ? w.rho * vel[d] : u[1 + d];
      f[1][d] = u[1] * vel[d] + (d == 0 ? w.p : 0.0);
      f[2][d] = u[2] * vel[d] + (d == 1 ? w.p : 0.0);
      f[3][d] = u[3] * vel[d] + (d == 2 ? w.p : 0.0);
      f[4][d] = (u[4] + w.p) * vel[d];
    }
#pragma unroll
    for (int k = 0; k < kK; ++k)
      add_gradient<M>(t, f[k][0] * g.w, f[k][1] * g.w, f[k][2] * g.w,
                      [&](int j) -> double & { return RT(k, j); });
  }
  // faces: holder -= w F^ T(x - centre), sharer += w F^ T(x - shift - centre)
  const double4 ctr = a.center[c];
  for (int slot = 0; slot < 6; ++slot) {
    const int code = a.cell_faces[c * 6 + slot];
    if (code < 0) continue;
    const int f = code >> 1;
    const bool sharer = code & 1;
    double4 sh = make_double4(0, 0, 0, 0);
    if (sharer) sh = a.fshift[f];
    const int p0 = a.face_off[f], p1 = a.face_off[f + 1];
    for (int p = p0; p < p1; ++p) {
      const double4 x = a.fpt[p];
      double t[M];
      taylor_values<M>((x.x - sh.x) - ctr.x, (x.y - sh.y) - ctr.y, (x.z - sh.z) - ctr.z, t);
      const double *fl = a.flux + (int64_t)p * kK;
#pragma unroll
      for (int k = 0; k < kK; ++k) {
        const double v = sharer ? fl[k] : -fl[k];
#pragma unroll
        for (int j = 0; j < M; ++j) RT(k, j) += v * t[j];
      }
    }
  }
  // R = S Rt, then the stage combination (temporal/rk.hpp:16-49)
  const double *sc = a.s + c * NS;
  const double *uin = a.u_in + c * KM;
  double *out = a.u_out + c * KM;
  const double dt = STAGE == kStageResidual ? 0.0
                    : (a.cs.dt ? a.cs.dt[a.cs.cell_case[c]] : a.state->dt);
  const double dts = StageCoef<STAGE>::cd * dt;  // the increment's stage weight folded in
  bool bad = false;
#pragma unroll
  for (int m = 0; m < M; ++m) {
    double srow[M];
#pragma unroll
    for (int j = 0; j <= m; ++j) srow[j] = sc[m * (m + 1) / 2 + j];
#pragma unroll
    for (int k = 0; k < kK; ++k) {
      double r = 0;
#pragma unroll
      for (int j = 0; j <= m; ++j) r += srow[j] * RT(k, j);
      double v;
      if (STAGE == kStageResidual) {
        v = r;
      } else if (STAGE == kStageEuler) {
        v = fma(r, dts, uin[m * kK + k]);
      } else {
        v = fma(StageCoef<STAGE>::c0, a.u0[c * KM + m * kK + k],
                fma(StageCoef<STAGE>::cu, uin[m * kK + k], r * dts));
      }
      bad |= !finite64(v);
      out[m * kK + k] = v;
    }
  }
  if (bad) atomicOr(&a.state->status, (unsigned)kStatusNonFinite);
  if (a.advance_time && !a.cs.dt && c == 0) a.state->t += a.state->dt;
}

// max of `rate` into the handle's word, or into each cell's case word (cases
// are contiguous cell runs, so warps are almost always uniform)
__device__ __forceinline__ void reduce_cell_rate(double rate, int64_t c, int64_t n_cells,
                                                 DevState *state, const int32_t *cell_case,
                                                 unsigned long long *case_rate) {
  // (rates are >= 1e-5 / length, or 0 for idle lanes: never negative or NaN)
  block_max_bits(bits64(rate),
                 (case_rate && c < n_cells) ? cell_case[c] : -1, &state->max_rate_bits, case_rate);
}

__device__ __forceinline__ double point_speed(const double *v) {
  const Prim w = cons_to_prim(v[0], v[1], v[2], v[3], v[4]);
  return sound_speed(w) + sqrt(w.u * w.u + w.v * w.v + w.w * w.w);
}

// max over the first M quadrature points of (|u| + c) / length, per cell
// (fem.hpp:417-435 with Projection::GetValue(i), projection.hpp:109-118):
// the value as the reference forms it, c . (S T(x_i - centre))
template <int M>
__global__ void __launch_bounds__(512)
modal_dt_basis_kernel(const double *u, const double *s, const double4 *center,
                      const int32_t *vol_off, const double4 *vol, int64_t n_cells,
                      DevState *state, const int32_t *cell_case, unsigned long long *case_rate) {
  constexpr int KM = kK * M, NS = M * (M + 1) / 2;
  const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  double rate = 0;
  if (c < n_cells) {
    const double *sc = s + c * NS;
    const double *uc = u + c * KM;
    double max_speed = 1e-5;
    const int q0 = vol_off[c];
    for (int i = 0; i < M; ++i) {
      const double4 g = vol[q0 + i];
      double t[M], psi[M], v[kK];
      taylor_values<M>(g.x, g.y, g.z, t);
#pragma unroll
      for (int m = 0; m < M; ++m) {
        double acc = 0;
#pragma unroll
        for (int j = 0; j <= m; ++j) acc += sc[m * (m + 1) / 2 + j] * t[j];
        psi[m] = acc;
      }
#pragma unroll
      for (int k = 0; k < kK; ++k) {
        double acc = 0;
#pragma unroll
        for (int m = 0; m < M; ++m) acc += uc[m * kK + k] * psi[m];
        v[k] = acc;
      }
      max_speed = fmax(max_speed, point_speed(v));
    }
    rate = max_speed * center[c].w;
  }
  reduce_cell_rate(rate, c, n_cells, state, cell_case, case_rate);
}

// The same maximum from the Taylor coefficients a = S^T c of the input:
// u(x_i) = a . T(x_i - centre), reassociated (rounding-level difference).
template <int M>
__global__ void __launch_bounds__(512)
modal_dt_kernel(const double *taylor, const double4 *center,
                const int32_t *vol_off, const double4 *vol, int64_t n_cells,
                DevState *state, const int32_t *cell_case, unsigned long long *case_rate) {
  constexpr int KM = kK * M;
  const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  double rate = 0;
  if (c < n_cells) {
    const double *ac = taylor + c * KM;
    double max_speed = 1e-5;
    const int q0 = vol_off[c];
    for (int i = 0; i < M; ++i) {
      const double4 g = vol[q0 + i];
      double t[M], v[kK];
      taylor_values<M>(g.x, g.y, g.z, t);
      eval_taylor<M>(ac, t, v);
      max_speed = fmax(max_speed, point_speed(v));
    }
    rate = max_speed * center[c].w;
  }
  reduce_cell_rate(rate, c, n_cells, state, cell_case, case_rate);
}

// Projection::Approximate (projection.hpp:28-42): coeff = sum_q (f_q psi(x_q)) w_q
template <int M>
__global__ void __launch_bounds__(256)
modal_project_kernel(const double *values, const double *s, const int32_t *vol_off,
                     const double4 *vol, double *u, int64_t n) {
  constexpr int KM = kK * M, NS = M * (M + 1) / 2;
  int64_t gid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (gid >= n) return;
  const int64_t c = gid / KM;
  const int r = (int)(gid - c * KM), m = r / kK, k = r - m * kK;
  const double *sc = s + c * NS;
  double acc = 0;
  for (int q = vol_off[c]; q < vol_off[c + 1]; ++q) {
    const double4 g = vol[q];
    double t[M];
    taylor_values<M>(g.x, g.y, g.z, t);
    double psi = 0;
    for (int j = 0; j <= m; ++j) psi += sc[m * (m + 1) / 2 + j] * t[j];
    acc += values[(int64_t)q * kK + k] * psi * g.w;
  }
  u[gid] = acc;
}

// ---------------------------------------------------------------------------
// Mixed form: the contractions (Taylor coefficients, values at quadrature
// points, volume flux, residual accumulation, S Rt) in FP32 on FP32 copies of
// S and of the point offsets; FP64 for the face states handed to the Riemann
// solver, the Riemann / boundary flux itself, the positivity decisions of the
// face states and the RK accumulation u + dt R and combinations.  FP64 <-> FP32
// conversions run on the integer pipes (f64_to_f32 / f32_to_f64).

// a32 = S^T c in FP32, one thread per (cell, component)
template <int M>
__global__ void __launch_bounds__(256)
modal_taylor32_kernel(const double *u, const float *s32, float *a32, int64_t n) {
  constexpr int KM = kK * M, NS = M * (M + 1) / 2;
  int64_t gid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (gid >= n) return;
  const int64_t c = gid / kK;
  const int k = (int)(gid - c * kK);
  const double *uc = u + c * KM;
  const float *sc = s32 + c * NS;
  float cf[M];
#pragma unroll
  for (int m = 0; m < M; ++m) cf[m] = f64_to_f32(uc[m * kK + k]);
  float *ac = a32 + c * KM;
#pragma unroll
  for (int j = 0; j < M; ++j) {
    float acc = 0.f;
#pragma unroll
    for (int m = j; m < M; ++m) acc = fmaf(sc[m * (m + 1) / 2 + j], cf[m], acc);
    ac[j * kK + k] = acc;
  }
}

struct ModalFace32Args {
  const float *taylor32;
  const int2 *face_cells;
  const int32_t *face_group;
  const int32_t *point_face;
  const double4 *fpt, *fnrm;
  const float4 *foff32;
  const BcDev *bcs;
  float *flux32;
  DevState *state;
  double stage_c;
  int64_t n_points;
  int n_groups;
  CaseView cs;
  const int32_t *bc_row;  // [points] row in the group's boundary table, or null
};

template <int M, int R>
__global__ void __launch_bounds__(512, R == kHllc ? 2 : 0) modal_face32_kernel(ModalFace32Args a) {
  int64_t gid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (gid >= a.n_points) return;
  const int f = a.point_face[gid];
  const int2 cells = a.face_cells[f];
  const double4 x = a.fpt[gid];
  const double4 nv = a.fnrm[gid];
  const double n[3] = {nv.x, nv.y, nv.z};
  const float4 oh = a.foff32[gid * 2];
  float t[M], v[kK];
  double uh[kK], out[kK];
  taylor_values<M, float>(oh.x, oh.y, oh.z, t);
  eval_taylor<M, float>(a.taylor32 + (int64_t)cells.x * M * kK, t, v);
#pragma unroll
  for (int k = 0; k < kK; ++k) uh[k] = f32_to_f64(v[k]);
  bool not_converged = false;
  if (cells.y >= 0) {
    const float4 os = a.foff32[gid * 2 + 1];
    double us[kK];
    taylor_values<M, float>(os.x, os.y, os.z, t);
    eval_taylor<M, float>(a.taylor32 + (int64_t)cells.y * M * kK, t, v);
#pragma unroll
    for (int k = 0; k < kK; ++k) us[k] = f32_to_f64(v[k]);
    // the point weight folded into the flux (as in modal_face_kernel)
    interior_flux_weighted<R, true>(uh, us, n, x.w, out, &not_converged);
  } else {
    Prim l = cons_to_prim(uh[0], uh[1], uh[2], uh[3], uh[4]);
    const int grp = a.face_group[f];
    if (grp >= 0 && grp < a.n_groups && a.bcs[grp].kind != kBcNone) {
      const BcDev &bc = a.bcs[grp];
      double given[kK];
      double tt = a.state->t + a.stage_c * a.state->dt;
      if (a.cs.t) {
        const int k = a.cs.cell_case[cells.x];
        tt = a.cs.t[k] + a.stage_c * a.cs.dt[k];
      }
      boundary_given(bc, x.x, x.y, x.z, tt, a.bc_row ? a.bc_row[gid] : -1, given);
      flux_boundary<R>(bc.kind, l, given, n, out, &not_converged);
    } else {
#pragma unroll
      for (int k = 0; k < kK; ++k) out[k] = 0;
    }
#pragma unroll
    for (int k = 0; k < kK; ++k) out[k] *= x.w;
  }
  if (not_converged) atomicOr(&a.state->status, (unsigned)kStatusNotConverged);
  float *dst = a.flux32 + gid * kK;
#pragma unroll
  for (int k = 0; k < kK; ++k) dst[k] = f64_to_f32(out[k]);
}

struct ModalCell32Args {
  const double *u_in, *u0;
  double *u_out;
  const float *taylor32;
  const float *s32;
  const int32_t *vol_off;
  const float4 *vol32;
  const int32_t *cell_faces;
  const int32_t *face_off;
  const float4 *foff32;
  const float *flux32;
  DevState *state;
  int64_t n_cells;
  int advance_time;
  CaseView cs;
};

template <int M>
struct ModalCfg32 {
  static constexpr int kBlock = 64;
};

template <int M, int STAGE>
__global__ void __launch_bounds__(ModalCfg32<M>::kBlock) modal_cell32_kernel(ModalCell32Args a) {
  constexpr int KM = kK * M, NS = M * (M + 1) / 2, B = ModalCfg32<M>::kBlock;
  __shared__ float s_a[KM][B];  // thread-private Taylor coefficients
  const int tid = threadIdx.x;
  const int64_t c = (int64_t)blockIdx.x * B + tid;
  if (c >= a.n_cells) return;
  {
    const float *ac = a.taylor32 + c * KM;
#pragma unroll
    for (int i = 0; i < KM; ++i) s_a[i][tid] = ac[i];
  }
  float rt[kK][M];
#pragma unroll
  for (int k = 0; k < kK; ++k)
#pragma unroll
    for (int j = 0; j < M; ++j) rt[k][j] = 0.f;
  // volume: sum_q w F(u_q) . grad T(x_q), all FP32 (types.hpp:288-333 with
  // the positivity clamp)
  const int q0 = a.vol_off[c], q1 = a.vol_off[c + 1];
  for (int q = q0; q < q1; ++q) {
    const float4 g = a.vol32[q];
    float t[M], u[kK];
    taylor_values<M, float>(g.x, g.y, g.z, t);
#pragma unroll
    for (int k = 0; k < kK; ++k) {
      float s = 0.f;
#pragma unroll
      for (int j = 0; j < M; ++j) s = fmaf(s_a[j * kK + k][tid], t[j], s);
      u[k] = s;
    }
    float rho = u[0], vx = u[1], vy = u[2], vz = u[3], p = u[4];
    if (u[0] < 0.f || u[4] < 0.f) {
      rho = vx = vy = vz = p = 0.f;
    } else if (u[0] != 0.f) {
      const float inv = 1.0f / u[0];
      vx = u[1] * inv; vy = u[2] * inv; vz = u[3] * inv;
      p = (u[4] - u[0] * (0.5f * (vx * vx + vy * vy + vz * vz))) * (float)kGm1;
      if (p < 0.f) rho = vx = vy = vz = p = 0.f;
    }
    const bool converted = rho != 0.f;
    const float vel[3] = {vx, vy, vz};
    float f[kK][3];
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      f[0][d] = converted ? rho * vel[d] : u[1 + d];
      f[1][d] = u[1] * vel[d] + (d == 0 ? p : 0.f);
      f[2][d] = u[2] * vel[d] + (d == 1 ? p : 0.f);
      f[3][d] = u[3] * vel[d] + (d == 2 ? p : 0.f);
      f[4][d] = (u[4] + p) * vel[d];
    }
#pragma unroll
    for (int k = 0; k < kK; ++k)
      add_gradient<M, float>(t, f[k][0] * g.w, f[k][1] * g.w, f[k][2] * g.w,
                             [&](int j) -> float & { return rt[k][j]; });
  }
  // faces: holder -= w F^ T, sharer += w F^ T (FP32 lift of the FP64 flux)
  for (int slot = 0; slot < 6; ++slot) {
    const int code = a.cell_faces[c * 6 + slot];
    if (code < 0) continue;
    const int f = code >> 1;
    const int side = code & 1;
    const int p0 = a.face_off[f], p1 = a.face_off[f + 1];
    for (int p = p0; p < p1; ++p) {
      const float4 o = a.foff32[(int64_t)p * 2 + side];
      float t[M];
      taylor_values<M, float>(o.x, o.y, o.z, t);
      const float *fl = a.flux32 + (int64_t)p * kK;
#pragma unroll
      for (int k = 0; k < kK; ++k) {
        const float v = side ? fl[k] : -fl[k];
#pragma unroll
        for (int j = 0; j < M; ++j) rt[k][j] = fmaf(v, t[j], rt[k][j]);
      }
    }
  }
  // R = S Rt in FP32; u + dt R and the RK combinations in FP64
  const float *sc = a.s32 + c * NS;
  const double *uin = a.u_in + c * KM;
  double *out = a.u_out + c * KM;
  const double dt = STAGE == kStageResidual ? 0.0
                    : (a.cs.dt ? a.cs.dt[a.cs.cell_case[c]] : a.state->dt);
  // the increment's stage weight folded in (2/3 rounds to FP32 like the increment)
  const float dt32 = f64_to_f32(dt) * (float)StageCoef<STAGE>::cd;
  bool bad = false;
#pragma unroll
  for (int m = 0; m < M; ++m) {
    float srow[M];
#pragma unroll
    for (int j = 0; j <= m; ++j) srow[j] = sc[m * (m + 1) / 2 + j];
#pragma unroll
    for (int k = 0; k < kK; ++k) {
      float r = 0.f;
#pragma unroll
      for (int j = 0; j <= m; ++j) r = fmaf(srow[j], rt[k][j], r);
      double v;
      if (STAGE == kStageResidual) {
        v = f32_to_f64(r);
      } else if (STAGE == kStageEuler) {
        v = uin[m * kK + k] + f32_to_f64(r * dt32);
      } else {
        v = fma(StageCoef<STAGE>::c0, a.u0[c * KM + m * kK + k],
                fma(StageCoef<STAGE>::cu, uin[m * kK + k], f32_to_f64(r * dt32)));
      }
      bad |= !finite64(v);
      out[m * kK + k] = v;
    }
  }
  if (bad) atomicOr(&a.state->status, (unsigned)kStatusNonFinite);
  if (a.advance_time && !a.cs.dt && c == 0) a.state->t += a.state->dt;
}

// Mixed-form time step: values at the first M quadrature points from the
// FP32 Taylor coefficients, wave speeds in FP32.
template <int M>
__global__ void __launch_bounds__(512)
modal_dt32_kernel(const float *taylor32, const double4 *center, const int32_t *vol_off,
                  const float4 *vol32, int64_t n_cells, DevState *state,
                  const int32_t *cell_case, unsigned long long *case_rate) {
  constexpr int KM = kK * M;
  const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  double rate = 0;
  if (c < n_cells) {
    const float *ac = taylor32 + c * KM;
    float max_speed = 1e-5f;
    const int q0 = vol_off[c];
    for (int i = 0; i < M; ++i) {
      const float4 g = vol32[q0 + i];
      float t[M], v[kK];
      taylor_values<M, float>(g.x, g.y, g.z, t);
      eval_taylor<M, float>(ac, t, v);
      float speed = 0.f;
      if (v[0] > 0.f && v[4] >= 0.f) {
        const float inv = 1.0f / v[0];
        const float uu = (v[1] * v[1] + v[2] * v[2] + v[3] * v[3]) * inv * inv;
        const float pp = (v[4] - 0.5f * v[0] * uu) * (float)kGm1;
        const float cs = pp > 0.f ? sqrtf((float)kGamma * pp * inv) : 0.f;
        speed = pp >= 0.f ? cs + sqrtf(uu) : 0.f;
      } else if (v[0] == 0.f && v[4] >= 0.f) {
        speed = sqrtf(v[1] * v[1] + v[2] * v[2] + v[3] * v[3]);
      }
      max_speed = fmaxf(max_speed, speed);
    }
    rate = (double)max_speed * center[c].w;
  }
  reduce_cell_rate(rate, c, n_cells, state, cell_case, case_rate);
}

template <int M>
int taylor32_launch(mcfd_handle *h, const double *u) {
  const int64_t n = h->mesh.n_cells * kK;
  modal_taylor32_kernel<M><<<(unsigned)((n + 255) / 256), 256, 0, h->stream>>>(
      u, h->modal.s32, h->modal.taylor32, n);
  return 1;
}

template <int M, int R>
void modal_face32_launch(mcfd_handle *h, const ModalFace32Args &fa) {
  const int bs = h->tune.face_block;
  modal_face32_kernel<M, R><<<(unsigned)((fa.n_points + bs - 1) / bs), bs, 0, h->stream>>>(fa);
}

template <int M>
void modal_face32_dispatch(mcfd_handle *h, const ModalFace32Args &fa) {
  switch (h->opt.riemann) {
    case kExact: modal_face32_launch<M, kExact>(h, fa); break;
    case kHllc: modal_face32_launch<M, kHllc>(h, fa); break;
    case kAusm: modal_face32_launch<M, kAusm>(h, fa); break;
    case kRoe: modal_face32_launch<M, kRoe>(h, fa); break;
    default: modal_face32_launch<M, kRusanov>(h, fa); break;
  }
}

template <int M, int S>
void modal_cell32_launch(mcfd_handle *h, const ModalCell32Args &ca) {
  constexpr int B = ModalCfg32<M>::kBlock;
  const int64_t blocks = (ca.n_cells + B - 1) / B;
  modal_cell32_kernel<M, S><<<(unsigned)blocks, B, 0, h->stream>>>(ca);
}

template <int M>
void modal_cell32_dispatch(mcfd_handle *h, int stage, const ModalCell32Args &ca) {
  switch (stage) {
    case kStageEuler: modal_cell32_launch<M, kStageEuler>(h, ca); break;
    case kStageRk2Last: modal_cell32_launch<M, kStageRk2Last>(h, ca); break;
    case kStageRk3Mid: modal_cell32_launch<M, kStageRk3Mid>(h, ca); break;
    case kStageRk3Last: modal_cell32_launch<M, kStageRk3Last>(h, ca); break;
    default: modal_cell32_launch<M, kStageResidual>(h, ca); break;
  }
}

template <int M>
int taylor_launch(mcfd_handle *h, const double *u) {
  const int64_t n = h->mesh.n_cells * kK * (M / 2);  // one thread per row pair
  modal_taylor_kernel<M><<<(unsigned)((n + 255) / 256), 256, 0, h->stream>>>(
      u, h->modal.s, h->modal.taylor, n);
  return 1;
}

template <int M, int R>
void modal_face_launch(mcfd_handle *h, const ModalFaceArgs &fa) {
  const int bs = h->tune.face_block;
  modal_face_kernel<M, R><<<(unsigned)((fa.n_points + bs - 1) / bs), bs, 0, h->stream>>>(fa);
}

template <int M>
void modal_face_dispatch(mcfd_handle *h, const ModalFaceArgs &fa) {
  switch (h->opt.riemann) {
    case kExact: modal_face_launch<M, kExact>(h, fa); break;
    case kHllc: modal_face_launch<M, kHllc>(h, fa); break;
    case kAusm: modal_face_launch<M, kAusm>(h, fa); break;
    case kRoe: modal_face_launch<M, kRoe>(h, fa); break;
    default: modal_face_launch<M, kRusanov>(h, fa); break;
  }
}

template <int M, int S>
void modal_cell_launch(mcfd_handle *h, const ModalCellArgs &ca) {
  constexpr int B = ModalCfg<M>::kBlock, SMEM = ModalCfg<M>::kSmemBytes;
  static_assert(SMEM <= 48 * 1024, "cell kernel shared memory above the default limit");
  const int64_t blocks = (ca.n_cells + B - 1) / B;
  modal_cell_kernel<M, S><<<(unsigned)blocks, B, SMEM, h->stream>>>(ca);
}

template <int M>
void modal_cell_dispatch(mcfd_handle *h, int stage, const ModalCellArgs &ca) {
  switch (stage) {
    case kStageEuler: modal_cell_launch<M, kStageEuler>(h, ca); break;
    case kStageRk2Last: modal_cell_launch<M, kStageRk2Last>(h, ca); break;
    case kStageRk3Mid: modal_cell_launch<M, kStageRk3Mid>(h, ca); break;
    case kStageRk3Last: modal_cell_launch<M, kStageRk3Last>(h, ca); break;
    default: modal_cell_launch<M, kStageResidual>(h, ca); break;
  }
}

// Writer<Part>::Prepare (mesh/vtk.hpp:428-493) for the modal scheme: one
// thread per (cell, VTK node slot); Hex8 cells sample the Hexahedron27
// locals, Tet4 cells the Tetrahedron10 locals (slots 10..26 idle).  Global
// point from the cell's map, value = sum_j a_j T_j(x - centre) with the
// Taylor coefficients a = S^T c (Projection::LocalToGlobalAndValue).
struct ModalSampleArgs {
  const double *taylor;
  const double4 *center;
  const double *corners;
  const uint8_t *type;
  const int64_t *off;
  double *xyz;
  double *values;
  int64_t n_cells;
  int points_given;  // quadratic / wedge cells: xyz holds the points already (host-mapped)
};

template <int M>
__global__ void __launch_bounds__(256) modal_vtk_sample_kernel(ModalSampleArgs a) {
  const int64_t gid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t c = gid / 27;
  const int s = (int)(gid - c * 27);
  if (c >= a.n_cells) return;
  const bool tet = a.type[c] == 1;
  // VTK points per cell: Tetrahedron10, Wedge15 (host-mapped), Hexahedron27
  if (s >= (tet ? 10 : a.type[c] == 2 ? 15 : 27)) return;
  const double *xn = a.corners + c * 24;
  const int64_t pt = a.off[c] + s;
  double g[3];
  if (a.points_given) {
#pragma unroll
    for (int e = 0; e < 3; ++e) g[e] = a.xyz[pt * 3 + e];
  } else if (!tet) {
    const double loc[3] = {(double)kVtkHex27[s][0], (double)kVtkHex27[s][1],
                           (double)kVtkHex27[s][2]};
    g[0] = g[1] = g[2] = 0;
#pragma unroll
    for (int v = 0; v < 8; ++v) {
      const double w = (1 + kVtkHex27[v][0] * loc[0]) * (1 + kVtkHex27[v][1] * loc[1]) *
                       (1 + kVtkHex27[v][2] * loc[2]) * 0.125;
#pragma unroll
      for (int e = 0; e < 3; ++e) g[e] += xn[v * 3 + e] * w;
    }
  } else {
    // Tetrahedron4 shapes (x, y, z, 1 - x - y - z), coordinate/tetrahedron.hpp:98-103
    const double l0 = kVtkTet10Half[s][0] * 0.5, l1 = kVtkTet10Half[s][1] * 0.5,
                 l2 = kVtkTet10Half[s][2] * 0.5;
    const double l3 = 1.0 - l0 - l1 - l2;
#pragma unroll
    for (int e = 0; e < 3; ++e)
      g[e] = xn[e] * l0 + xn[3 + e] * l1 + xn[6 + e] * l2 + xn[9 + e] * l3;
  }
  const double4 ch = a.center[c];
  double t[M], v[kK];
  taylor_values<M>(g[0] - ch.x, g[1] - ch.y, g[2] - ch.z, t);
  eval_taylor<M>(a.taylor + c * M * kK, t, v);
  if (!a.points_given) {
#pragma unroll
    for (int e = 0; e < 3; ++e) a.xyz[pt * 3 + e] = g[e];
  }
#pragma unroll
  for (int e = 0; e < kK; ++e) a.values[pt * kK + e] = v[e];
}

template <int M>
int modal_vtk_launch(mcfd_handle *h, const double *u, const ModalSampleArgs &sa) {
  taylor_launch<M>(h, u);
  const int64_t threads = h->mesh.n_cells * 27;
  modal_vtk_sample_kernel<M><<<(unsigned)((threads + 255) / 256), 256, 0, h->stream>>>(sa);
  return 2;
}

}  // namespace

int launch_modal_vtk_sample(mcfd_handle *h, const double *u, const int64_t *off, double *xyz,
                            double *values) {
  const Modal &md = h->modal;
  ModalSampleArgs sa{md.taylor, md.center, h->mesh.corners, h->mesh.cell_type, off, xyz, values,
                     h->mesh.n_cells, h->mesh.curved ? 1 : 0};
  switch (md.m) {
    case 4: return modal_vtk_launch<4>(h, u, sa);
    case 10: return modal_vtk_launch<10>(h, u, sa);
    default: return modal_vtk_launch<20>(h, u, sa);
  }
}

int launch_modal_face_flux(mcfd_handle *h, const double *u, double stage_c) {
  const Mesh &m = h->mesh;
  const Modal &md = h->modal;
  int n = 0;
  if (h->opt.precision == 1) {
    switch (md.m) {
      case 4: n += taylor32_launch<4>(h, u); break;
      case 10: n += taylor32_launch<10>(h, u); break;
      default: n += taylor32_launch<20>(h, u); break;
    }
    if (md.n_fpts == 0) return n;
    ModalFace32Args fa{md.taylor32, m.face_cells, m.face_group, md.point_face, md.fpt, md.fnrm,
                       md.foff32, m.bcs, reinterpret_cast<float *>(h->buf.flux), h->buf.state,
                       stage_c, md.n_fpts, m.n_groups, case_view(h), m.bc_row};
    switch (md.m) {
      case 4: modal_face32_dispatch<4>(h, fa); break;
      case 10: modal_face32_dispatch<10>(h, fa); break;
      default: modal_face32_dispatch<20>(h, fa); break;
    }
    return n + 1;
  }
  switch (md.m) {
    case 4: n += taylor_launch<4>(h, u); break;
    case 10: n += taylor_launch<10>(h, u); break;
    default: n += taylor_launch<20>(h, u); break;
  }
  if (md.n_fpts == 0) return n;
  ModalFaceArgs fa{md.taylor, md.center, m.face_cells, m.face_group, md.point_face,
                   md.fpt, md.fnrm, md.fshift, m.bcs, h->buf.flux, h->buf.state,
                   stage_c, md.n_fpts, m.n_groups, case_view(h), m.bc_row};
  switch (md.m) {
    case 4: modal_face_dispatch<4>(h, fa); break;
    case 10: modal_face_dispatch<10>(h, fa); break;
    default: modal_face_dispatch<20>(h, fa); break;
  }
  return n + 1;
}

int launch_modal_cell_update(mcfd_handle *h, int stage, const double *u_in,
                             const double *u0, double *u_out, int advance_time) {
  const Modal &md = h->modal;
  if (h->opt.precision == 1) {
    ModalCell32Args ca{u_in, u0, u_out, md.taylor32, md.s32, md.vol_off, md.vol32,
                       md.cell_faces, md.face_off, md.foff32,
                       reinterpret_cast<const float *>(h->buf.flux), h->buf.state,
                       h->mesh.n_cells, advance_time, case_view(h)};
    switch (md.m) {
      case 4: modal_cell32_dispatch<4>(h, stage, ca); break;
      case 10: modal_cell32_dispatch<10>(h, stage, ca); break;
      default: modal_cell32_dispatch<20>(h, stage, ca); break;
    }
    return 1;
  }
  ModalCellArgs ca{u_in, u0, u_out, md.taylor, md.s, md.center, md.vol_off, md.vol,
                   md.cell_faces, md.face_off, md.fpt, md.fshift, h->buf.flux,
                   h->buf.state, h->mesh.n_cells, advance_time, case_view(h)};
  switch (md.m) {
    case 4: modal_cell_dispatch<4>(h, stage, ca); break;
    case 10: modal_cell_dispatch<10>(h, stage, ca); break;
    default: modal_cell_dispatch<20>(h, stage, ca); break;
  }
  return 1;
}

int launch_modal_dt(mcfd_handle *h, const double *u) {
  const Modal &md = h->modal;
  const int64_t C = h->mesh.n_cells;
  const int bs = h->tune.dt_block;
  const unsigned blocks = (unsigned)((C + bs - 1) / bs);
  const int32_t *cc = h->cases.cell_case;
  unsigned long long *cr = h->cases.n ? h->cases.rate : nullptr;
  if (h->opt.precision == 1) {
    int n = 0;
    switch (md.m) {
      case 4: n += taylor32_launch<4>(h, u);
        modal_dt32_kernel<4><<<blocks, bs, 0, h->stream>>>(md.taylor32, md.center, md.vol_off, md.vol32, C, h->buf.state, cc, cr); break;
      case 10: n += taylor32_launch<10>(h, u);
        modal_dt32_kernel<10><<<blocks, bs, 0, h->stream>>>(md.taylor32, md.center, md.vol_off, md.vol32, C, h->buf.state, cc, cr); break;
      default: n += taylor32_launch<20>(h, u);
        modal_dt32_kernel<20><<<blocks, bs, 0, h->stream>>>(md.taylor32, md.center, md.vol_off, md.vol32, C, h->buf.state, cc, cr); break;
    }
    return n + 1 + launch_dt_finalize(h);
  }
  // values at the first M quadrature points: c . psi(x_i) up to M = 10; at
  // M = 20 through the Taylor coefficients (3050 instead of 6200 FMAs per cell)
  switch (md.m) {
    case 4: modal_dt_basis_kernel<4><<<blocks, bs, 0, h->stream>>>(u, md.s, md.center, md.vol_off, md.vol, C, h->buf.state, cc, cr); break;
    case 10: modal_dt_basis_kernel<10><<<blocks, bs, 0, h->stream>>>(u, md.s, md.center, md.vol_off, md.vol, C, h->buf.state, cc, cr); break;
    default:
      taylor_launch<20>(h, u);
      modal_dt_kernel<20><<<blocks, bs, 0, h->stream>>>(md.taylor, md.center, md.vol_off, md.vol, C, h->buf.state, cc, cr);
      return 2 + launch_dt_finalize(h);
  }
  return 1 + launch_dt_finalize(h);
}

int launch_modal_project(mcfd_handle *h, double *u) {
  const Modal &md = h->modal;
  const int64_t n = h->mesh.column;
  const unsigned blocks = (unsigned)((n + 255) / 256);
  switch (md.m) {
    case 4: modal_project_kernel<4><<<blocks, 256, 0, h->stream>>>(md.values, md.s, md.vol_off, md.vol, u, n); break;
    case 10: modal_project_kernel<10><<<blocks, 256, 0, h->stream>>>(md.values, md.s, md.vol_off, md.vol, u, n); break;
    default: modal_project_kernel<20><<<blocks, 256, 0, h->stream>>>(md.values, md.s, md.vol_off, md.vol, u, n); break;
  }
  return 1;
}

}  // namespace mcfd
