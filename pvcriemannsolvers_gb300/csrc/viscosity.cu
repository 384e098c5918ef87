// Energy-based artificial viscosity on fr::Lobatto (Hex8 cells), FP64, on
// sm_103a.
//
//   visc_properties_kernel<Q>  one warp per cell, the cell's nodal block in
//                              shared memory.  UpdateProperties of
//                              EnergyBasedViscosity (spatial/viscosity.hpp:
//                              446-572) for the stage input:
//                              * face jump integral: sum over the cell's
//                                interior face points of (u - u_other)^2 w h
//                                (IntegrateJumpOnFaces, :446-475);
//                              * maximum wave speed and reference squares
//                                over the nodes (:490-503);
//                              * nu_k = 0 and the stable step (:504-536) of
//                                a cell none of whose components has a jump
//                                reaching its reference square; the other
//                                cells go to a work list.
//   visc_rate_kernel<Q>        persistent grid over the work list, one warp
//                              per listed cell: the damping rate
//                              -u_k^T D u_k, where D u is the viscous FR
//                              residual of the cell with nu = 1 and zero
//                              neighbours (BuildDampingMatrices, :299-384),
//                              evaluated matrix-free (no N x N matrix per
//                              cell is stored or read), then nu_k and the
//                              stable step.  Apart from the pass over every
//                              cell so that its registers do not bound that
//                              pass's occupancy.
//   visc_face_kernel<Q>        one thread per face point, after the
//                              convective face kernel: minus nu_avg n .
//                              common_gradient (fr/general.hpp:316-350).  The DDG common
//                              gradient (riemann/diffusive/direct.hpp:45-78)
//                              dotted with the normal needs n . grad(u) and
//                              n^T H n on both sides; with m = J^-T n and a
//                              per-point geometric vector q (the J^-1
//                              derivative term of polynomial/hexahedron.hpp:
//                              495-525), n^T H n = m^T H_loc m + q . g_loc.
//                              They are evaluated only where nu_avg != 0 (the
//                              reference subtracts 0 * flux elsewhere).
//                              No-slip walls subtract nu n . grad(u)
//                              (:460-476); the other boundaries carry no
//                              viscous flux (the Neumann-wall hook returns at
//                              once, spatial/viscosity.hpp:140-147).
//   visc_dt_finalize_kernel    dt = min(2 cfl min_dt, dt_guess)
//                              (with_viscosity.hpp:67-71, fr/lobatto.hpp:431).
//   average_kernel, majority_kernel  the initial limiters of the viscous
//                              demos (limiter/average.hpp, limiter/majority.hpp).
#include <cuda_runtime.h>

#include <algorithm>
#include <climits>
#include <cstdint>

#include "euler.cuh"
#include "handle.hpp"

namespace mcfd {
namespace {

constexpr int kWarps = 4;  // cells (warps) per block of the properties kernel

// axis and orientation of each local hex face (fr/lobatto.hpp:81-152)
__device__ __forceinline__ int side_dir(int side) { return (0x201012 >> (4 * side)) & 0xf; }
__device__ __forceinline__ double side_sign(int side) { return ((0x2c >> side) & 1) ? 1.0 : -1.0; }

struct PropArgs {
  const double *u;
  const double *cell_geo;   // [cells][N][10]: adj(J) row-major, 1/det(J)
  const int32_t *cell_flux; // [cells][6][QF] face-point slots
  const int2 *face_cells;
  const short2 *face_map;
  const double4 *face_geo;  // unit normal, area element |adj(J) e_dir|
  const double *dmat, *d2, *wloc;
  const double *side, *pt, *cell;
  double *nu;
  DevState *state;
  // cells whose jump reaches the reference square: count, cell, and per
  // entry the wave speed, the five jump integrals and the component flags
  unsigned *rate_count;
  int32_t *rate_cell;
  double *rate_data;
  int64_t n_cells;
  double g1, time_scale, spatial_factor;
  int p;
  int dt_mode;
};

// Local gradient g [3][K] and the local second derivatives h [6][K] (XX XY
// XZ YY YZ ZZ) of a nodal block U [N][K] at node (i, j, l).
template <int Q>
__device__ __forceinline__ void local_grad_hess(const double *U, const double *D, const double *D2,
                                                int i, int j, int l, double (&g)[3][kK],
                                                double (&h)[6][kK]) {
#pragma unroll
  for (int k = 0; k < kK; ++k) {
    g[0][k] = g[1][k] = g[2][k] = 0;
    h[0][k] = h[1][k] = h[2][k] = h[3][k] = h[4][k] = h[5][k] = 0;
  }
#pragma unroll
  for (int m = 0; m < Q; ++m) {
    const double dx = D[i * Q + m], dy = D[j * Q + m], dz = D[l * Q + m];
    const double ex = D2[i * Q + m], ey = D2[j * Q + m], ez = D2[l * Q + m];
#pragma unroll
    for (int k = 0; k < kK; ++k) {
      const double ux = U[((m * Q + j) * Q + l) * kK + k];
      const double uy = U[((i * Q + m) * Q + l) * kK + k];
      const double uz = U[((i * Q + j) * Q + m) * kK + k];
      g[0][k] += dx * ux;
      g[1][k] += dy * uy;
      g[2][k] += dz * uz;
      h[0][k] += ex * ux;
      h[3][k] += ey * uy;
      h[5][k] += ez * uz;
    }
#pragma unroll
    for (int n = 0; n < Q; ++n) {
      const double wxy = dx * D[j * Q + n], wxz = dx * D[l * Q + n], wyz = dy * D[l * Q + n];
#pragma unroll
      for (int k = 0; k < kK; ++k) {
        h[1][k] += wxy * U[((m * Q + n) * Q + l) * kK + k];
        h[2][k] += wxz * U[((m * Q + j) * Q + n) * kK + k];
        h[4][k] += wyz * U[((i * Q + m) * Q + n) * kK + k];
      }
    }
  }
}

// n . grad(u_k) = m . g_k and n^T H_k n = m^T h_k m + q . g_k from the side
// vectors sg = (m, q) of a face point side.
__device__ __forceinline__ void normal_traces(const double (&g)[3][kK], const double (&h)[6][kK],
                                              const double *sg, double *s1, double *s2) {
  const double mv[3] = {sg[0], sg[1], sg[2]}, qv[3] = {sg[3], sg[4], sg[5]};
#pragma unroll
  for (int k = 0; k < kK; ++k) {
    s1[k] = mv[0] * g[0][k] + mv[1] * g[1][k] + mv[2] * g[2][k];
    const double hm0 = h[0][k] * mv[0] + h[1][k] * mv[1] + h[2][k] * mv[2];
    const double hm1 = h[1][k] * mv[0] + h[3][k] * mv[1] + h[4][k] * mv[2];
    const double hm2 = h[2][k] * mv[0] + h[4][k] * mv[1] + h[5][k] * mv[2];
    s2[k] = (mv[0] * hm0 + mv[1] * hm1 + mv[2] * hm2) + (qv[0] * g[0][k] + qv[1] * g[1][k] + qv[2] * g[2][k]);
  }
}

// the slots (local face side, point) of node (i, j, l) on the cell surface
template <int Q, class F>
__device__ __forceinline__ void for_slots(int i, int j, int l, F &&fn) {
  if (l == 0) fn(0, i * Q + j);
  if (l == Q - 1) fn(5, i * Q + j);
  if (j == 0) fn(1, i * Q + l);
  if (j == Q - 1) fn(3, i * Q + l);
  if (i == 0) fn(4, j * Q + l);
  if (i == Q - 1) fn(2, j * Q + l);
}

template <int Q>
__global__ void __launch_bounds__(32 * kWarps) visc_properties_kernel(PropArgs a) {
  constexpr int N = Q * Q * Q, QF = Q * Q, KN = kK * N;
  __shared__ double s_u[kWarps][KN];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int64_t c = (int64_t)blockIdx.x * kWarps + warp;
  const bool active = c < a.n_cells;
  if (active)
    for (int e = lane; e < KN; e += 32) s_u[warp][e] = a.u[c * KN + e];
  __syncthreads();
  if (!active) return;
  const double *U = s_u[warp];
  const int32_t *cf = a.cell_flux + c * 6 * QF;
  // cheap pass: wave speeds, reference squares and the face jump integral
  double speed_max = 1e-5, sq_max[kK], jump_acc[kK];
#pragma unroll
  for (int k = 0; k < kK; ++k) {
    sq_max[k] = 1e-5;
    jump_acc[k] = 0;
  }
  for (int q = lane; q < N; q += 32) {
    const double *uq = U + q * kK;
    const Prim w = cons_to_prim(uq[0], uq[1], uq[2], uq[3], uq[4]);
    const double speed = sound_speed(w) + sqrt(w.u * w.u + w.v * w.v + w.w * w.w);
    double sq[kK];
    sq[0] = uq[0] * uq[0];
    sq[4] = uq[4] * uq[4];
    sq[1] = sq[2] = sq[3] = sq[0] * speed * speed;
    speed_max = (speed_max < speed) ? speed : speed_max;
#pragma unroll
    for (int k = 0; k < kK; ++k) sq_max[k] = (sq_max[k] < sq[k]) ? sq[k] : sq_max[k];
    const int i = q / QF, j = (q / Q) % Q, l = q % Q;
    for_slots<Q>(i, j, l, [&](int side, int t) {
      const int32_t v = cf[side * QF + t];
      if (v == INT32_MIN) return;
      const int64_t pt = v >= 0 ? v : ~(int64_t)v;
      const int role = v >= 0 ? 0 : 1;
      const int2 cells = a.face_cells[pt / QF];
      if (cells.y < 0) return;
      const short2 mp = a.face_map[pt];
      const int64_t oc = role == 0 ? cells.y : cells.x;
      const int on = role == 0 ? mp.y : mp.x;
      const double *uo = a.u + oc * KN + on * kK;
      const double wh = a.pt[pt * 4 + 2 + role];
#pragma unroll
      for (int k = 0; k < kK; ++k) {
        double jump = uq[k] - uo[k];
        jump *= jump;
        jump_acc[k] += jump * wh;
      }
    });
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const double sp = __shfl_xor_sync(0xffffffffu, speed_max, o);
    speed_max = (speed_max < sp) ? sp : speed_max;
#pragma unroll
    for (int k = 0; k < kK; ++k) {
      const double sq = __shfl_xor_sync(0xffffffffu, sq_max[k], o);
      sq_max[k] = (sq_max[k] < sq) ? sq : sq_max[k];
      jump_acc[k] += __shfl_xor_sync(0xffffffffu, jump_acc[k], o);
    }
  }
  const double L = a.cell[c * 2], Lp = a.cell[c * 2 + 1];
  // components whose jump reaches the reference square (viscosity.hpp:515)
  unsigned flagged = 0;
#pragma unroll
  for (int k = 0; k < kK; ++k)
    if (!(jump_acc[k] < sq_max[k] * Lp)) flagged |= 1u << k;
  if (lane != 0) return;
  if (flagged) {
    // the damping rate follows in visc_rate_kernel
    const unsigned idx = atomicAdd(a.rate_count, 1u);
    a.rate_cell[idx] = (int32_t)c;
    double *d = a.rate_data + (int64_t)idx * kViscRateData;
    d[0] = speed_max;
#pragma unroll
    for (int k = 0; k < kK; ++k) d[1 + k] = jump_acc[k];
    d[1 + kK] = (double)flagged;
    return;
  }
  const double min_dt = L / speed_max;
#pragma unroll
  for (int k = 0; k < kK; ++k) a.nu[c * kK + k] = 0.0;
  if (a.dt_mode) atomicMin(&a.state->min_dt_bits, bits64(min_dt));
}

// The damping rate, nu and the stable step of the cells that the properties
// kernel listed (a persistent grid, one warp per listed cell at a time).
// Kept apart from the cheap pass so that its register count (the gradient,
// flux and Hessian arrays of the matrix-free rate) does not bound the
// occupancy of the pass over every cell.
template <int Q>
__global__ void __launch_bounds__(32 * kWarps) visc_rate_kernel(PropArgs a) {
  constexpr int N = Q * Q * Q, QF = Q * Q, KN = kK * N;
  __shared__ double s_u[kWarps][KN];
  __shared__ double s_ft[kWarps][3 * kK][N];
  __shared__ double s_d[Q * Q], s_d2[Q * Q], s_w[N];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  for (int e = threadIdx.x; e < Q * Q; e += blockDim.x) {
    s_d[e] = a.dmat[e];
    s_d2[e] = a.d2[e];
  }
  for (int e = threadIdx.x; e < N; e += blockDim.x) s_w[e] = a.wloc[e];
  __syncthreads();
  const unsigned count = *a.rate_count;
  for (unsigned idx = blockIdx.x * kWarps + warp; idx < count; idx += gridDim.x * kWarps) {
    const int64_t c = a.rate_cell[idx];
    for (int e = lane; e < KN; e += 32) s_u[warp][e] = a.u[c * KN + e];
    __syncwarp();
    const double *U = s_u[warp];
    const int32_t *cf = a.cell_flux + c * 6 * QF;
    const double *d = a.rate_data + (int64_t)idx * kViscRateData;
    const double speed_max = d[0];
    double jump_acc[kK];
#pragma unroll
    for (int k = 0; k < kK; ++k) jump_acc[k] = d[1 + k];
    const unsigned flagged = (unsigned)d[1 + kK];
    const double L = a.cell[c * 2];
    double rate_acc[kK];
#pragma unroll
    for (int k = 0; k < kK; ++k) rate_acc[k] = 0;
    // damping rate -u^T D u: D u is the viscous residual of this cell alone
    // (nu = 1, zero neighbours, before the det(J) scaling), weighted by the
    // local GLL weights.  Pass 1: the contravariant flux of -grad(u).
    for (int q = lane; q < N; q += 32) {
      const int i = q / QF, j = (q / Q) % Q, l = q % Q;
      double g[3][kK];
#pragma unroll
      for (int k = 0; k < kK; ++k) g[0][k] = g[1][k] = g[2][k] = 0;
#pragma unroll
      for (int m = 0; m < Q; ++m) {
        const double dx = s_d[i * Q + m], dy = s_d[j * Q + m], dz = s_d[l * Q + m];
#pragma unroll
        for (int k = 0; k < kK; ++k) {
          g[0][k] += dx * U[((m * Q + j) * Q + l) * kK + k];
          g[1][k] += dy * U[((i * Q + m) * Q + l) * kK + k];
          g[2][k] += dz * U[((i * Q + j) * Q + m) * kK + k];
        }
      }
      const double *geo = a.cell_geo + (c * N + q) * 10;
      double A[9];
#pragma unroll
      for (int e = 0; e < 9; ++e) A[e] = geo[e];
      const double inv_det = geo[9];
#pragma unroll
      for (int k = 0; k < kK; ++k) {
        double gu[3];
#pragma unroll
        for (int d = 0; d < 3; ++d)
          gu[d] = inv_det * (A[d * 3 + 0] * g[0][k] + A[d * 3 + 1] * g[1][k] + A[d * 3 + 2] * g[2][k]);
#pragma unroll
        for (int e = 0; e < 3; ++e)
          s_ft[warp][k * 3 + e][q] = -(gu[0] * A[0 * 3 + e] + gu[1] * A[1 * 3 + e] + gu[2] * A[2 * 3 + e]);
      }
    }
    __syncwarp();
    // pass 2: divergence and the lifts of the cell's own face points
    for (int q = lane; q < N; q += 32) {
      const int i = q / QF, j = (q / Q) % Q, l = q % Q;
      double res[kK];
#pragma unroll
      for (int k = 0; k < kK; ++k) {
        double sum = 0;
#pragma unroll
        for (int m = 0; m < Q; ++m) {
          sum -= s_ft[warp][k * 3 + 0][(m * Q + j) * Q + l] * s_d[i * Q + m];
          sum -= s_ft[warp][k * 3 + 1][(i * Q + m) * Q + l] * s_d[j * Q + m];
          sum -= s_ft[warp][k * 3 + 2][(i * Q + j) * Q + m] * s_d[l * Q + m];
        }
        res[k] = sum;
      }
      const bool surface = i == 0 || i == Q - 1 || j == 0 || j == Q - 1 || l == 0 || l == Q - 1;
      if (surface) {
        double g[3][kK], h[6][kK];
        local_grad_hess<Q>(U, s_d, s_d2, i, j, l, g, h);
        for_slots<Q>(i, j, l, [&](int side, int t) {
          const int32_t v = cf[side * QF + t];
          if (v == INT32_MIN) return;
          const int64_t pt = v >= 0 ? v : ~(int64_t)v;
          const int role = v >= 0 ? 0 : 1;
          double s1[kK], s2[kK];
          normal_traces(g, h, a.side + (pt * 2 + role) * 6, s1, s2);
          const double b0d = a.pt[pt * 4 + 0], b1d = a.pt[pt * 4 + 1];
          const double area = a.face_geo[pt].w;
          const int dir = side_dir(side);
          const double sigma = side_sign(side), out_sign = role == 0 ? 1.0 : -1.0;
#pragma unroll
          for (int k = 0; k < kK; ++k) {
            // the other side zero: holder u_s = 0, sharer u_h = 0
            const double uq = U[q * kK + k];
            const double cn = role == 0 ? (0.5 * s1[k] - b0d * uq - b1d * s2[k])
                                        : (0.5 * s1[k] + b0d * uq + b1d * s2[k]);
            const double fup = -cn;
            res[k] -= a.g1 * (out_sign * (fup * area) - sigma * s_ft[warp][k * 3 + dir][q]);
          }
        });
      }
#pragma unroll
      for (int k = 0; k < kK; ++k) rate_acc[k] += (s_w[q] * U[q * kK + k]) * res[k];
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
#pragma unroll
      for (int k = 0; k < kK; ++k) rate_acc[k] += __shfl_xor_sync(0xffffffffu, rate_acc[k], o);
    if (lane == 0) {
    double min_dt = L / speed_max;
    const double max_visc = speed_max * L / a.p;
    const double time_base = L / speed_max;
  #pragma unroll
    for (int k = 0; k < kK; ++k) {
      double val = 0.0;
      if (flagged & (1u << k)) {
        const double rate = -rate_acc[k];
        const double damping_time = time_base * a.time_scale;
        const double ratio = jump_acc[k] / (rate * damping_time);
        const double lo = (0.0 < ratio) ? ratio : 0.0;
        val = (lo < max_visc) ? lo : max_visc;
        const double t1 = L / (speed_max + a.spatial_factor * val / L);
        min_dt = (t1 < min_dt) ? t1 : min_dt;
      }
      a.nu[c * kK + k] = val;
    }
    if (a.dt_mode) atomicMin(&a.state->min_dt_bits, bits64(min_dt));
    }
    __syncwarp();  // s_u and s_ft are rewritten for the next listed cell
  }
}


struct ViscFaceArgs {
  const double *u;
  const int2 *face_cells;
  const int32_t *face_group;
  const double4 *face_geo;
  const short2 *face_map;
  const BcDev *bcs;
  const double *nu, *side, *pt, *dmat, *d2;
  double *flux;  // convective face fluxes (times the area element), corrected in place
  int64_t n_points;
  int n_groups;
};

// n . grad(u_k) and n^T H_k n of component k on one side of a face point,
// from the cell's nodal block in global memory.
template <int Q>
__device__ __forceinline__ void side_trace(const double *uc, int node, int k, const double *sg,
                                           const double *D, const double *D2, double *s1,
                                           double *s2) {
  const int i = node / (Q * Q), j = (node / Q) % Q, l = node % Q;
  double g0 = 0, g1 = 0, g2 = 0, hxx = 0, hxy = 0, hxz = 0, hyy = 0, hyz = 0, hzz = 0;
#pragma unroll
  for (int m = 0; m < Q; ++m) {
    const double ux = uc[((m * Q + j) * Q + l) * kK + k];
    const double uy = uc[((i * Q + m) * Q + l) * kK + k];
    const double uz = uc[((i * Q + j) * Q + m) * kK + k];
    g0 += D[i * Q + m] * ux;
    g1 += D[j * Q + m] * uy;
    g2 += D[l * Q + m] * uz;
    hxx += D2[i * Q + m] * ux;
    hyy += D2[j * Q + m] * uy;
    hzz += D2[l * Q + m] * uz;
#pragma unroll
    for (int n = 0; n < Q; ++n) {
      hxy += (D[i * Q + m] * D[j * Q + n]) * uc[((m * Q + n) * Q + l) * kK + k];
      hxz += (D[i * Q + m] * D[l * Q + n]) * uc[((m * Q + j) * Q + n) * kK + k];
      hyz += (D[j * Q + m] * D[l * Q + n]) * uc[((i * Q + m) * Q + n) * kK + k];
    }
  }
  const double m0 = sg[0], m1 = sg[1], m2 = sg[2];
  *s1 = m0 * g0 + m1 * g1 + m2 * g2;
  const double hm0 = hxx * m0 + hxy * m1 + hxz * m2;
  const double hm1 = hxy * m0 + hyy * m1 + hyz * m2;
  const double hm2 = hxz * m0 + hyz * m1 + hzz * m2;
  *s2 = (m0 * hm0 + m1 * hm1 + m2 * hm2) + (sg[3] * g0 + sg[4] * g1 + sg[5] * g2);
}

// Viscous part of the face fluxes, one thread per face point, after the
// convective kernel: interior points subtract nu_avg n . common_gradient
// (fr/general.hpp:316-350), no-slip walls nu n . grad(u) (:460-476), both
// times the area element.  Points whose viscosity is zero keep the
// convective flux (the reference subtracts 0 there).
template <int Q>
__global__ void __launch_bounds__(256) visc_face_kernel(ViscFaceArgs a) {
  constexpr int QF = Q * Q, KN = kK * Q * Q * Q;
  __shared__ double s_d[Q * Q], s_d2[Q * Q];
  if (threadIdx.x < Q * Q) {
    s_d[threadIdx.x] = a.dmat[threadIdx.x];
    s_d2[threadIdx.x] = a.d2[threadIdx.x];
  }
  __syncthreads();
  const int64_t gid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (gid >= a.n_points) return;
  const int64_t f = gid / QF;
  const int2 cells = a.face_cells[f];
  const double *nh = a.nu + (int64_t)cells.x * kK;
  double prop[kK];
  bool any = false;
  if (cells.y >= 0) {
    const double *ns = a.nu + (int64_t)cells.y * kK;
#pragma unroll
    for (int k = 0; k < kK; ++k) {
      prop[k] = nh[k];
      prop[k] += ns[k];
      prop[k] *= 0.5;
      any = any || prop[k] != 0;
    }
  } else {
    const int grp = a.face_group[f];
    if (!(grp >= 0 && grp < a.n_groups && a.bcs[grp].kind == kBcNoSlipWall)) return;
#pragma unroll
    for (int k = 0; k < kK; ++k) {
      prop[k] = nh[k];
      any = any || prop[k] != 0;
    }
  }
  if (!any) return;
  const short2 map = a.face_map[gid];
  const double area = a.face_geo[gid].w;
  const double *uch = a.u + (int64_t)cells.x * KN;
  const double *sgh = a.side + gid * 12;
  double *d = a.flux + gid * kK;
  if (cells.y >= 0) {
    const double *ucs = a.u + (int64_t)cells.y * KN;
    const double b0d = a.pt[gid * 4 + 0], b1d = a.pt[gid * 4 + 1];
#pragma unroll 1
    for (int k = 0; k < kK; ++k) {
      double th1, th2, ts1, ts2;
      side_trace<Q>(uch, map.x, k, sgh, s_d, s_d2, &th1, &th2);
      side_trace<Q>(ucs, map.y, k, sgh + 6, s_d, s_d2, &ts1, &ts2);
      const double jump = ucs[map.y * kK + k] - uch[map.x * kK + k];
      const double cn = 0.5 * (th1 + ts1) + b0d * jump + b1d * (ts2 - th2);
      d[k] -= (prop[k] * cn) * area;
    }
  } else {
#pragma unroll 1
    for (int k = 0; k < kK; ++k) {
      double th1, th2;
      side_trace<Q>(uch, map.x, k, sgh, s_d, s_d2, &th1, &th2);
      d[k] -= (prop[k] * th1) * area;
    }
  }
}

__global__ void visc_dt_finalize_kernel(DevState *state) {
  const double min_dt = __longlong_as_double((long long)state->min_dt_bits);
  const double dt = (2 * state->cfl) * min_dt;
  state->dt = fmin(dt, state->dt_guess);
  state->min_dt_bits = (unsigned long long)__double_as_longlong(1.e+100);
}

// limiter::average::Reconstruct: every node takes the cell average
// sum_q u_q w_q / sum_q w_q (global weights w_q).  One thread per cell and
// component.
__global__ void average_kernel(double *u, const double *node_w, int64_t n_cells, int n) {
  const int64_t gid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (gid >= n_cells * kK) return;
  const int64_t c = gid / kK;
  const int k = (int)(gid - c * kK);
  double *uc = u + c * n * kK;
  const double *w = node_w + c * n;
  double avg = 0, vol = 0;
  for (int q = 0; q < n; ++q) avg += uc[q * kK + k] * w[q];
  for (int q = 0; q < n; ++q) vol += w[q];
  avg /= vol;
  for (int q = 0; q < n; ++q) uc[q * kK + k] = avg;
}

// limiter::majority::Reconstruct: per component the value that first holds
// a strict majority of the nodes in node order; a cell with a component
// without one stays unchanged and is counted.  One thread per cell.
__global__ void majority_kernel(double *u, int64_t n_cells, int n, unsigned long long *missing) {
  const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= n_cells) return;
  double *uc = u + c * n * kK;
  double value[kK];
  bool all = true;
  for (int k = 0; k < kK; ++k) {
    bool found = false;
    for (int q = 0; q < n && !found; ++q) {
      const double val = uc[q * kK + k];
      int count = 0;
      for (int e = 0; e <= q; ++e) count += (uc[e * kK + k] == val);
      if (count * 2 > n) {
        value[k] = val;
        found = true;
      }
    }
    all = all && found;
  }
  if (!all) {
    atomicAdd(missing, 1ull);
    return;
  }
  for (int q = 0; q < n; ++q)
    for (int k = 0; k < kK; ++k) uc[q * kK + k] = value[k];
}

template <int Q>
int props_launch(mcfd_handle *h, const PropArgs &pa) {
  const unsigned blocks = (unsigned)((pa.n_cells + kWarps - 1) / kWarps);
  cudaMemsetAsync(pa.rate_count, 0, sizeof(unsigned), h->stream);
  visc_properties_kernel<Q><<<blocks, 32 * kWarps, 0, h->stream>>>(pa);
  // persistent grid of the rate kernel: the blocks that fit on the device at once
  const unsigned grid = (unsigned)std::min<int64_t>(blocks, h->visc.rate_blocks);
  visc_rate_kernel<Q><<<grid, 32 * kWarps, 0, h->stream>>>(pa);
  return 2;
}

template <int Q>
int rate_blocks_per_sm() {
  int per_sm = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, visc_rate_kernel<Q>, 32 * kWarps, 0) !=
      cudaSuccess)
    return 1;
  return std::max(per_sm, 1);
}

template <int Q>
int visc_face_launch(mcfd_handle *h, const ViscFaceArgs &fa) {
  const unsigned blocks = (unsigned)((fa.n_points + 255) / 256);
  visc_face_kernel<Q><<<blocks, 256, 0, h->stream>>>(fa);
  return 1;
}

double spatial_factor(int p) {
  // EnergyBasedViscosity::GetSpatialFactor (spatial/viscosity.hpp:581-601)
  static const double kF[7] = {1., 4., 10., 40., 28., 50., 90.};
  return (p >= 0 && p < 7) ? kF[p] : -1;
}

}  // namespace

int visc_rate_blocks_per_sm(int q) {
  switch (q) {
    case 2: return rate_blocks_per_sm<2>();
    case 3: return rate_blocks_per_sm<3>();
    default: return rate_blocks_per_sm<4>();
  }
}

int launch_visc_properties(mcfd_handle *h, const double *u, int dt_mode) {
  const Mesh &m = h->mesh;
  const Visc &v = h->visc;
  PropArgs pa{u, m.cell_geo, m.cell_flux, m.face_cells, m.face_map, m.face_geo,
              m.dmat, v.d2, v.wloc, v.side, v.pt, v.cell, v.nu, h->buf.state,
              v.rate_count, v.rate_cell, v.rate_data, m.n_cells, h->opt.fr_g1, v.time_scale, spatial_factor(m.p), m.p, dt_mode};
  switch (m.q) {
    case 2: return props_launch<2>(h, pa);
    case 3: return props_launch<3>(h, pa);
    default: return props_launch<4>(h, pa);
  }
}

int launch_visc_face_flux(mcfd_handle *h, const double *u) {
  const Mesh &m = h->mesh;
  if (m.n_points == 0) return 0;
  const Visc &v = h->visc;
  ViscFaceArgs fa{u, m.face_cells, m.face_group, m.face_geo, m.face_map, m.bcs,
                  v.nu, v.side, v.pt, m.dmat, v.d2, h->buf.flux, m.n_points, m.n_groups};
  switch (m.q) {
    case 2: return visc_face_launch<2>(h, fa);
    case 3: return visc_face_launch<3>(h, fa);
    default: return visc_face_launch<4>(h, fa);
  }
}

int launch_visc_dt_finalize(mcfd_handle *h) {
  visc_dt_finalize_kernel<<<1, 1, 0, h->stream>>>(h->buf.state);
  return 1;
}

int launch_initial_limiter(mcfd_handle *h, int kind, double *u, unsigned long long *missing) {
  const Mesh &m = h->mesh;
  if (kind == 1) {
    const int64_t threads = m.n_cells * kK;
    average_kernel<<<(unsigned)((threads + 255) / 256), 256, 0, h->stream>>>(u, m.node_w, m.n_cells, m.n);
    return 1;
  }
  majority_kernel<<<(unsigned)((m.n_cells + 127) / 128), 128, 0, h->stream>>>(u, m.n_cells, m.n, missing);
  return 1;
}

}  // namespace mcfd
