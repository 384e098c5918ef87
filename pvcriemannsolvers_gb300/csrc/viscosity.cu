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
//                              * damping rate -u_k^T D u_k, where D u is the
//                                viscous FR residual of the cell with nu = 1
//                                and zero neighbours (BuildDampingMatrices,
//                                :299-384) evaluated matrix-free: no N x N
//                                matrix per cell is stored or read;
//                              * nu_k and the stable step (:504-536).
//                              It also writes, for every face point side of
//                              the cell, n . grad(u_k) and n^T H_k n, the two
//                              numbers the DDG common gradient needs
//                              (riemann/diffusive/direct.hpp:45-78) once it
//                              is dotted with the normal: n^T H n =
//                              m^T H_loc m + q . g_loc with m = J^-T n and q
//                              a per-point geometric vector (the J^-1
//                              derivative term of polynomial/hexahedron.hpp:
//                              495-525).
//   visc_face_kernel<Q, R>     one thread per face point: convective Riemann
//                              flux minus nu_avg n . common_gradient
//                              (fr/general.hpp:316-350); no-slip walls
//                              subtract nu n . grad(u) (:460-476); the other
//                              boundaries carry no viscous flux (the
//                              Neumann-wall hook returns at once, spatial/
//                              viscosity.hpp:140-147).
//   visc_dt_finalize_kernel    dt = min(2 cfl min_dt, dt_guess)
//                              (with_viscosity.hpp:67-71, fr/lobatto.hpp:431).
//   average_kernel, majority_kernel  the initial limiters of the viscous
//                              demos (limiter/average.hpp, limiter/majority.hpp).
#include <cuda_runtime.h>

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
  double *trace;
  DevState *state;
  int64_t n_cells;
  double g1, time_scale, spatial_factor;
  int p;
  int dt_mode;
};

template <int Q>
__global__ void __launch_bounds__(32 * kWarps) visc_properties_kernel(PropArgs a) {
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
  const int64_t c = (int64_t)blockIdx.x * kWarps + warp;
  const bool active = c < a.n_cells;
  if (active)
    for (int e = lane; e < KN; e += 32) s_u[warp][e] = a.u[c * KN + e];
  __syncthreads();
  if (!active) return;
  const double *U = s_u[warp];
  // pass 1: wave speeds, reference squares and the contravariant flux of
  // -grad(u) (the viscous flux with nu = 1) at every node
  double speed_max = 1e-5, sq_max[kK];
#pragma unroll
  for (int k = 0; k < kK; ++k) sq_max[k] = 1e-5;
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
  // pass 2: divergence, face traces, lifts of the isolated cell, jump
  // integral and the per-component damping sums
  double rate_acc[kK], jump_acc[kK];
#pragma unroll
  for (int k = 0; k < kK; ++k) rate_acc[k] = jump_acc[k] = 0;
  const int32_t *cf = a.cell_flux + c * 6 * QF;
  for (int q = lane; q < N; q += 32) {
    const int i = q / QF, j = (q / Q) % Q, l = q % Q;
    double res[kK];
#pragma unroll
    for (int k = 0; k < kK; ++k) {
      double s = 0;
#pragma unroll
      for (int m = 0; m < Q; ++m) {
        s -= s_ft[warp][k * 3 + 0][(m * Q + j) * Q + l] * s_d[i * Q + m];
        s -= s_ft[warp][k * 3 + 1][(i * Q + m) * Q + l] * s_d[j * Q + m];
        s -= s_ft[warp][k * 3 + 2][(i * Q + j) * Q + m] * s_d[l * Q + m];
      }
      res[k] = s;
    }
    const bool surface = i == 0 || i == Q - 1 || j == 0 || j == Q - 1 || l == 0 || l == Q - 1;
    if (surface) {
      // local gradient and Hessian (XX XY XZ YY YZ ZZ) at the node
      double g[3][kK], h[6][kK];
#pragma unroll
      for (int k = 0; k < kK; ++k) {
        g[0][k] = g[1][k] = g[2][k] = 0;
        h[0][k] = h[1][k] = h[2][k] = h[3][k] = h[4][k] = h[5][k] = 0;
      }
#pragma unroll
      for (int m = 0; m < Q; ++m) {
        const double dx = s_d[i * Q + m], dy = s_d[j * Q + m], dz = s_d[l * Q + m];
        const double ex = s_d2[i * Q + m], ey = s_d2[j * Q + m], ez = s_d2[l * Q + m];
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
          const double wxy = dx * s_d[j * Q + n], wxz = dx * s_d[l * Q + n], wyz = dy * s_d[l * Q + n];
#pragma unroll
          for (int k = 0; k < kK; ++k) {
            h[1][k] += wxy * U[((m * Q + n) * Q + l) * kK + k];
            h[2][k] += wxz * U[((m * Q + j) * Q + n) * kK + k];
            h[4][k] += wyz * U[((i * Q + m) * Q + n) * kK + k];
          }
        }
      }
      auto slot = [&](int side, int t) {
        const int32_t v = cf[side * QF + t];
        if (v == INT32_MIN) return;
        const int64_t p = v >= 0 ? v : ~(int64_t)v;
        const int role = v >= 0 ? 0 : 1;
        const double *sg = a.side + (p * 2 + role) * 6;
        const double mv[3] = {sg[0], sg[1], sg[2]}, qv[3] = {sg[3], sg[4], sg[5]};
        const double *pp = a.pt + p * 4;
        const double b0d = pp[0], b1d = pp[1], wh = pp[2 + role];
        const double area = a.face_geo[p].w;
        const int dir = side_dir(side);
        const double sigma = side_sign(side), out_sign = role == 0 ? 1.0 : -1.0;
        double *tr = a.trace + (p * 2 + role) * 2 * kK;
#pragma unroll
        for (int k = 0; k < kK; ++k) {
          const double s1 = mv[0] * g[0][k] + mv[1] * g[1][k] + mv[2] * g[2][k];
          const double hm0 = h[0][k] * mv[0] + h[1][k] * mv[1] + h[2][k] * mv[2];
          const double hm1 = h[1][k] * mv[0] + h[3][k] * mv[1] + h[4][k] * mv[2];
          const double hm2 = h[2][k] * mv[0] + h[4][k] * mv[1] + h[5][k] * mv[2];
          const double s2 = (mv[0] * hm0 + mv[1] * hm1 + mv[2] * hm2) +
                            (qv[0] * g[0][k] + qv[1] * g[1][k] + qv[2] * g[2][k]);
          tr[k] = s1;
          tr[kK + k] = s2;
          // the other side zero: holder u_s = 0, sharer u_h = 0
          const double uq = U[q * kK + k];
          const double cn = role == 0 ? (0.5 * s1 - b0d * uq - b1d * s2)
                                      : (0.5 * s1 + b0d * uq + b1d * s2);
          const double fup = -cn;
          res[k] -= a.g1 * (out_sign * (fup * area) - sigma * s_ft[warp][k * 3 + dir][q]);
        }
        const int2 cells = a.face_cells[p / QF];
        if (cells.y >= 0) {
          const short2 mp = a.face_map[p];
          const int64_t oc = role == 0 ? cells.y : cells.x;
          const int on = role == 0 ? mp.y : mp.x;
          const double *uo = a.u + oc * KN + on * kK;
#pragma unroll
          for (int k = 0; k < kK; ++k) {
            double jump = U[q * kK + k] - uo[k];
            jump *= jump;
            jump_acc[k] += jump * wh;
          }
        }
      };
      if (l == 0) slot(0, i * Q + j);
      if (l == Q - 1) slot(5, i * Q + j);
      if (j == 0) slot(1, i * Q + l);
      if (j == Q - 1) slot(3, i * Q + l);
      if (i == 0) slot(4, j * Q + l);
      if (i == Q - 1) slot(2, j * Q + l);
    }
#pragma unroll
    for (int k = 0; k < kK; ++k) rate_acc[k] += (s_w[q] * U[q * kK + k]) * res[k];
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const double sp = __shfl_xor_sync(0xffffffffu, speed_max, o);
    speed_max = (speed_max < sp) ? sp : speed_max;
#pragma unroll
    for (int k = 0; k < kK; ++k) {
      const double sq = __shfl_xor_sync(0xffffffffu, sq_max[k], o);
      sq_max[k] = (sq_max[k] < sq) ? sq : sq_max[k];
      rate_acc[k] += __shfl_xor_sync(0xffffffffu, rate_acc[k], o);
      jump_acc[k] += __shfl_xor_sync(0xffffffffu, jump_acc[k], o);
    }
  }
  if (lane != 0) return;
  const double L = a.cell[c * 2], Lp = a.cell[c * 2 + 1];
  double min_dt = L / speed_max;
  const double max_visc = speed_max * L / a.p;
  const double time_base = L / speed_max;
#pragma unroll
  for (int k = 0; k < kK; ++k) {
    const double ref = sq_max[k] * Lp;
    double val = 0.0;
    if (!(jump_acc[k] < ref)) {
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
  if (a.dt_mode) atomicMin(&a.state->min_dt_bits, (unsigned long long)__double_as_longlong(min_dt));
}

struct ViscFaceArgs {
  const double *u;
  const int2 *face_cells;
  const int32_t *face_group;
  const double4 *face_geo;
  const double *face_xyz;
  const short2 *face_map;
  const BcDev *bcs;
  const double *nu, *trace, *pt;
  double *flux;
  DevState *state;
  double stage_c;
  int64_t n_points;
  int n_groups;
};

template <int Q, int R>
__global__ void __launch_bounds__(256) visc_face_kernel(ViscFaceArgs a) {
  constexpr int QF = Q * Q, KN = kK * Q * Q * Q;
  const int64_t gid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (gid >= a.n_points) return;
  const int64_t f = gid / QF;
  const int2 cells = a.face_cells[f];
  const short2 map = a.face_map[gid];
  const double4 g = a.face_geo[gid];
  const double n[3] = {g.x, g.y, g.z};
  const double *uh = a.u + (int64_t)cells.x * KN + map.x * kK;
  double ch[kK];
#pragma unroll
  for (int k = 0; k < kK; ++k) ch[k] = uh[k];
  const Prim l = cons_to_prim(ch[0], ch[1], ch[2], ch[3], ch[4]);
  const double *th = a.trace + gid * 4 * kK;
  double out[kK];
  bool not_converged = false;
  if (cells.y >= 0) {
    const double *us = a.u + (int64_t)cells.y * KN + map.y * kK;
    double cs[kK];
#pragma unroll
    for (int k = 0; k < kK; ++k) cs[k] = us[k];
    const Prim r = cons_to_prim(cs[0], cs[1], cs[2], cs[3], cs[4]);
    flux_upwind<R>(l, r, n, out, &not_converged);
    const double *ts = th + 2 * kK;
    const double b0d = a.pt[gid * 4 + 0], b1d = a.pt[gid * 4 + 1];
    const double *nh = a.nu + (int64_t)cells.x * kK, *ns = a.nu + (int64_t)cells.y * kK;
#pragma unroll
    for (int k = 0; k < kK; ++k) {
      const double cn = 0.5 * (th[k] + ts[k]) + b0d * (cs[k] - ch[k]) + b1d * (ts[kK + k] - th[kK + k]);
      double prop = nh[k];
      prop += ns[k];
      prop *= 0.5;
      out[k] -= prop * cn;
    }
  } else {
    const int grp = a.face_group[f];
    if (grp >= 0 && grp < a.n_groups && a.bcs[grp].kind != kBcNone) {
      const BcDev &bc = a.bcs[grp];
      if (bc.kind == kBcNoSlipWall) {
        flux_boundary<R>(kBcInviscidWall, l, ch, n, out, &not_converged);
        const double *nh = a.nu + (int64_t)cells.x * kK;
#pragma unroll
        for (int k = 0; k < kK; ++k) out[k] -= nh[k] * th[k];
      } else {
        const double t = a.state->t + a.stage_c * a.state->dt;
        double given[kK];
        const double *x = a.face_xyz + gid * 3;
        const double *src = bc.a;
        if (bc.program == 1 && (x[bc.axis] - bc.speed * t) >= bc.position) src = bc.b;
#pragma unroll
        for (int k = 0; k < kK; ++k) given[k] = src[k];
        flux_boundary<R>(bc.kind, l, given, n, out, &not_converged);
      }
    } else {
      // no boundary condition: no correction (the FR lift skips NaN fluxes)
#pragma unroll
      for (int k = 0; k < kK; ++k) out[k] = 0;
      out[0] = __longlong_as_double(0x7ff8dead0000beefll);
    }
  }
  if (not_converged) atomicOr(&a.state->status, (unsigned)kStatusNotConverged);
  double *d = a.flux + gid * kK;
#pragma unroll
  for (int k = 0; k < kK; ++k) d[k] = out[k] * g.w;
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
  visc_properties_kernel<Q><<<blocks, 32 * kWarps, 0, h->stream>>>(pa);
  return 1;
}

template <int Q, int R>
int visc_face_launch(mcfd_handle *h, const ViscFaceArgs &fa) {
  const unsigned blocks = (unsigned)((fa.n_points + 255) / 256);
  visc_face_kernel<Q, R><<<blocks, 256, 0, h->stream>>>(fa);
  return 1;
}

template <int Q>
int visc_face_dispatch(mcfd_handle *h, const ViscFaceArgs &fa) {
  switch (h->opt.riemann) {
    case kExact: return visc_face_launch<Q, kExact>(h, fa);
    case kHllc: return visc_face_launch<Q, kHllc>(h, fa);
    case kAusm: return visc_face_launch<Q, kAusm>(h, fa);
    case kRoe: return visc_face_launch<Q, kRoe>(h, fa);
    default: return visc_face_launch<Q, kRusanov>(h, fa);
  }
}

double spatial_factor(int p) {
  // EnergyBasedViscosity::GetSpatialFactor (spatial/viscosity.hpp:581-601)
  static const double kF[7] = {1., 4., 10., 40., 28., 50., 90.};
  return (p >= 0 && p < 7) ? kF[p] : -1;
}

}  // namespace

int launch_visc_properties(mcfd_handle *h, const double *u, int dt_mode) {
  const Mesh &m = h->mesh;
  const Visc &v = h->visc;
  PropArgs pa{u, m.cell_geo, m.cell_flux, m.face_cells, m.face_map, m.face_geo,
              m.dmat, v.d2, v.wloc, v.side, v.pt, v.cell, v.nu, v.trace, h->buf.state,
              m.n_cells, h->opt.fr_g1, v.time_scale, spatial_factor(m.p), m.p, dt_mode};
  switch (m.q) {
    case 2: return props_launch<2>(h, pa);
    case 3: return props_launch<3>(h, pa);
    default: return props_launch<4>(h, pa);
  }
}

int launch_visc_face_flux(mcfd_handle *h, const double *u, double stage_c) {
  const Mesh &m = h->mesh;
  if (m.n_points == 0) return 0;
  const Visc &v = h->visc;
  ViscFaceArgs fa{u, m.face_cells, m.face_group, m.face_geo, m.face_xyz, m.face_map, m.bcs,
                  v.nu, v.trace, v.pt, h->buf.flux, h->buf.state, stage_c, m.n_points, m.n_groups};
  switch (m.q) {
    case 2: return visc_face_dispatch<2>(h, fa);
    case 3: return visc_face_dispatch<3>(h, fa);
    default: return visc_face_dispatch<4>(h, fa);
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
