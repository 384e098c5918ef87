// WENO limiter on DGSEM cells (limiter/weno.hpp, limiter/reconstruct.hpp,
// polynomial/extrapolation.hpp), FP64, for sm_103a.
//
// A limiter pass runs two kernels over the solution buffer:
//   weno_modal_kernel        one thread per (cell, component, mode): the modal
//                            coefficients of every cell, modal = nodal x
//                            modal_to_nodal (UpdateModalCoeff).
//   weno_reconstruct_kernel  one 64-thread block per cell: the jump detector
//                            (DETECT_LAZY), then the Lazy reconstruction —
//                            neighbour polynomials projected onto the cell's
//                            basis through precomputed M x M matrices (the
//                            reference evaluates the neighbour at the cell's
//                            quadrature points and projects; the map is linear
//                            in the neighbour's coefficients, so it is one
//                            matrix per face), offset to the cell's average,
//                            smoothness indicators as quadratic forms of the
//                            modal coefficients (the reference integrates
//                            squared partial derivatives; same quadratic form),
//                            nonlinear weights, and the new nodal values
//                            (UpdateNodalCoeff), written in place.
// MODE 3 (weno::Eigen, limiter/weno.hpp:259-348) reconstructs characteristic-
// wise instead: for every adjacent face the candidates are mapped by L of the
// Euler eigen-system at the cell average in the face's frame (first quadrature
// point, rotated/euler.hpp:330-338), weighted per characteristic field, mapped
// back by R, and the face results are averaged with the neighbours' volumes.
// Every cell reads the modal buffer only, so the in-place write is safe and
// the pass is Jacobi-like, as in limiter::Reconstruct (all new projections
// are computed before any is written back).
// The modal scheme (WithLimiter<dg::General> over Projection, the reference's
// DGFEM build) runs the same kernels on the cells' own orthonormal bases: its
// column already holds the modal coefficients ([M][K] per cell), so
// weno_transpose_kernel replaces the nodal -> modal product and the
// reconstruction writes the new coefficients back in the column's order
// (MODAL); the tables come from each cell's own volume quadrature, for every
// cell type (hexahedra, tetrahedra, wedges, pyramids, curved or straight).
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>

#include "euler.cuh"
#include "handle.hpp"

namespace mcfd {
namespace {

struct WenoArgs {
  double *u;
  const double *modal;
  const double *psi;
  const double *proj;
  const double *beta;
  const double *eval;
  const double *s00;
  const double *divisor;
  const int32_t *adj;
  const double *frame;   // [cells][6][9] face frame at its first point (MODE 3)
  const double *volume;  // [cells] (MODE 3)
  unsigned long long *troubled;
  int64_t n_cells;
  double w0, eps, smooth_ref;
  double *trace;   // node traces of u to rewrite for the reconstructed cells, or null
  int trace_fast;  // the mixed form's seeded roots in the traces
  int trace_roe;   // third trace entry sqrt(rho) (Roe), else the sound speed
  uint8_t *cell_hot;  // per cell the detector's flag (FP64 shock cells), or null
};

// FP64 shock cells of the mixed form: a cell is hot when it or a face
// neighbour was flagged (one layer); with two layers, when it or a face
// neighbour is hot after the first.  A block of the cell kernel is hot when
// one of its cells is.
__global__ void __launch_bounds__(256)
weno_dilate_kernel(const int32_t *__restrict__ adj, const uint8_t *__restrict__ in,
                   uint8_t *__restrict__ out, int64_t n_cells) {
  const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= n_cells) return;
  bool hot = in[c] != 0;
#pragma unroll
  for (int s = 0; s < 6; ++s) {
    const int b = adj[c * 6 + s];
    hot |= b >= 0 && in[b] != 0;
  }
  out[c] = hot ? 1 : 0;
}

__global__ void __launch_bounds__(256)
weno_mark_blocks_kernel(const int32_t *__restrict__ adj, const uint8_t *__restrict__ cell_hot,
                        uint8_t *__restrict__ block_hot, int64_t n_cells, int cells_per_block) {
  const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= n_cells) return;
  bool hot = cell_hot[c] != 0;
#pragma unroll
  for (int s = 0; s < 6; ++s) {
    const int b = adj[c * 6 + s];
    hot |= b >= 0 && cell_hot[b] != 0;
  }
  if (hot) block_hot[c / cells_per_block] = 1;
}

// one thread per (cell, mode): all five components, so each modal_to_nodal
// entry is loaded once.  RHO_E: density and energy only (the jump detector's
// inputs); the momenta of the cells that a reconstruction reads follow in
// weno_modal_momenta_kernel once the troubled cells are known.
template <int N, int M, bool RHO_E = false>
__global__ void __launch_bounds__(256)
weno_modal_kernel(const double *__restrict__ u, const double *__restrict__ mn,
                  double *__restrict__ modal, int64_t n_cells) {
  int64_t gid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (gid >= n_cells * M) return;
  const int64_t c = gid / M;
  const int m = (int)(gid - c * M);
  const double *uc = u + c * kK * N;
  const double *mc = mn + c * N * M;
  double s[kK] = {0, 0, 0, 0, 0};
#pragma unroll 3
  for (int q = 0; q < N; ++q) {
    const double w = mc[q * M + m];
#pragma unroll
    for (int k = 0; k < kK; ++k)
      if (!RHO_E || k == 0 || k == kK - 1) s[k] += uc[q * kK + k] * w;
  }
#pragma unroll
  for (int k = 0; k < kK; ++k)
    if (!RHO_E || k == 0 || k == kK - 1) modal[(c * kK + k) * M + m] = s[k];
}

// The momenta's modal coefficients of every troubled cell and of its face
// neighbours (the reconstruction's candidates), after the detector: a
// grid-stride loop over (troubled cell, slot 0..5 neighbour or 6 own, mode).
// A cell next to several troubled cells is computed once per such cell, each
// time to the same values.
template <int N, int M>
__global__ void __launch_bounds__(256)
weno_modal_momenta_kernel(const double *__restrict__ u, const double *__restrict__ mn,
                          double *__restrict__ modal, const int32_t *__restrict__ adj,
                          const int32_t *__restrict__ list, const unsigned *count) {
  const int64_t n_items = (int64_t)*count * 7 * M;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n_items;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t l = i / (7 * M);
    const int r = (int)(i - l * 7 * M), slot = r / M, m = r - slot * M;
    const int64_t own = list[l];
    const int64_t c = slot == 6 ? own : adj[own * 6 + slot];
    if (c < 0) continue;
    const double *uc = u + c * kK * N;
    const double *mc = mn + c * N * M;
    double s[3] = {0, 0, 0};
#pragma unroll 3
    for (int q = 0; q < N; ++q) {
      const double w = mc[q * M + m];
#pragma unroll
      for (int d = 0; d < 3; ++d) s[d] += uc[q * kK + 1 + d] * w;
    }
#pragma unroll
    for (int d = 0; d < 3; ++d) modal[(c * kK + 1 + d) * M + m] = s[d];
  }
}

// Modal scheme: modal[c][k][m] = column[c][m][k], one thread per (cell, mode).
template <int M>
__global__ void __launch_bounds__(256)
weno_transpose_kernel(const double *__restrict__ u, double *__restrict__ modal, int64_t n_cells) {
  const int64_t gid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (gid >= n_cells * M) return;
  const int64_t c = gid / M;
  const int m = (int)(gid - c * M);
  const double *src = u + gid * kK;
#pragma unroll
  for (int k = 0; k < kK; ++k) modal[(c * kK + k) * M + m] = src[k];
}

// Mixed form: the momenta's product in FP32, density and energy in FP64.
// The jump detector reads only density and energy, so its decisions are the
// FP64 form's; the momenta enter only the reconstruction of troubled cells.
// A block holds CB cells: their nodal momenta are converted to FP32 once into
// shared memory (integer-pipe conversions), then one thread per (cell, mode)
// accumulates them with FP32 FMAs over the FP32 copy of the table, and
// density and energy with FP64 FMAs over the FP64 table; all coefficients
// are stored in FP64.
template <int N, int M>
struct Modal32Cfg {
  static constexpr int kCells = M >= 20 ? 16 : 32;
  static constexpr int kThreads = kCells * M;
};

template <int N, int M>
__global__ void __launch_bounds__(Modal32Cfg<N, M>::kThreads)
weno_modal32_kernel(const double *__restrict__ u, const double *__restrict__ mn,
                    const float *__restrict__ mn32, double *__restrict__ modal, int64_t n_cells) {
  constexpr int CB = Modal32Cfg<N, M>::kCells, NT = Modal32Cfg<N, M>::kThreads;
  __shared__ float s_m[CB][N * 3];  // momenta, FP32
  const int64_t c0 = (int64_t)blockIdx.x * CB;
  const int t = threadIdx.x;
  const int64_t avail = n_cells - c0;
  const int nc = avail < CB ? (int)avail : CB;
  for (int i = t; i < nc * N * 3; i += NT) {
    const int cl = i / (N * 3), r = i - cl * (N * 3), q = r / 3, d = r - q * 3;
    s_m[cl][r] = f64_to_f32(u[((c0 + cl) * N + q) * kK + 1 + d]);
  }
  __syncthreads();
  const int cl = t / M, m = t - cl * M;
  if (cl >= nc) return;
  const int64_t c = c0 + cl;
  const float *mc32 = mn32 + c * N * M;
  const double *mc = mn + c * N * M;
  const double *uc = u + c * kK * N;
  float s[3] = {0.f, 0.f, 0.f};
  double rho = 0, e = 0;
#pragma unroll 3
  for (int q = 0; q < N; ++q) {
    const float w = mc32[q * M + m];
#pragma unroll
    for (int d = 0; d < 3; ++d) s[d] = fmaf(s_m[cl][q * 3 + d], w, s[d]);
    const double wd = mc[q * M + m];
    rho += uc[q * kK] * wd;
    e += uc[q * kK + 4] * wd;
  }
  modal[(c * kK + 0) * M + m] = rho;
#pragma unroll
  for (int d = 0; d < 3; ++d) modal[(c * kK + 1 + d) * M + m] = f32_to_f64(s[d]);
  modal[(c * kK + 4) * M + m] = e;
}

// Frame-independent scalars of EigenMatrices (riemann/euler/eigen.hpp:27-56)
// at one state, computed once per cell: velocity, a, 1/a, b1 = 1/e0
// (e0 = a^2 / (gamma - 1)), ek, h0 = e0 + ek.  Columns of R: u - a,
// u (entropy), two shear waves, u + a; L = R^-1.
struct EigenState {
  double vel[3], a, ia, b1, ek, h0;
};

__device__ EigenState eigen_state(const Prim &w) {
  EigenState s;
  s.vel[0] = w.u; s.vel[1] = w.v; s.vel[2] = w.w;
  s.a = sqrt(kGamma * w.p / w.rho);
  s.ia = 1 / s.a;
  s.ek = (w.u * w.u + w.v * w.v + w.w * w.w) / 2;
  const double e0 = s.a * s.a * (1 / kGm1);
  s.b1 = 1 / e0;
  s.h0 = e0 + s.ek;
  return s;
}

// L (row-major, entries 0..24) and R (25..49) of EigenMatrices
// (riemann/euler/eigen.hpp:27-56) for the frame {nu, mu, pi}, by one thread in
// straight-line code: the frame's dot products once, every entry at most two
// FP64 operations from them.  (Spread over the block entry by entry, the
// entries' different formulas made each warp step through all of them.)
__device__ void eigen_matrices(const EigenState &s, const double *nu, const double *mu,
                               const double *pi, double *lr) {
  const double *vel = s.vel;
  const double u_nu = vel[0] * nu[0] + vel[1] * nu[1] + vel[2] * nu[2];
  const double u_mu = vel[0] * mu[0] + vel[1] * mu[1] + vel[2] * mu[2];
  const double u_pi = vel[0] * pi[0] + vel[1] * pi[1] + vel[2] * pi[2];
  const double a = s.a, ek = s.ek, b1 = s.b1, b2 = b1 * ek, ia = s.ia;
  double *L = lr, *R = lr + 25;
  // L: columns 0 and 4
  L[0 * 5 + 0] = (b2 + u_nu * ia) / 2;
  L[1 * 5 + 0] = 1 - b2;
  L[2 * 5 + 0] = -u_mu;
  L[3 * 5 + 0] = -u_pi;
  L[4 * 5 + 0] = (b2 - u_nu * ia) / 2;
  L[0 * 5 + 4] = b1 / 2;
  L[1 * 5 + 4] = -b1;
  L[2 * 5 + 4] = 0.0;
  L[3 * 5 + 4] = 0.0;
  L[4 * 5 + 4] = b1 / 2;
  // R: rows 0 and 4
  R[0 * 5 + 0] = 1.0; R[0 * 5 + 1] = 1.0; R[0 * 5 + 2] = 0.0; R[0 * 5 + 3] = 0.0; R[0 * 5 + 4] = 1.0;
  R[4 * 5 + 0] = s.h0 - a * u_nu;
  R[4 * 5 + 1] = ek;
  R[4 * 5 + 2] = u_mu;
  R[4 * 5 + 3] = u_pi;
  R[4 * 5 + 4] = s.h0 + a * u_nu;
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    const double bv = b1 * vel[d], ni = nu[d] * ia, an = a * nu[d];
    // L column 1 + d
    L[0 * 5 + 1 + d] = -(bv + ni) / 2;
    L[1 * 5 + 1 + d] = bv;
    L[2 * 5 + 1 + d] = mu[d];
    L[3 * 5 + 1 + d] = pi[d];
    L[4 * 5 + 1 + d] = -(bv - ni) / 2;
    // R row 1 + d
    R[(1 + d) * 5 + 0] = vel[d] - an;
    R[(1 + d) * 5 + 1] = vel[d];
    R[(1 + d) * 5 + 2] = mu[d];
    R[(1 + d) * 5 + 3] = pi[d];
    R[(1 + d) * 5 + 4] = vel[d] + an;
  }
}

// weno::Eigen reconstruction of cell c from its candidates (slots 0..n_adj-1
// neighbours, slot 6 own) into s_new, all adjacent faces at once so that the
// 64 threads stay busy:
//   G_i = C_i B C_i^T     (K x K, face-independent, symmetric: its upper
//                          triangle) for each candidate
//   L_f, R_f              every entry of every face's eigen-matrices
//   beta[f][i][k] = L_f[k] G_i L_f[k]^T   (= GetSmoothness of L_f C_i)
//   w[f][i][k]            the reference's weights per face and field
//   nw[f] = sum_i w[f][i] (L_f C_i),  new = sum_f vol_f R_f nw[f] / sum_f vol_f
template <int M, class Args>
__device__ void eigen_reconstruct(const Args &a, int64_t c, int n_adj,
                                  double (*s_cand)[kK][M], double (*s_new)[M]) {
  __shared__ double s_cb[7][kK][M];     // C_i B
  __shared__ double s_G[7][kK][kK];
  __shared__ double s_LR[6][50];        // per face: L (25) then R (25)
  __shared__ double s_beta[6][7][kK];
  __shared__ double s_w[6][7][kK];
  __shared__ double s_nw[6][kK][M];
  __shared__ double s_vol[6];
  __shared__ EigenState s_es;
  const int t = threadIdx.x, nt = blockDim.x;
  const int nc = n_adj + 1;  // candidates: 0..n_adj-1 neighbours, then own (slot 6)
  const double *B = a.beta + c * M * M;
  // C_i B and the face data
  for (int i = t; i < nc * kK * M; i += nt) {
    const int cand = i / (kK * M), r = i - cand * kK * M, k = r / M, m = r - k * M;
    const int src = cand < n_adj ? cand : 6;
    double v = 0;
    for (int j = 0; j < M; ++j) v += s_cand[src][k][j] * B[j * M + m];
    s_cb[cand][k][m] = v;
  }
  if (t == 0) {
    const double s00 = a.s00[c];
    s_es = eigen_state(cons_to_prim(s_cand[6][0][0] * s00, s_cand[6][1][0] * s00, s_cand[6][2][0] * s00,
                                    s_cand[6][3][0] * s00, s_cand[6][4][0] * s00));
  }
  if (t < n_adj) s_vol[t] = a.volume[a.adj[c * 6 + t]];
  __syncthreads();
  if (t < n_adj) {
    const double *fr = a.frame + (c * 6 + t) * 9;
    eigen_matrices(s_es, fr, fr + 3, fr + 6, s_LR[t]);
  }
  __syncthreads();
  // G is symmetric (B is): its upper triangle only, the off-diagonal entries
  // doubled, so that L G L^T = sum_j L_j (G_jj L_j + sum_{l > j} 2 G_jl L_l)
  constexpr int kUpper = kK * (kK + 1) / 2;  // 15 entries l >= j
  for (int i = t; i < nc * kUpper; i += nt) {
    const int cand = i / kUpper;
    int r = i - cand * kUpper, j = 0;
    while (r >= kK - j) {  // row j holds the kK - j entries l = j .. kK - 1
      r -= kK - j;
      ++j;
    }
    const int l = j + r;
    const int src = cand < n_adj ? cand : 6;
    double v = 0;
    for (int m = 0; m < M; ++m) v += s_cb[cand][j][m] * s_cand[src][l][m];
    s_G[cand][j][l] = l == j ? v : 2 * v;
  }
  __syncthreads();
  for (int i = t; i < n_adj * nc * kK; i += nt) {
    const int f = i / (nc * kK), r = i - f * nc * kK, cand = r / kK, k = r - cand * kK;
    const double *Lk = &s_LR[f][k * 5];
    double b = 0;
#pragma unroll
    for (int j = 0; j < kK; ++j) {
      double row = s_G[cand][j][j] * Lk[j];
#pragma unroll
      for (int l = j + 1; l < kK; ++l) row += s_G[cand][j][l] * Lk[l];
      b += Lk[j] * row;
    }
    s_beta[f][cand][k] = b;
  }
  __syncthreads();
  // weights (weno.hpp:306-326): w0 for the neighbours, 1 - n w0 for the own
  // candidate, divided by (beta + eps)^2, normalised per field
  for (int i = t; i < n_adj * kK; i += nt) {
    const int f = i / kK, k = i - f * kK;
    double sum = 0;
    for (int cand = 0; cand < nc; ++cand) {
      double w = a.w0;
      if (cand == n_adj) {
        w *= -n_adj;
        w += 1.0;
      }
      double b = s_beta[f][cand][k] + a.eps;
      b *= b;
      w *= rcp_newton(b);
      s_w[f][cand][k] = w;
      sum += w;
    }
    const double isum = rcp_newton(sum);
    for (int cand = 0; cand < nc; ++cand) s_w[f][cand][k] *= isum;
  }
  __syncthreads();
  // nw[f] = w_own (L_f C_own) + sum_i w_i (L_f C_i)   (weno.hpp:327-333)
  for (int i = t; i < n_adj * kK * M; i += nt) {
    const int f = i / (kK * M), r = i - f * kK * M, k = r / M, m = r - k * M;
    const double *Lk = &s_LR[f][k * 5];
    double lc = 0;
#pragma unroll
    for (int j = 0; j < kK; ++j) lc += Lk[j] * s_cand[6][j][m];
    double v = lc * s_w[f][n_adj][k];
    for (int cand = 0; cand < n_adj; ++cand) {
      lc = 0;
#pragma unroll
      for (int j = 0; j < kK; ++j) lc += Lk[j] * s_cand[cand][j][m];
      v += lc * s_w[f][cand][k];
    }
    s_nw[f][k][m] = v;
  }
  __syncthreads();
  // back to conservative variables, volume-weighted over the faces
  // (weno.hpp:334-347)
  for (int i = t; i < kK * M; i += nt) {
    const int k = i / M, m = i - k * M;
    double acc = 0, total = 0;
    for (int f = 0; f < n_adj; ++f) {
      double v = 0;
#pragma unroll
      for (int j = 0; j < kK; ++j) v += s_LR[f][25 + k * 5 + j] * s_nw[f][j][m];
      acc += v * s_vol[f];
      total += s_vol[f];
    }
    s_new[k][m] = acc * rcp_newton(total);
  }
  __syncthreads();
}

// weno::Eigen::IsNotSmooth (weno.hpp:230-258) on density and energy, one
// thread per cell; flagged cells are appended to the troubled list, one
// atomic per warp (their order does not matter: each reconstruction writes
// only its own cell).
// A warp-cooperative form (eight lanes per cell splitting the modes, shuffle
// reductions) measured five times slower on the four-quadrant case: on this
// FP64-bound part the shuffle trees replicate the FP64 adds and the per-cell
// bookkeeping on every lane, which costs more than the coalescing gains.
template <int M>
__global__ void __launch_bounds__(256)
weno_detect_kernel(WenoArgs a, int32_t *list, unsigned *count) {
  const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= a.n_cells) return;
  const double s00 = a.s00[c];
  const double *ev = a.eval + c * 7 * M;
  const double *own = a.modal + c * kK * M;
  int adj[6], n = 0;
  for (int s = 0; s < 6; ++s) {
    adj[s] = a.adj[c * 6 + s];
    n += adj[s] >= 0;
  }
  bool troubled = false;
  const int comps[2] = {0, kK - 1};
  for (int ci = 0; ci < 2; ++ci) {
    const int k = comps[ci];
    double max_abs = fmax(1e-9, fabs(own[k * M] * s00));
    double mine = 0;
    for (int m = 0; m < M; ++m) mine += own[k * M + m] * ev[6 * M + m];
    double sum_abs = 0;
    for (int s = 0; s < n; ++s) {
      const int b = adj[s];
      const double *cb = a.modal + ((int64_t)b * kK + k) * M;
      double v = 0;
      for (int m = 0; m < M; ++m) v += cb[m] * ev[s * M + m];
      sum_abs += fabs(mine - v);
      max_abs = fmax(max_abs, fabs(cb[0] * a.s00[b]));
    }
    if (sum_abs / max_abs / a.divisor[c] > a.smooth_ref) troubled = true;
  }
  if (a.cell_hot) a.cell_hot[c] = troubled ? 1 : 0;
  // one atomic per warp for its troubled cells (the list's order is free)
  const unsigned active = __activemask();
  const unsigned mask = __ballot_sync(active, troubled);
  if (mask) {
    const int lane = threadIdx.x & 31, leader = __ffs(mask) - 1;
    unsigned base = 0;
    if (lane == leader) base = atomicAdd(count, (unsigned)__popc(mask));
    base = __shfl_sync(active, base, leader);
    if (troubled) list[base + __popc(mask & ((1u << lane) - 1u))] = (int32_t)c;
  }
}

// Reconstruction of the listed cells (every cell when list is null) by a
// persistent grid of 64-thread blocks, one cell at a time per block.  MODAL:
// the new coefficients go to the modal column; otherwise the new nodal
// values (UpdateNodalCoeff).
template <int N, int M, int MODE, bool MODAL = false>
__global__ void __launch_bounds__(64)
weno_reconstruct_kernel(WenoArgs a, const int32_t *list, const unsigned *count) {
  const int t = threadIdx.x;
  __shared__ double s_cand[7][kK][M];  // slots 0..5 neighbours, 6 own
  __shared__ double s_beta[7][kK];
  __shared__ double s_new[kK][M];
  __shared__ int s_adj[6];
  __shared__ int s_nadj;
  const int64_t n_work = list ? (int64_t)*count : a.n_cells;
  if (blockIdx.x == 0 && t == 0 && n_work > 0) atomicAdd(a.troubled, (unsigned long long)n_work);
  for (int64_t item = blockIdx.x; item < n_work; item += gridDim.x) {
  const int64_t c = list ? (int64_t)list[item] : item;
  if (t < 6) s_adj[t] = a.adj[c * 6 + t];
  for (int i = t; i < kK * M; i += blockDim.x) s_cand[6][i / M][i % M] = a.modal[c * kK * M + i];
  __syncthreads();
  if (t == 0) {
    int n = 0;
    for (int s = 0; s < 6; ++s) n += s_adj[s] >= 0;
    s_nadj = n;
  }
  __syncthreads();
  const int n_adj = s_nadj;
  // Borrow: neighbour coefficients projected onto the own basis, shifted to
  // the own average (weno.hpp:138-166, projection.hpp:260-264).  weno::Eigen
  // (throughput-bound: many cells per SM) takes one thread per (neighbour,
  // field) with the neighbour's coefficients in registers; the Lazy modes
  // (every cell of small meshes: latency-bound) one thread per (neighbour,
  // field, mode), ten times shorter dependent chains, the mode-0 thread
  // applying the shift.
  if constexpr (MODE == 3) {
    if (t < 6 * kK) {
      const int slot = t / kK, k = t - slot * kK;
      if (slot < n_adj) {
        const int b = s_adj[slot];
        const double *P = a.proj + ((c * 6 + slot) * M) * M;
        const double *cb = a.modal + ((int64_t)b * kK + k) * M;
        double cbl[M];
#pragma unroll
        for (int j = 0; j < M; ++j) cbl[j] = cb[j];
#pragma unroll
        for (int m = 0; m < M; ++m) {
          double s = 0;
#pragma unroll
          for (int j = 0; j < M; ++j) s += cbl[j] * P[j * M + m];
          s_cand[slot][k][m] = s;
        }
        const double s00 = a.s00[c];
        const double my_avg = s_cand[6][k][0] * s00;
        const double adj_avg = s_cand[slot][k][0] * s00;
        s_cand[slot][k][0] += (my_avg - adj_avg) / s00;
      }
    }
  } else {
    for (int i = t; i < 6 * kK * M; i += blockDim.x) {
      const int slot = i / (kK * M), r = i - slot * (kK * M), k = r / M, m = r - k * M;
      if (slot < n_adj) {
        const int b = s_adj[slot];
        const double *P = a.proj + ((c * 6 + slot) * M) * M;
        const double *cb = a.modal + ((int64_t)b * kK + k) * M;
        double s = 0;
#pragma unroll
        for (int j = 0; j < M; ++j) s += cb[j] * P[j * M + m];
        if (m == 0) {
          const double s00 = a.s00[c];
          const double my_avg = s_cand[6][k][0] * s00;
          const double adj_avg = s * s00;
          s += (my_avg - adj_avg) / s00;
        }
        s_cand[slot][k][m] = s;
      }
    }
  }
  __syncthreads();
  if constexpr (MODE == 3) {
    eigen_reconstruct<M>(a, c, n_adj, s_cand, s_new);
  } else {
  // The phases are spread over the block so that the warps' FP64 lanes stay
  // busy: the rows B c by (candidate, field, mode), the quadratic forms by
  // (candidate, field), the weights by field, the new projection by (field,
  // mode).
  __shared__ double s_row[7][kK][M];
  __shared__ double s_wt[kK][7];
  // smoothness indicators beta = c^T B c (weno.hpp:25-95)
  const double *B = a.beta + c * M * M;
  for (int i = t; i < 7 * kK * M; i += blockDim.x) {
    const int slot = i / (kK * M), r = i - slot * (kK * M), k = r / M, m = r - k * M;
    if (slot == 6 || slot < n_adj) {
      double row = 0;
#pragma unroll
      for (int j = 0; j < M; ++j) row += B[m * M + j] * s_cand[slot][k][j];
      s_row[slot][k][m] = row;
    }
  }
  __syncthreads();
  if (t < 7 * kK) {
    const int slot = t / kK, k = t - slot * kK;
    if (slot == 6 || slot < n_adj) {
      double b = 0;
#pragma unroll
      for (int m = 0; m < M; ++m) b += s_cand[slot][k][m] * s_row[slot][k][m];
      s_beta[slot][k] = b;
    }
  }
  __syncthreads();
  // weights (weno.hpp:167-194): w0 for the neighbours, 1 - n w0 for the own
  // candidate, divided by (beta + eps)^2 and normalised per field (the
  // divisions as Newton reciprocals)
  if (t < kK) {
    const int k = t;
    double w[7];
    for (int s = 0; s < n_adj; ++s) w[s] = a.w0;
    double ws = a.w0;
    ws *= -n_adj;
    ws += 1.0;
    w[n_adj] = ws;
    double sum = 0;
    for (int s = 0; s <= n_adj; ++s) {
      double b = (s < n_adj ? s_beta[s][k] : s_beta[6][k]) + a.eps;
      b *= b;
      w[s] *= rcp_newton(b);
    }
    for (int s = 0; s <= n_adj; ++s) sum += w[s];
    const double isum = rcp_newton(sum);
    for (int s = 0; s <= n_adj; ++s) s_wt[k][s] = w[s] * isum;
  }
  __syncthreads();
  // the new projection (weno.hpp:182-194)
  for (int i = t; i < kK * M; i += blockDim.x) {
    const int k = i / M, m = i - k * M;
    double v = s_cand[6][k][m] * s_wt[k][n_adj];
    for (int s = 0; s < n_adj; ++s) v += s_cand[s][k][m] * s_wt[k][s];
    s_new[k][m] = v;
  }
  }
  __syncthreads();
  if constexpr (MODAL) {
    // SetCoeff: the column block [M][K] takes the new coefficients
    double *uc = a.u + c * kK * M;
    for (int i = t; i < M * kK; i += blockDim.x) {
      const int m = i / kK, k = i - m * kK;
      uc[i] = s_new[k][m];
    }
  } else if (a.trace) {
    // UpdateNodalCoeff, one node per thread, and the node's new trace
    const double *pc = a.psi + c * N * M;
    double *uc = a.u + c * kK * N;
    for (int q = t; q < N; q += blockDim.x) {
      double v[kK];
#pragma unroll
      for (int k = 0; k < kK; ++k) {
        double s = 0;
#pragma unroll
        for (int m = 0; m < M; ++m) s += s_new[k][m] * pc[q * M + m];
        v[k] = s;
        uc[q * kK + k] = s;
      }
      double tr[3];
      if (a.trace_fast)
        node_trace<true>(v, tr, a.trace_roe != 0);
      else
        node_trace<false>(v, tr, a.trace_roe != 0);
      double *dst = a.trace + (c * N + q) * 3;
      dst[0] = tr[0]; dst[1] = tr[1]; dst[2] = tr[2];
    }
  } else {
    // UpdateNodalCoeff: nodal values = modal expansion at the nodes
    const double *pc = a.psi + c * N * M;
    double *uc = a.u + c * kK * N;
    for (int i = t; i < N * kK; i += blockDim.x) {
      const int q = i / kK, k = i - q * kK;
      double v = 0;
#pragma unroll
      for (int m = 0; m < M; ++m) v += s_new[k][m] * pc[q * M + m];
      uc[q * kK + k] = v;
    }
  }
  __syncthreads();  // the shared arrays are reused by the next cell
  }
}

template <int Q>
int limiter_dispatch(mcfd_handle *h, double *u) {
  constexpr int N = Q * Q * Q;
  constexpr int M = Q * (Q + 1) * (Q + 2) / 6;
  const Mesh &mesh = h->mesh;
  Limiter &l = h->lim;
  int64_t total = mesh.n_cells * M;
  // FP64 shock cells: the troubled region's momenta take the FP64 product too
  // FP64 products with a detector: density and energy of every cell now, the
  // momenta of the reconstructions' candidates after the detector
  const bool deferred = !(l.mn32 && !l.block_hot) && l.kind != 1;
  if (l.mn32 && !l.block_hot) {
    constexpr int CB = Modal32Cfg<N, M>::kCells;
    weno_modal32_kernel<N, M><<<(unsigned)((mesh.n_cells + CB - 1) / CB), Modal32Cfg<N, M>::kThreads, 0,
                                h->stream>>>(u, l.mn, l.mn32, l.modal, mesh.n_cells);
  } else if (deferred) {
    weno_modal_kernel<N, M, true><<<(unsigned)((total + 255) / 256), 256, 0, h->stream>>>(
        u, l.mn, l.modal, mesh.n_cells);
  } else {
    weno_modal_kernel<N, M><<<(unsigned)((total + 255) / 256), 256, 0, h->stream>>>(
        u, l.mn, l.modal, mesh.n_cells);
  }
  // a stage state whose node traces the face kernels will read gets the
  // reconstructed cells' traces rewritten
  double *trace = (h->use_trace && h->trace_for == u) ? h->buf.trace : nullptr;
  WenoArgs wa{u, l.modal, l.psi, l.proj, l.beta, l.eval, l.s00, l.divisor, l.adj,
              l.frame, l.volume, l.troubled, mesh.n_cells, l.w0, l.eps, (Q - 1) < 3 ? 1.0 : 3.0,
              trace, h->opt.precision == 1, h->opt.riemann == kRoe, l.cell_hot};
  // persistent grid: limiter_blocks_per_sm blocks of 64 threads per SM
  int sms = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, h->device);
  const unsigned grid =
      (unsigned)std::min<int64_t>(mesh.n_cells, (int64_t)std::max(sms, 1) * h->tune.limiter_blocks_per_sm);
  if (l.kind == 1 /* MCFD_LIMITER_LAZY: every cell */) {
    weno_reconstruct_kernel<N, M, 1><<<grid, 64, 0, h->stream>>>(wa, nullptr, nullptr);
    if (l.block_hot) cudaMemsetAsync(l.block_hot, 1, l.n_blocks, h->stream);
    return 2;
  }
  cudaMemsetAsync(l.list_count, 0, sizeof(unsigned), h->stream);
  weno_detect_kernel<M><<<(unsigned)((mesh.n_cells + 255) / 256), 256, 0, h->stream>>>(
      wa, l.list, l.list_count);
  int n = 3;
  if (l.block_hot) {
    const unsigned cgrid = (unsigned)((mesh.n_cells + 255) / 256);
    const uint8_t *flags = l.cell_hot;
    if (h->opt.shock_fp64 > 1) {  // a second layer of neighbours
      weno_dilate_kernel<<<cgrid, 256, 0, h->stream>>>(l.adj, l.cell_hot, l.cell_hot2, mesh.n_cells);
      flags = l.cell_hot2;
      ++n;
    }
    cudaMemsetAsync(l.block_hot, 0, l.n_blocks, h->stream);
    weno_mark_blocks_kernel<<<cgrid, 256, 0, h->stream>>>(l.adj, flags, l.block_hot, mesh.n_cells,
                                                           Q == 4 ? 4 : (Q == 3 ? 9 : 32));
    ++n;
  }
  if (deferred) {
    weno_modal_momenta_kernel<N, M><<<(unsigned)std::max(sms, 1) * 8, 256, 0, h->stream>>>(
        u, l.mn, l.modal, l.adj, l.list, l.list_count);
    ++n;
  }
  if (l.kind == 2 /* MCFD_LIMITER_DETECT_LAZY */)
    weno_reconstruct_kernel<N, M, 2><<<grid, 64, 0, h->stream>>>(wa, l.list, l.list_count);
  else
    weno_reconstruct_kernel<N, M, 3><<<grid, 64, 0, h->stream>>>(wa, l.list, l.list_count);
  return n;
}

// The modal scheme's limiter pass (M = basis size of degree p).
template <int M>
int limiter_dispatch_modal(mcfd_handle *h, double *u) {
  const Mesh &mesh = h->mesh;
  Limiter &l = h->lim;
  const int64_t total = mesh.n_cells * M;
  weno_transpose_kernel<M><<<(unsigned)((total + 255) / 256), 256, 0, h->stream>>>(u, l.modal, mesh.n_cells);
  WenoArgs wa{u, l.modal, nullptr, l.proj, l.beta, l.eval, l.s00, l.divisor, l.adj,
              l.frame, l.volume, l.troubled, mesh.n_cells, l.w0, l.eps, mesh.p < 3 ? 1.0 : 3.0,
              nullptr, 0, 0, nullptr};
  int sms = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, h->device);
  const unsigned grid =
      (unsigned)std::min<int64_t>(mesh.n_cells, (int64_t)std::max(sms, 1) * h->tune.limiter_blocks_per_sm);
  if (l.kind == 1 /* MCFD_LIMITER_LAZY: every cell */) {
    weno_reconstruct_kernel<0, M, 1, true><<<grid, 64, 0, h->stream>>>(wa, nullptr, nullptr);
    return 2;
  }
  cudaMemsetAsync(l.list_count, 0, sizeof(unsigned), h->stream);
  weno_detect_kernel<M><<<(unsigned)((mesh.n_cells + 255) / 256), 256, 0, h->stream>>>(
      wa, l.list, l.list_count);
  if (l.kind == 2 /* MCFD_LIMITER_DETECT_LAZY */)
    weno_reconstruct_kernel<0, M, 2, true><<<grid, 64, 0, h->stream>>>(wa, l.list, l.list_count);
  else
    weno_reconstruct_kernel<0, M, 3, true><<<grid, 64, 0, h->stream>>>(wa, l.list, l.list_count);
  return 3;
}

}  // namespace

int launch_limiter(mcfd_handle *h, double *u) {
  if (h->lim.kind == 0) return 0;
  if (h->opt.scheme == kSchemeModal) {
    switch (h->mesh.p) {
      case 1: return limiter_dispatch_modal<4>(h, u);
      case 2: return limiter_dispatch_modal<10>(h, u);
      default: return limiter_dispatch_modal<20>(h, u);
    }
  }
  switch (h->mesh.q) {
    case 2: return limiter_dispatch<2>(h, u);
    case 3: return limiter_dispatch<3>(h, u);
    default: return limiter_dispatch<4>(h, u);
  }
}

}  // namespace mcfd
