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
// Every cell reads the modal buffer only, so the in-place write is safe and
// the pass is Jacobi-like, as in limiter::Reconstruct (all new projections
// are computed before any is written back).
#include <cuda_runtime.h>

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
  unsigned long long *troubled;
  int64_t n_cells;
  double w0, eps, smooth_ref;
};

template <int N, int M>
__global__ void __launch_bounds__(256)
weno_modal_kernel(const double *__restrict__ u, const double *__restrict__ mn,
                  double *__restrict__ modal, int64_t n_cells) {
  int64_t gid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (gid >= n_cells * kK * M) return;
  const int64_t c = gid / (kK * M);
  const int r = (int)(gid - c * kK * M);
  const int k = r / M, m = r - k * M;
  const double *uc = u + c * kK * N;
  const double *mc = mn + c * N * M;
  double s = 0;
#pragma unroll 4
  for (int q = 0; q < N; ++q) s += uc[q * kK + k] * mc[q * M + m];
  modal[gid] = s;
}

template <int N, int M, int MODE>
__global__ void __launch_bounds__(64) weno_reconstruct_kernel(WenoArgs a) {
  const int64_t c = blockIdx.x;
  const int t = threadIdx.x;
  __shared__ double s_cand[7][kK][M];  // slots 0..5 neighbours, 6 own
  __shared__ double s_beta[7][kK];
  __shared__ double s_new[kK][M];
  __shared__ int s_adj[6];
  __shared__ int s_nadj, s_troubled;
  if (t < 6) s_adj[t] = a.adj[c * 6 + t];
  for (int i = t; i < kK * M; i += blockDim.x) s_cand[6][i / M][i % M] = a.modal[c * kK * M + i];
  __syncthreads();
  if (t == 0) {
    int n = 0;
    for (int s = 0; s < 6; ++s) n += s_adj[s] >= 0;
    s_nadj = n;
    int troubled = 1;
    if (MODE == 2) {
      // weno::Eigen::IsNotSmooth on density and energy (weno.hpp:230-258)
      troubled = 0;
      const double s00 = a.s00[c];
      const double *ev = a.eval + c * 7 * M;
      const int comps[2] = {0, kK - 1};
      for (int ci = 0; ci < 2; ++ci) {
        const int k = comps[ci];
        double max_abs = fmax(1e-9, fabs(s_cand[6][k][0] * s00));
        double mine = 0;
        for (int m = 0; m < M; ++m) mine += s_cand[6][k][m] * ev[6 * M + m];
        double sum_abs = 0;
        for (int s = 0; s < n; ++s) {
          const int b = s_adj[s];
          const double *cb = a.modal + ((int64_t)b * kK + k) * M;
          double v = 0;
          for (int m = 0; m < M; ++m) v += cb[m] * ev[s * M + m];
          sum_abs += fabs(mine - v);
          max_abs = fmax(max_abs, fabs(cb[0] * a.s00[b]));
        }
        if (sum_abs / max_abs / a.divisor[c] > a.smooth_ref) troubled = 1;
      }
    }
    s_troubled = troubled;
  }
  __syncthreads();
  if (!s_troubled) return;
  const int n_adj = s_nadj;
  // Borrow: neighbour coefficients projected onto the own basis, shifted to
  // the own average (weno.hpp:138-166, projection.hpp:260-264)
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
  __syncthreads();
  // smoothness indicators beta = c^T B c (weno.hpp:25-95)
  if (t < 7 * kK) {
    const int slot = t / kK, k = t - slot * kK;
    if (slot == 6 || slot < n_adj) {
      const double *B = a.beta + c * M * M;
      double b = 0;
#pragma unroll
      for (int m = 0; m < M; ++m) {
        double row = 0;
#pragma unroll
        for (int j = 0; j < M; ++j) row += B[m * M + j] * s_cand[slot][k][j];
        b += s_cand[slot][k][m] * row;
      }
      s_beta[slot][k] = b;
    }
  }
  __syncthreads();
  // weights and the new projection (weno.hpp:167-194)
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
      w[s] /= b;
    }
    for (int s = 0; s <= n_adj; ++s) sum += w[s];
    for (int s = 0; s <= n_adj; ++s) w[s] /= sum;
    for (int m = 0; m < M; ++m) {
      double v = s_cand[6][k][m] * w[n_adj];
      for (int s = 0; s < n_adj; ++s) v += s_cand[s][k][m] * w[s];
      s_new[k][m] = v;
    }
  }
  __syncthreads();
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
  if (t == 0) atomicAdd(a.troubled, 1ull);
}

template <int Q>
void limiter_dispatch(mcfd_handle *h, double *u) {
  constexpr int N = Q * Q * Q;
  constexpr int M = Q * (Q + 1) * (Q + 2) / 6;
  const Mesh &mesh = h->mesh;
  Limiter &l = h->lim;
  int64_t total = mesh.n_cells * kK * M;
  weno_modal_kernel<N, M><<<(unsigned)((total + 255) / 256), 256, 0, h->stream>>>(
      u, l.mn, l.modal, mesh.n_cells);
  WenoArgs wa{u, l.modal, l.psi, l.proj, l.beta, l.eval, l.s00, l.divisor, l.adj,
              l.troubled, mesh.n_cells, l.w0, l.eps, (Q - 1) < 3 ? 1.0 : 3.0};
  if (l.kind == 1 /* MCFD_LIMITER_LAZY */)
    weno_reconstruct_kernel<N, M, 1><<<(unsigned)mesh.n_cells, 64, 0, h->stream>>>(wa);
  else
    weno_reconstruct_kernel<N, M, 2><<<(unsigned)mesh.n_cells, 64, 0, h->stream>>>(wa);
}

}  // namespace

int launch_limiter(mcfd_handle *h, double *u) {
  if (h->lim.kind == 0) return 0;
  switch (h->mesh.q) {
    case 2: limiter_dispatch<2>(h, u); break;
    case 3: limiter_dispatch<3>(h, u); break;
    default: limiter_dispatch<4>(h, u); break;
  }
  return 2;
}

}  // namespace mcfd
