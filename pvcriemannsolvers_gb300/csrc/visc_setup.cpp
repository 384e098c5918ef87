// Host set-up of the artificial-viscosity tables (mcfd_set_viscosity): the
// geometric data the properties, face and cell kernels read per cell, per
// face point and per face point side.  Everything is computed once from the
// Hex8 corners kept by mcfd_create.
//
//   cell length        cbrt(V) / 2 (mesh/part.hpp:230) and length^(p + 4)
//                      (spatial/viscosity.hpp:511-512)
//   distance d         normal . holder_to_sharer at every face point
//                      (spatial/fem.hpp:79-85); holder_to_sharer is the
//                      sharer centre minus the holder centre, or twice the
//                      way from the holder centre to the face centre on a
//                      boundary (mesh/part.hpp:118-132); centres are the
//                      maps' LocalToGlobal at the local origin
//                      (coordinate/hexahedron.hpp:40-48)
//   penalties          beta0 / d and beta1 d (riemann/diffusive/direct.hpp:85-90)
//   jump weights       w_f V_cell / area_face for both sides
//                      (spatial/viscosity.hpp:446-475, part.hpp:123-124)
//   side vectors       m = J^-T n and q = sum_j m_j (d_j J^-1)^T n at the
//                      side's node: n^T H n = m^T H_loc m + q . g_loc for the
//                      global Hessian of polynomial/hexahedron.hpp:495-525
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/mcfd.h"
#include "handle.hpp"

namespace mcfd {
namespace {

constexpr int kK = 5;  // conserved variables

const int kCorner[8][3] = {{-1, -1, -1}, {+1, -1, -1}, {+1, +1, -1}, {-1, +1, -1},
                           {-1, -1, +1}, {+1, -1, +1}, {+1, +1, +1}, {-1, +1, +1}};
const int kFaceCorners[6][4] = {{0, 3, 2, 1}, {0, 1, 5, 4}, {1, 2, 6, 5},
                                {2, 3, 7, 6}, {0, 4, 7, 3}, {4, 5, 6, 7}};

void gll_weights(int q, double *w) {
  if (q == 2) {
    w[0] = w[1] = 1;
  } else if (q == 3) {
    w[0] = 1.0 / 3; w[1] = 4.0 / 3; w[2] = 1.0 / 3;
  } else {
    w[0] = 1.0 / 6; w[1] = 5.0 / 6; w[2] = 5.0 / 6; w[3] = 1.0 / 6;
  }
}

// x, J (rows: local directions) and d_a J of the Hex8 map at loc.
void hex8_map(const double *xn, const double *loc, double *x, double *J, double *dJ) {
  for (int e = 0; e < 3; ++e) x[e] = 0;
  for (int e = 0; e < 9; ++e) J[e] = 0;
  for (int e = 0; e < 27; ++e) dJ[e] = 0;
  for (int v = 0; v < 8; ++v) {
    const double f0 = 1 + kCorner[v][0] * loc[0], f1 = 1 + kCorner[v][1] * loc[1],
                 f2 = 1 + kCorner[v][2] * loc[2];
    const double s = f0 * f1 * f2 / 8;
    const double g[3] = {kCorner[v][0] * f1 * f2 / 8, kCorner[v][1] * f0 * f2 / 8,
                         kCorner[v][2] * f0 * f1 / 8};
    for (int e = 0; e < 3; ++e) {
      x[e] += s * xn[v * 3 + e];
      for (int r = 0; r < 3; ++r) J[r * 3 + e] += g[r] * xn[v * 3 + e];
    }
    for (int a = 0; a < 3; ++a)
      for (int b = 0; b < 3; ++b) {
        if (a == b) continue;
        const int c = 3 - a - b;
        const double h = kCorner[v][a] * kCorner[v][b] * (1 + kCorner[v][c] * loc[c]) / 8;
        for (int e = 0; e < 3; ++e) dJ[a * 9 + b * 3 + e] += xn[v * 3 + e] * h;
      }
  }
}

double inverse3(const double *m, double *inv) {
  const double det = m[0] * (m[4] * m[8] - m[5] * m[7]) - m[1] * (m[3] * m[8] - m[5] * m[6]) +
                     m[2] * (m[3] * m[7] - m[4] * m[6]);
  inv[0] = (m[4] * m[8] - m[5] * m[7]) / det;
  inv[1] = (m[2] * m[7] - m[1] * m[8]) / det;
  inv[2] = (m[1] * m[5] - m[2] * m[4]) / det;
  inv[3] = (m[5] * m[6] - m[3] * m[8]) / det;
  inv[4] = (m[0] * m[8] - m[2] * m[6]) / det;
  inv[5] = (m[2] * m[3] - m[0] * m[5]) / det;
  inv[6] = (m[3] * m[7] - m[4] * m[6]) / det;
  inv[7] = (m[1] * m[6] - m[0] * m[7]) / det;
  inv[8] = (m[0] * m[4] - m[1] * m[3]) / det;
  return det;
}

void mul3(const double *a, const double *b, double *c) {
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j)
      c[i * 3 + j] = a[i * 3 + 0] * b[0 * 3 + j] + a[i * 3 + 1] * b[1 * 3 + j] + a[i * 3 + 2] * b[2 * 3 + j];
}

template <class T>
cudaError_t upload_vec(T **dst, const std::vector<T> &src) {
  cudaError_t e = cudaMalloc(dst, sizeof(T) * std::max<size_t>(src.size(), 1));
  if (e == cudaSuccess && !src.empty())
    e = cudaMemcpy(*dst, src.data(), sizeof(T) * src.size(), cudaMemcpyHostToDevice);
  return e;
}

template <class T>
cudaError_t download_vec(std::vector<T> *dst, const T *src, size_t n) {
  dst->resize(n);
  if (n == 0) return cudaSuccess;
  return cudaMemcpy(dst->data(), src, sizeof(T) * n, cudaMemcpyDeviceToHost);
}

}  // namespace

void release_viscosity(mcfd_handle *h) {
  Visc &v = h->visc;
  void *ptrs[] = {v.nu, v.side, v.pt, v.cell, v.d2, v.wloc, v.rate_count, v.rate_cell, v.rate_data};
  for (void *p : ptrs)
    if (p) cudaFree(p);
  v = Visc{};
}

int build_viscosity(mcfd_handle *h, double beta0, double beta1, double time_scale) {
  Mesh &m = h->mesh;
  const int Q = m.q, N = m.n, QF = m.qf;
  const int64_t nc = m.n_cells, nf = m.n_faces, np = m.n_points;
  if (m.host_corners.size() != (size_t)nc * 24) {
    h->err = "the handle keeps no corner coordinates";
    return MCFD_ERR_MESH;
  }
  double xq[4], wq[4], D[16], D2[16];
  for (int i = 0; i < Q; ++i) xq[i] = m.xq[i];
  gll_weights(Q, wq);
  std::vector<double> dm;
  std::vector<int2> fcells;
  std::vector<double4> fgeo;
  cudaError_t e = download_vec(&dm, m.dmat, (size_t)Q * Q);
  if (e == cudaSuccess) e = download_vec(&fcells, m.face_cells, (size_t)nf);
  if (e == cudaSuccess) e = download_vec(&fgeo, m.face_geo, (size_t)np);
  if (e != cudaSuccess) {
    h->err = std::string("viscosity set-up download: ") + cudaGetErrorString(e);
    return MCFD_ERR_CUDA;
  }
  for (int i = 0; i < Q * Q; ++i) D[i] = dm[i];
  // second derivatives of the degree-p interpolant: D applied twice
  for (int a = 0; a < Q; ++a)
    for (int i = 0; i < Q; ++i) {
      double s = 0;
      for (int b = 0; b < Q; ++b) s += D[a * Q + b] * D[b * Q + i];
      D2[a * Q + i] = s;
    }
  std::vector<double> wloc(N);
  for (int i = 0; i < Q; ++i)
    for (int j = 0; j < Q; ++j)
      for (int k = 0; k < Q; ++k) wloc[(i * Q + j) * Q + k] = wq[i] * wq[j] * wq[k];
  // cells: volume, length, centre
  std::vector<double> cell(nc * 2), volume(nc), center(nc * 3);
  const int p = m.p;
#pragma omp parallel for schedule(static)
  for (int64_t c = 0; c < nc; ++c) {
    const double *xn = &m.host_corners[c * 24];
    double vol = 0;
    for (int i = 0; i < Q; ++i)
      for (int j = 0; j < Q; ++j)
        for (int k = 0; k < Q; ++k) {
          const double loc[3] = {xq[i], xq[j], xq[k]};
          double x[3], J[9], dJ[27], inv[9];
          hex8_map(xn, loc, x, J, dJ);
          const double det = inverse3(J, inv);
          vol += wq[i] * wq[j] * wq[k] * det;
        }
    volume[c] = vol;
    const double L = std::cbrt(vol) * 0.5;
    cell[c * 2 + 0] = L;
    cell[c * 2 + 1] = std::pow(L, (p + 1) + 3);
    const double zero[3] = {0, 0, 0};
    double J[9], dJ[27];
    hex8_map(xn, zero, &center[c * 3], J, dJ);
  }
  // face points and sides
  std::vector<double> pt(np * 4, 0.0), side(np * 12, 0.0);
  const bool shifted = m.host_shift.size() == (size_t)nf * 3;
  if (m.host_face_sides.size() != (size_t)nf * 2) {
    h->err = "the handle keeps no face sides";
    return MCFD_ERR_MESH;
  }
  int bad = 0;
#pragma omp parallel for schedule(static) reduction(| : bad)
  for (int64_t f = 0; f < nf; ++f) {
    const int2 fc = fcells[f];
    double area = 0;
    for (int a = 0; a < Q; ++a)
      for (int b = 0; b < Q; ++b) area += wq[a] * wq[b] * fgeo[f * QF + a * Q + b].w;
    double hs[3];
    const double *ch = &center[(int64_t)fc.x * 3];
    if (fc.y >= 0) {
      for (int d = 0; d < 3; ++d)
        hs[d] = (center[(int64_t)fc.y * 3 + d] + (shifted ? m.host_shift[f * 3 + d] : 0.0)) - ch[d];
    } else {
      const int sd = m.host_face_sides[f * 2];
      const double *xn = &m.host_corners[(int64_t)fc.x * 24];
      for (int d = 0; d < 3; ++d) {
        double cen = 0;
        for (int w = 0; w < 4; ++w) cen += xn[kFaceCorners[sd][w] * 3 + d];
        cen *= 0.25;
        hs[d] = (cen - ch[d]) * 2;
      }
    }
    for (int a = 0; a < Q; ++a)
      for (int b = 0; b < Q; ++b) {
        const int64_t id = f * QF + a * Q + b;
        const double4 g = fgeo[id];
        const double n[3] = {g.x, g.y, g.z};
        const double dist = n[0] * hs[0] + n[1] * hs[1] + n[2] * hs[2];
        if (!(dist > 0)) bad = 1;
        const double wf = wq[a] * wq[b] * g.w;
        pt[id * 4 + 0] = beta0 / dist;
        pt[id * 4 + 1] = beta1 * dist;
        pt[id * 4 + 2] = wf * (volume[fc.x] / area);
        pt[id * 4 + 3] = fc.y >= 0 ? wf * (volume[fc.y] / area) : 0.0;
        for (int role = 0; role < 2; ++role) {
          const int64_t cell_id = role ? fc.y : fc.x;
          if (cell_id < 0) continue;
          const int node = role ? m.map_s[id] : m.map_h[id];
          const int i = node / QF, j = (node / Q) % Q, k = node % Q;
          const double loc[3] = {xq[i], xq[j], xq[k]};
          double x[3], J[9], dJ[27], inv[9];
          hex8_map(&m.host_corners[cell_id * 24], loc, x, J, dJ);
          inverse3(J, inv);
          double mv[3], qv[3] = {0, 0, 0};
          for (int r = 0; r < 3; ++r) mv[r] = inv[0 * 3 + r] * n[0] + inv[1 * 3 + r] * n[1] + inv[2 * 3 + r] * n[2];
          for (int r = 0; r < 3; ++r) {
            // (d_r J^-1)^T n = -(J^-1 d_r J J^-1)^T n
            double t1[9], bm[9];
            mul3(inv, &dJ[r * 9], t1);
            mul3(t1, inv, bm);
            for (int e = 0; e < 3; ++e)
              qv[e] += mv[r] * -(bm[0 * 3 + e] * n[0] + bm[1 * 3 + e] * n[1] + bm[2 * 3 + e] * n[2]);
          }
          double *sg = &side[(id * 2 + role) * 6];
          for (int e = 0; e < 3; ++e) { sg[e] = mv[e]; sg[3 + e] = qv[e]; }
        }
      }
  }
  if (bad) {
    h->err = "a face point has a non-positive holder-to-sharer distance";
    return MCFD_ERR_MESH;
  }
  release_viscosity(h);
  Visc &v = h->visc;
  v.beta0 = beta0;
  v.beta1 = beta1;
  v.time_scale = time_scale;
  std::vector<double> d2(D2, D2 + Q * Q);
  e = upload_vec(&v.side, side);
  if (e == cudaSuccess) e = upload_vec(&v.pt, pt);
  if (e == cudaSuccess) e = upload_vec(&v.cell, cell);
  if (e == cudaSuccess) e = upload_vec(&v.d2, d2);
  if (e == cudaSuccess) e = upload_vec(&v.wloc, wloc);
  if (e == cudaSuccess) e = cudaMalloc(&v.nu, sizeof(double) * kK * std::max<int64_t>(nc, 1));
  if (e == cudaSuccess) e = cudaMemset(v.nu, 0, sizeof(double) * kK * std::max<int64_t>(nc, 1));
  if (e == cudaSuccess) e = cudaMalloc(&v.rate_count, sizeof(unsigned));
  if (e == cudaSuccess) e = cudaMalloc(&v.rate_cell, sizeof(int32_t) * std::max<int64_t>(nc, 1));
  if (e == cudaSuccess) e = cudaMalloc(&v.rate_data, sizeof(double) * kViscRateData * std::max<int64_t>(nc, 1));
  if (e == cudaSuccess) {
    int sms = 0;
    e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, h->device);
    v.rate_blocks = std::max(sms, 1) * visc_rate_blocks_per_sm(Q);
  }
  if (e == cudaSuccess) {
    const double init = 1.e+100;
    unsigned long long bits;
    std::memcpy(&bits, &init, sizeof(bits));
    e = cudaMemcpy(&h->buf.state->min_dt_bits, &bits, sizeof(bits), cudaMemcpyHostToDevice);
  }
  if (e != cudaSuccess) {
    release_viscosity(h);
    h->err = std::string("viscosity set-up: ") + cudaGetErrorString(e);
    return MCFD_ERR_CUDA;
  }
  v.on = true;
  return MCFD_OK;
}

}  // namespace mcfd
