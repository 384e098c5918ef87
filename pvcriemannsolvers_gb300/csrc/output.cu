// Output and restart kernels on sm_103a.
//
//   fields_transpose_kernel  the solution column [cells][F] (F values per
//                            cell) <-> the DataOnCells fields [F][cells] of
//                            Part::GatherSolutions / ScatterSolutions
//                            (mesh/part.hpp:380-395, 1061-1069): a 32 x 32
//                            tile through shared memory, both sides coalesced.
//                            HBM-bound: 16 B per value (one read, one write).
//   vtk_sample_kernel<Q>     Writer<Part>::Prepare (mesh/vtk.hpp:428-493) for
//                            the nodal schemes: one thread per (cell, VTK
//                            node) evaluates the Hex8 map and the GLL Lagrange
//                            interpolant at the Hexahedron27 local points
//                            (LocalToGlobalAndValue).
// The modal scheme's sampling lives with its basis helpers in modal.cu.
#include <cuda_runtime.h>

#include <cstdint>

#include "euler.cuh"
#include "handle.hpp"
#include "vtk_locals.cuh"

namespace mcfd {

namespace {

constexpr int kTile = 32;
constexpr int kTileRows = 8;

// TO_FIELDS: src = column [cells][F], dst = fields [F][cells]; else the reverse.
template <bool TO_FIELDS>
__global__ void __launch_bounds__(kTile * kTileRows)
fields_transpose_kernel(const double *__restrict__ src, double *__restrict__ dst,
                        int64_t n_cells, int n_fields) {
  __shared__ double tile[kTile][kTile + 1];
  const int64_t c0 = (int64_t)blockIdx.x * kTile;
  const int f0 = blockIdx.y * kTile;
  const int tx = threadIdx.x;
  // load: tile[r][tx] = value (cell c0 + r, field f0 + tx) for the column,
  //       value (field f0 + r, cell c0 + tx) for the fields
  for (int r = threadIdx.y; r < kTile; r += kTileRows) {
    if (TO_FIELDS) {
      const int64_t c = c0 + r;
      const int f = f0 + tx;
      if (c < n_cells && f < n_fields) tile[r][tx] = src[c * n_fields + f];
    } else {
      const int f = f0 + r;
      const int64_t c = c0 + tx;
      if (c < n_cells && f < n_fields) tile[r][tx] = src[(int64_t)f * n_cells + c];
    }
  }
  __syncthreads();
  for (int r = threadIdx.y; r < kTile; r += kTileRows) {
    if (TO_FIELDS) {
      const int f = f0 + r;
      const int64_t c = c0 + tx;
      if (c < n_cells && f < n_fields) dst[(int64_t)f * n_cells + c] = tile[tx][r];
    } else {
      const int64_t c = c0 + r;
      const int f = f0 + tx;
      if (c < n_cells && f < n_fields) dst[c * n_fields + f] = tile[tx][r];
    }
  }
}

struct SampleArgs {
  const double *u;
  const double *corners;
  const int64_t *off;  // point offset of each cell (null: 27 per cell)
  double *xyz;
  double *values;
  int64_t n_cells;
  double xq[4];
  int points_given;  // curved cells: xyz holds the points already (host-mapped)
};

template <int Q>
__global__ void __launch_bounds__(256) vtk_sample_kernel(SampleArgs a) {
  constexpr int N = Q * Q * Q;
  const int64_t gid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t c = gid / 27;
  const int s = (int)(gid - c * 27);
  if (c >= a.n_cells) return;
  const double loc[3] = {(double)kVtkHex27[s][0], (double)kVtkHex27[s][1],
                         (double)kVtkHex27[s][2]};
  // Hex8 map (coordinate/hexahedron.hpp:397-527 shape functions)
  const double *xn = a.corners + c * 24;
  double g[3] = {0, 0, 0};
#pragma unroll
  for (int v = 0; v < 8; ++v) {
    const double w = (1 + kVtkHex27[v][0] * loc[0]) * (1 + kVtkHex27[v][1] * loc[1]) *
                     (1 + kVtkHex27[v][2] * loc[2]) * 0.125;
#pragma unroll
    for (int e = 0; e < 3; ++e) g[e] += xn[v * 3 + e] * w;
  }
  // GLL Lagrange weights per direction (basis/lagrange.hpp:53-142)
  double lw[3][Q];
#pragma unroll
  for (int d = 0; d < 3; ++d)
#pragma unroll
    for (int i = 0; i < Q; ++i) {
      double l = 1;
#pragma unroll
      for (int m = 0; m < Q; ++m)
        if (m != i) l *= (loc[d] - a.xq[m]) / (a.xq[i] - a.xq[m]);
      lw[d][i] = l;
    }
  double v[kK] = {0, 0, 0, 0, 0};
  const double *uc = a.u + c * N * kK;
#pragma unroll
  for (int i = 0; i < Q; ++i)
#pragma unroll
    for (int j = 0; j < Q; ++j)
#pragma unroll
      for (int k = 0; k < Q; ++k) {
        const double w = lw[0][i] * lw[1][j] * lw[2][k];
        const double *un = uc + ((i * Q + j) * Q + k) * kK;
#pragma unroll
        for (int e = 0; e < kK; ++e) v[e] += w * un[e];
      }
  const int64_t pt = (a.off ? a.off[c] : c * 27) + s;
  if (!a.points_given) {
#pragma unroll
    for (int e = 0; e < 3; ++e) a.xyz[pt * 3 + e] = g[e];
  }
#pragma unroll
  for (int e = 0; e < kK; ++e) a.values[pt * kK + e] = v[e];
}

}  // namespace

int launch_fields_transpose(mcfd_handle *h, const double *src, double *dst, int to_fields) {
  const int64_t nc = h->mesh.n_cells;
  const int nf = (int)(h->mesh.column / nc);
  const dim3 block(kTile, kTileRows);
  const dim3 grid((unsigned)((nc + kTile - 1) / kTile), (unsigned)((nf + kTile - 1) / kTile));
  if (to_fields)
    fields_transpose_kernel<true><<<grid, block, 0, h->stream>>>(src, dst, nc, nf);
  else
    fields_transpose_kernel<false><<<grid, block, 0, h->stream>>>(src, dst, nc, nf);
  return 1;
}

int launch_vtk_sample(mcfd_handle *h, const double *u, const int64_t *off, double *xyz,
                      double *values) {
  if (h->opt.scheme == 2) return launch_modal_vtk_sample(h, u, off, xyz, values);
  const Mesh &m = h->mesh;
  SampleArgs a{u, m.corners, off, xyz, values, m.n_cells, {m.xq[0], m.xq[1], m.xq[2], m.xq[3]},
               m.curved ? 1 : 0};
  const int64_t threads = m.n_cells * 27;
  const unsigned blocks = (unsigned)((threads + 255) / 256);
  switch (m.q) {
    case 2: vtk_sample_kernel<2><<<blocks, 256, 0, h->stream>>>(a); break;
    case 3: vtk_sample_kernel<3><<<blocks, 256, 0, h->stream>>>(a); break;
    default: vtk_sample_kernel<4><<<blocks, 256, 0, h->stream>>>(a); break;
  }
  return 1;
}

}  // namespace mcfd
