// Device probes: the flux routines and the hand-written arithmetic of the
// face and cell kernels, evaluated on caller-owned device arrays.
//
// The face kernels evaluate interior_flux_weighted / flux_boundary on states
// that they gather from the solution column; these probes call the same
// device functions (the same template instances: solver, FP64 or mixed form)
// on states given point by point, so that the reference's known-answer
// Riemann problems (test/riemann/euler/{exact,hllc,ausm}.cpp: strong shocks,
// blast waves, vacuum and near-vacuum states) and states that the positivity
// clamp zeroes (riemann/euler/types.hpp:194-202) reach the device code paths
// without a mesh whose cells would first have to hold them.
//
// mcfd_probe_numerics evaluates the arithmetic that replaces CUDA's own
// operators on the FP64-bound paths (Newton reciprocals, the seeded square
// root, the integer-pipe FP64 <-> FP32 conversions, the Exact solver's
// inverse-root powers) next to CUDA's operators on the same inputs.
#include <cuda_runtime.h>

#include <cstdint>

#include "../../include/mcfd.h"
#include "euler.cuh"
#include "handle.hpp"

namespace mcfd {
namespace {

template <int R, bool FAST_SQRT>
__global__ void __launch_bounds__(256)
probe_flux_kernel(int bc_kind, int64_t n, const double *left, const double *right,
                  const double *normal, double *flux, unsigned *status) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double cl[kK], cr[kK], out[kK];
#pragma unroll
  for (int k = 0; k < kK; ++k) {
    cl[k] = left[i * kK + k];
    cr[k] = right[i * kK + k];
  }
  const double nv[3] = {normal[i * 3], normal[i * 3 + 1], normal[i * 3 + 2]};
  bool not_converged = false;
  if (bc_kind == kBcNone) {
    interior_flux_weighted<R, FAST_SQRT>(cl, cr, nv, 1.0, out, &not_converged);
  } else {
    const Prim in = cons_to_prim(cl[0], cl[1], cl[2], cl[3], cl[4]);
    flux_boundary<R>(bc_kind, in, cr, nv, out, &not_converged);
  }
  if (not_converged) atomicOr(status, (unsigned)kStatusNotConverged);
#pragma unroll
  for (int k = 0; k < kK; ++k) flux[i * kK + k] = out[k];
}

__global__ void __launch_bounds__(256)
probe_numerics_kernel(int op, int64_t n, const void *in, void *out) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double *x = static_cast<const double *>(in);
  const float *xf = static_cast<const float *>(in);
  double *y = static_cast<double *>(out);
  float *yf = static_cast<float *>(out);
  switch (op) {
    case MCFD_PROBE_RCP: y[i] = rcp_newton(x[i]); break;
    case MCFD_PROBE_RCP_SIGNED: y[i] = rcp_signed(x[i]); break;
    case MCFD_PROBE_SQRT_SEEDED: y[i] = sqrt_seeded(x[i]); break;
    case MCFD_PROBE_F64_TO_F32: yf[i] = f64_to_f32(x[i]); break;
    case MCFD_PROBE_F32_TO_F64: y[i] = f32_to_f64(xf[i]); break;
    case MCFD_PROBE_CUDA_RCP: y[i] = 1.0 / x[i]; break;
    case MCFD_PROBE_CUDA_SQRT: y[i] = sqrt(x[i]); break;
    case MCFD_PROBE_CUDA_F64_TO_F32: yf[i] = __double2float_rn(x[i]); break;
    case MCFD_PROBE_CUDA_F32_TO_F64: y[i] = (double)xf[i]; break;
    case MCFD_PROBE_RCP1: y[i] = rcp_newton1(x[i]); break;
    case MCFD_PROBE_ROOT7: y[i] = ex_root7(x[i]); break;
    case MCFD_PROBE_ROOT7_OVER_X: {
      double r67;
      ex_root7(x[i], &r67);
      y[i] = r67;
      break;
    }
    case MCFD_PROBE_POW_NEG_GAMMA: y[i] = ex_isentrope(1.0, x[i]); break;
    case MCFD_PROBE_CUDA_POW_ROOT7: y[i] = pow(x[i], kGm1Over2 / kGamma); break;
    case MCFD_PROBE_CUDA_POW_NEG_GAMMA: y[i] = 1.0 / pow(x[i], kGamma); break;
    default: break;
  }
}

template <int R>
void launch_probe_flux(int fast, int bc_kind, int64_t n, const double *l, const double *r,
                       const double *nv, double *f, unsigned *status) {
  const unsigned blocks = (unsigned)((n + 255) / 256);
  if (fast)
    probe_flux_kernel<R, true><<<blocks, 256>>>(bc_kind, n, l, r, nv, f, status);
  else
    probe_flux_kernel<R, false><<<blocks, 256>>>(bc_kind, n, l, r, nv, f, status);
}

}  // namespace
}  // namespace mcfd

extern "C" int mcfd_probe_flux(int32_t device, int32_t riemann, int32_t precision,
                               int32_t bc_kind, int64_t n, const double *d_left,
                               const double *d_right, const double *d_normal,
                               double *d_flux, uint32_t *status) {
  if (n < 0 || n > (int64_t)INT32_MAX * 256 || riemann < MCFD_EXACT || riemann > MCFD_RUSANOV ||
      (precision != MCFD_FP64 && precision != MCFD_MIXED) || bc_kind < MCFD_BC_NONE ||
      bc_kind > MCFD_BC_SMART)
    return MCFD_ERR_ARGUMENT;
  if (n > 0 && (!d_left || !d_right || !d_normal || !d_flux)) return MCFD_ERR_ARGUMENT;
  if (status) *status = 0;
  if (n == 0) return MCFD_OK;
  mcfd::DeviceGuard guard(device);
  unsigned *d_status = nullptr;
  if (cudaMallocAsync(&d_status, sizeof(unsigned), 0) != cudaSuccess) return MCFD_ERR_CUDA;
  cudaMemsetAsync(d_status, 0, sizeof(unsigned), 0);
  const int fast = precision == MCFD_MIXED;
  switch (riemann) {
    case MCFD_EXACT: mcfd::launch_probe_flux<mcfd::kExact>(fast, bc_kind, n, d_left, d_right, d_normal, d_flux, d_status); break;
    case MCFD_HLLC: mcfd::launch_probe_flux<mcfd::kHllc>(fast, bc_kind, n, d_left, d_right, d_normal, d_flux, d_status); break;
    case MCFD_AUSM: mcfd::launch_probe_flux<mcfd::kAusm>(fast, bc_kind, n, d_left, d_right, d_normal, d_flux, d_status); break;
    case MCFD_ROE: mcfd::launch_probe_flux<mcfd::kRoe>(fast, bc_kind, n, d_left, d_right, d_normal, d_flux, d_status); break;
    default: mcfd::launch_probe_flux<mcfd::kRusanov>(fast, bc_kind, n, d_left, d_right, d_normal, d_flux, d_status); break;
  }
  unsigned st = 0;
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaMemcpyAsync(&st, d_status, sizeof(unsigned), cudaMemcpyDeviceToHost, 0);
  cudaFreeAsync(d_status, 0);
  if (e == cudaSuccess) e = cudaStreamSynchronize(0);
  if (e != cudaSuccess) return MCFD_ERR_CUDA;
  if (status) *status = st;
  return (st & mcfd::kStatusNotConverged) ? MCFD_ERR_NOT_CONVERGED : MCFD_OK;
}

extern "C" int mcfd_probe_numerics(int32_t device, int32_t op, int64_t n, const void *d_in,
                                   void *d_out) {
  if (n < 0 || n > (int64_t)INT32_MAX * 256 || op < MCFD_PROBE_RCP || op > MCFD_PROBE_CUDA_POW_NEG_GAMMA)
    return MCFD_ERR_ARGUMENT;
  if (n == 0) return MCFD_OK;
  if (!d_in || !d_out) return MCFD_ERR_ARGUMENT;
  mcfd::DeviceGuard guard(device);
  mcfd::probe_numerics_kernel<<<(unsigned)((n + 255) / 256), 256>>>(op, n, d_in, d_out);
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaStreamSynchronize(0);
  return e == cudaSuccess ? MCFD_OK : MCFD_ERR_CUDA;
}
