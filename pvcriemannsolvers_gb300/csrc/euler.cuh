// Ideal-gas Euler physics for the device kernels (and host helpers).
//
// All functions work in the GLOBAL frame with the unit face normal only.  The
// reference rotates momenta into an orthonormal frame (n, t, b), calls a 1D
// solver with passive tangential velocities and rotates the flux back
// (include/mini/riemann/rotated/euler.hpp:68-88, 117-159).  Every solver used
// here is invariant under rotations about n, so with u_t = u - (u.n) n the
// rotated flux equals
//     F = F_1D[mass, normal momentum, energy] + (tangential part carried by
//         the upwind/star state)
// evaluated directly in global coordinates.  This needs 3 normal components
// per face point instead of a 9-entry frame and skips both rotations; the
// results agree with the rotated form to rounding.
//
// Sources restated (pvcStillInGradSchool/pvcRiemannSolvers):
//   gas                include/mini/riemann/euler/types.hpp:186-334
//   Exact              include/mini/riemann/euler/exact.hpp:44-320
//   HLLC               include/mini/riemann/euler/hllc.hpp:30-109
//   AUSM               include/mini/riemann/euler/ausm.hpp:146-187
//   Roe, Rusanov       python/riemann.py:405-476 (1D), here in 3D
//   boundary fluxes    include/mini/riemann/rotated/euler.hpp:144-318
#pragma once

#include <cmath>
#include <cstdint>

#ifdef __CUDACC__
#define MCFD_HD __host__ __device__ __forceinline__
#else
#define MCFD_HD inline
#endif

namespace mcfd {

constexpr int kK = 5;
constexpr double kGamma = 1.4;
constexpr double kGasR = 287.05;
constexpr double kGm1 = kGamma - 1.0;             // GammaMinusOne
constexpr double kGp1 = kGamma + 1.0;             // GammaPlusOne
constexpr double kOneOverGm1 = 1.0 / kGm1;        // OneOverGammaMinusOne
constexpr double kGm1Under2 = 2 / kGm1;           // GammaMinusOneUnderTwo
constexpr double kGm1Over2 = kGm1 / 2;            // GammaMinusOneOverTwo
constexpr double kGp1Over2 = kGp1 / 2;            // GammaPlusOneOverTwo
constexpr double kGp1Over4 = kGp1 / 4;            // GammaPlusOneOverFour
constexpr double kOneOverGamma = 1 / kGamma;      // OneOverGamma
constexpr double kGammaOverGm1 = kGamma / kGm1;   // GammaOverGammaMinusOne

enum Riemann { kExact = 0, kHllc = 1, kAusm = 2, kRoe = 3, kRusanov = 4 };
enum BcKind {
  kBcNone = 0, kBcInviscidWall = 1, kBcSupersonicInlet = 2,
  kBcSupersonicOutlet = 3, kBcSubsonicInlet = 4, kBcSubsonicOutlet = 5,
  kBcSmart = 6,
  kBcNoSlipWall = 7  // viscous fr::Lobatto only (fr/general.hpp:455-476)
};

// Status bits raised by kernels (read back by the host).
enum StatusBits : unsigned {
  kStatusNonFinite = 1u,
  kStatusNotConverged = 2u,
  kStatusTimeout = 4u,
};

struct Prim {
  double rho, u, v, w, p;
  double rinv;  // 1 / rho when rho > 0, else 0 (saves divisions downstream)
};

#ifdef __CUDA_ARCH__
__device__ __forceinline__ double rcp_newton(double x);
#else
inline double rcp_newton(double x);
#endif

MCFD_HD Prim make_prim(double rho, double u, double v, double w, double p) {
  return Prim{rho, u, v, w, p, rho > 0 ? rcp_newton(rho) : 0.0};
}

// x < 0, x > 0 and x != 0 with IEEE results (-0, infinities, NaN) decided on
// the bit pattern: on the device these run on the integer pipes instead of
// taking FP64 compare slots on the FP64 unit, which bounds the FP64 kernels.
#ifdef __CUDACC__
// The bit pattern of x through an opaque move: the integer tests below stay
// integer operations instead of being folded back into FP64 compares, which
// would issue on the FP64 pipe.
__device__ __forceinline__ unsigned long long bits64(double x) {
#ifdef __CUDA_ARCH__
  unsigned long long r;
  asm("mov.b64 %0, %1;" : "=l"(r) : "d"(x));
  return r;
#else
  return (unsigned long long)__double_as_longlong(x);
#endif
}
#endif
#ifdef __CUDA_ARCH__
__device__ __forceinline__ bool lt_zero(double x) {
  // negative finite or -inf: bit patterns 0x8000000000000001 .. 0xfff0000000000000
  return bits64(x) - 0x8000000000000001ull < 0x7ff0000000000000ull;
}
__device__ __forceinline__ bool gt_zero(double x) {
  // positive finite or +inf: 0x0000000000000001 .. 0x7ff0000000000000
  return bits64(x) - 1ull < 0x7ff0000000000000ull;
}
__device__ __forceinline__ bool ne_zero(double x) { return (bits64(x) << 1) != 0; }
__device__ __forceinline__ bool ge_zero(double x) {
  // +0 .. +inf, or -0
  const unsigned long long b = bits64(x);
  return b <= 0x7ff0000000000000ull || b == 0x8000000000000000ull;
}
__device__ __forceinline__ bool le_zero(double x) {
  // -0 .. -inf, or +0
  const unsigned long long b = bits64(x);
  return b - 0x8000000000000000ull <= 0x7ff0000000000000ull || b == 0ull;
}
// a <= b for a, b >= 0 (either zero's sign), compared as unsigned integers
__device__ __forceinline__ bool le_nonneg(double a, double b) {
  return (bits64(a) & 0x7fffffffffffffffull) <= (bits64(b) & 0x7fffffffffffffffull);
}
#else
inline bool lt_zero(double x) { return x < 0; }
inline bool gt_zero(double x) { return x > 0; }
inline bool ne_zero(double x) { return x != 0; }
inline bool ge_zero(double x) { return 0.0 <= x; }
inline bool le_zero(double x) { return x <= 0.0; }
inline bool le_nonneg(double a, double b) { return a <= b; }
#endif

// ConservativeToPrimitive with SetZeroIfNegative (types.hpp:194-202,288-301):
// a negative density or (first) energy, or a negative pressure after the
// conversion, zeroes the whole primitive state.  The three velocity
// divisions share one reciprocal.
MCFD_HD Prim cons_to_prim(double r, double mx, double my, double mz,
                          double e) {
  Prim w{r, mx, my, mz, e, 0.0};
  if (lt_zero(r) || lt_zero(e)) return Prim{0, 0, 0, 0, 0, 0};
  if (ne_zero(r)) {
    double inv = rcp_newton(r);
    w.rinv = inv;
    w.u = mx * inv;
    w.v = my * inv;
    w.w = mz * inv;
    double ke = 0.5 * (w.u * w.u + w.v * w.v + w.w * w.w);
    w.p = (e - r * ke) * kGm1;
    if (lt_zero(w.p)) return Prim{0, 0, 0, 0, 0, 0};
  }
  return w;
}

MCFD_HD double kinetic(const Prim &w) {
  return 0.5 * (w.u * w.u + w.v * w.v + w.w * w.w);
}

// GetSpeedOfSound(rho, p) (types.hpp:252-254).
MCFD_HD double sound_speed(const Prim &w) {
  return (gt_zero(w.rho) && gt_zero(w.p)) ? sqrt(kGamma * w.p * w.rinv) : 0.0;
}

// Total energy of a primitive state (PrimitiveToConservative, types.hpp:302-311).
MCFD_HD double prim_energy(const Prim &w) {
  return w.p * kOneOverGm1 + w.rho * kinetic(w);
}

// Physical flux through unit normal n, from a primitive state:
// the global-frame form of PrimitiveToFlux in the normal frame.
MCFD_HD void normal_flux(const Prim &w, double e, const double *n, double un,
                         double *f) {
  f[0] = w.rho * un;
  f[1] = w.rho * w.u * un + w.p * n[0];
  f[2] = w.rho * w.v * un + w.p * n[1];
  f[3] = w.rho * w.w * un + w.p * n[2];
  f[4] = (e + w.p) * un;
}

// ---------------------------------------------------------------- Rusanov
// Rusanov on conservative inputs: for a converted state (rho > 0, p >= 0)
// F_n = (m.n, m (m.n)/rho + p n, (E + p)(m.n)/rho) and U is the input itself,
// so no velocity vector is formed (u = m/rho appears only through m.n/rho).
// Degenerate (clamped or rho == 0) states fall back to the primitive form.
// Equal to flux_rusanov on the converted primitives up to rounding.
// 1/x for x > 0 with the FP64 pipe used only for two Newton-Raphson steps
// y <- y + y (1 - x y) (quadratic convergence: 2^-22 seed -> 2^-88, i.e.
// within an ulp of the rounded quotient).  The seed is the FP32 hardware
// reciprocal of x rounded to FP32, converted on the integer pipes.  Outside
// the normal FP32 range the plain FP64 division is used.
// FP64 <-> FP32 conversions on the integer pipes.  On this part the FP64
// unit is the bottleneck and hardware F2F conversions issue there.  These
// follow the IEEE-754 binary64/binary32 layouts with branch-free selects:
// round to nearest even, subnormal results flushed to a signed zero,
// overflow to infinity, NaN kept NaN.
__device__ __forceinline__ float f64_to_f32(double x) {
  const unsigned long long b = bits64(x);
  const unsigned sign = (unsigned)(b >> 32) & 0x80000000u;
  const int ex = (int)((b >> 52) & 0x7ff);
  const int e = ex - (1023 - 127);
  const unsigned long long mant = b & 0xFFFFFFFFFFFFFull;
  const unsigned long long rounded = mant + 0xFFFFFFFull + ((mant >> 29) & 1ull);
  // a mantissa carry (rounded >> 29 == 2^23) increments the exponent field
  unsigned bits = ((unsigned)e << 23) + (unsigned)(rounded >> 29);
  bits = e <= 0 ? 0u : bits;
  const unsigned special = 0x7f800000u | ((ex == 0x7ff && mant != 0ull) ? 0x400000u : 0u);
  bits = e >= 255 ? special : bits;
  return __uint_as_float(sign | bits);
}

__device__ __forceinline__ double f32_to_f64(float f) {
  const unsigned b = __float_as_uint(f);
  const unsigned e = (b >> 23) & 0xffu;
  const unsigned long long m = (unsigned long long)(b & 0x7fffffu) << 29;
  unsigned long long r = ((unsigned long long)(e + (1023u - 127u)) << 52) | m;
  r = e == 0u ? 0ull : r;
  r = e == 0xffu ? ((0x7ffull << 52) | m) : r;
  return __longlong_as_double((long long)(r | ((unsigned long long)(b & 0x80000000u) << 32)));
}

// x != 0 on the bit pattern.
__device__ __forceinline__ bool nonzero64(double x) {
  return (bits64(x) << 1) != 0;
}

// x < 0 for a finite or infinite double, tested on the bit pattern.
__device__ __forceinline__ bool negative64(double x) {
  const long long b = (long long)bits64(x);
  return b < 0 && (b << 1) != 0;
}

// isfinite on the bit pattern (exponent field not all ones).
__device__ __forceinline__ bool finite64(double x) {
  return ((bits64(x) >> 52) & 0x7ff) != 0x7ff;
}

#ifdef __CUDA_ARCH__
__device__ __forceinline__ double rcp_newton(double x) {
  const unsigned long long b = bits64(x);
  const int e = (int)((b >> 52) & 0x7ff) - (1023 - 127);
  if (e <= 1 || e >= 253) return 1.0 / x;
  const unsigned long long mant = b & 0xFFFFFFFFFFFFFull;
  const float xf = __uint_as_float(((unsigned)e << 23) + (unsigned)(mant >> 29));
  const unsigned yb = __float_as_uint(__frcp_rn(xf));
  const unsigned ye = (yb >> 23) & 0xffu;
  double y = __longlong_as_double((long long)(
      ((unsigned long long)(ye + (1023u - 127u)) << 52) |
      ((unsigned long long)(yb & 0x7fffffu) << 29)));
  double d = fma(-x, y, 1.0);
  y = fma(y, d, y);
  d = fma(-x, y, 1.0);
  return fma(y, d, y);
}
// rcp_newton with one Newton-Raphson step (relative error below 4e-14, the
// square of the FP32 seed's 1.8e-7): the mixed form's node traces, where the
// seeded square root beside it carries 1.4e-13.
__device__ __forceinline__ double rcp_newton1(double x) {
  const unsigned long long b = bits64(x);
  const int e = (int)((b >> 52) & 0x7ff) - (1023 - 127);
  if (e <= 1 || e >= 253) return 1.0 / x;
  const unsigned long long mant = b & 0xFFFFFFFFFFFFFull;
  const float xf = __uint_as_float(((unsigned)e << 23) + (unsigned)(mant >> 29));
  const unsigned yb = __float_as_uint(__frcp_rn(xf));
  const unsigned ye = (yb >> 23) & 0xffu;
  const double y = __longlong_as_double((long long)(
      ((unsigned long long)(ye + (1023u - 127u)) << 52) |
      ((unsigned long long)(yb & 0x7fffffu) << 29)));
  return fma(y, fma(-x, y, 1.0), y);
}
// Square root for the mixed form's wave speed: one Newton-Raphson step on
// the reciprocal square root, y <- y + y (1 - x y^2) / 2, from the FP32
// hardware estimate of 1/sqrt(x) (relative error below 3e-7, so ~1.4e-13
// after the step), then sqrt(x) = x y.  Written on t = x y0:
//   sqrt(x) = t + t (1/2 - t y0 / 2),
// three FP64 operations, with -y0/2 scaled in FP32 (exact) before its
// conversion.  Outside the normal FP32 range the FP64 square root is used.
__device__ __forceinline__ double sqrt_seeded(double x) {
  const unsigned long long b = bits64(x);
  const int e = (int)((b >> 52) & 0x7ff) - (1023 - 127);
  if (e <= 1 || e >= 253) return sqrt(x);
  const unsigned long long mant = b & 0xFFFFFFFFFFFFFull;
  const float xf = __uint_as_float(((unsigned)e << 23) + (unsigned)(mant >> 29));
  const float yf = rsqrtf(xf);
  // both normal: 1/sqrt(x) of a normal x in [2^-125, 2^126) is within [2^-63, 2^63)
  const unsigned yb = __float_as_uint(yf), hb = __float_as_uint(-0.5f * yf);
  const double y0 = __longlong_as_double((long long)(
      ((unsigned long long)(((yb >> 23) & 0xffu) + (1023u - 127u)) << 52) |
      ((unsigned long long)(yb & 0x7fffffu) << 29)));
  const double yh = __longlong_as_double((long long)(
      0x8000000000000000ull |
      ((unsigned long long)(((hb >> 23) & 0xffu) + (1023u - 127u)) << 52) |
      ((unsigned long long)(hb & 0x7fffffu) << 29)));
  const double t = x * y0;
  return fma(t, fma(t, yh, 0.5), t);
}

// Sign tests on the bit patterns (integer pipes): x > 0 and x < 0 for
// finite or infinite x.
__device__ __forceinline__ bool bits_positive(double x) { return (long long)bits64(x) > 0; }
// |x| by clearing the sign bit of the high word (an integer operation, where
// fabs feeding an FMA's addend issues on the FP64 pipe)
__device__ __forceinline__ double abs_bits(double x) {
  double r;
  asm("{\n\t.reg .b32 lo, hi;\n\tmov.b64 {lo, hi}, %1;\n\tand.b32 hi, hi, 0x7fffffff;\n\t"
      "mov.b64 %0, {lo, hi};\n\t}" : "=d"(r) : "d"(x));
  return r;
}
// -x by flipping the sign bit of the high word (an integer operation)
__device__ __forceinline__ double neg_bits(double x) {
  double r;
  asm("{\n\t.reg .b32 lo, hi;\n\tmov.b64 {lo, hi}, %1;\n\txor.b32 hi, hi, 0x80000000;\n\t"
      "mov.b64 %0, {lo, hi};\n\t}" : "=d"(r) : "d"(x));
  return r;
}
__device__ __forceinline__ bool bits_negative(double x) {
  const long long b = (long long)bits64(x);
  return b < 0 && (b << 1) != 0;
}
// 1/x of either sign: rcp_newton of |x| with x's sign.
__device__ __forceinline__ double rcp_signed(double x) {
  const long long b = (long long)bits64(x);
  const double y = rcp_newton(__longlong_as_double(b & 0x7fffffffffffffffll));
  return __longlong_as_double((long long)bits64(y) ^ (b & (long long)0x8000000000000000ull));
}
#else
inline double rcp_newton(double x) { return 1.0 / x; }
inline double rcp_newton1(double x) { return 1.0 / x; }
inline double rcp_signed(double x) { return 1.0 / x; }
inline double sqrt_seeded(double x) { return std::sqrt(x); }
inline bool bits_positive(double x) { return x > 0; }
inline double abs_bits(double x) { return std::fabs(x); }
inline double neg_bits(double x) { return -x; }
inline bool bits_negative(double x) { return x < 0; }
#endif

// One side of the conservative-form Rusanov flux.  FAST_SQRT (the mixed
// form) takes the sound speed from sqrt_seeded.
template <bool FAST_SQRT = false>
MCFD_HD bool rusanov_side(const double *c, const double *n, double *f,
                          double *speed) {
  double r = c[0], e = c[4];
  if (!bits_positive(r) || bits_negative(e)) return false;
  double rinv = rcp_newton(r);
  double m2 = c[1] * c[1] + c[2] * c[2] + c[3] * c[3];
  double p = (e - 0.5 * m2 * rinv) * kGm1;
  if (bits_negative(p)) return false;
  double mn = c[1] * n[0] + c[2] * n[1] + c[3] * n[2];
  double un = mn * rinv;
  f[0] = mn;
  f[1] = c[1] * un + p * n[0];
  f[2] = c[2] * un + p * n[1];
  f[3] = c[3] * un + p * n[2];
  f[4] = (e + p) * un;
  const double c2 = kGamma * p * rinv;
  if constexpr (FAST_SQRT) {
    *speed = bits_positive(p) ? sqrt_seeded(c2) : 0.0;  // sound speed; caller adds |un|
  } else {
    *speed = bits_positive(p) ? sqrt(c2) : 0.0;
  }
  speed[1] = fabs(un);
  return true;
}

// The per-node part of the conservative-input face fluxes, stored once per
// stage state ("trace"): tr = {1/rho, p, third}, third = the sound speed
// (Rusanov, HLLC) or sqrt(rho) (Roe, roe_sqrt_rho); p = -1 marks a state that
// takes the primitive fallback (non-positive density, negative energy or
// pressure).
template <bool FAST_SQRT = false>
MCFD_HD void node_trace(const double *c, double *tr, bool roe_sqrt_rho = false) {
  double r = c[0], e = c[4];
  if (!bits_positive(r) || bits_negative(e)) {
    tr[0] = 0; tr[1] = -1; tr[2] = 0;
    return;
  }
  // FAST_SQRT (the mixed form): one Newton step for 1/rho as well
  double rinv = FAST_SQRT ? rcp_newton1(r) : rcp_newton(r);
  double m2 = c[1] * c[1] + c[2] * c[2] + c[3] * c[3];
  double p = fma(-0.5 * m2, rinv, e) * kGm1;
  tr[0] = rinv;
  if (bits_negative(p)) {
    tr[1] = -1; tr[2] = 0;
    return;
  }
  tr[1] = p;
  if (roe_sqrt_rho) {
    if constexpr (FAST_SQRT) tr[2] = sqrt_seeded(r);
    else tr[2] = sqrt(r);
    return;
  }
  const double c2 = kGamma * p * rinv;
  if constexpr (FAST_SQRT) {
    tr[2] = bits_positive(p) ? sqrt_seeded(c2) : 0.0;
  } else {
    tr[2] = bits_positive(p) ? sqrt(c2) : 0.0;
  }
}

// rusanov_side with the node's trace supplied.
MCFD_HD bool rusanov_side_traced(const double *c, const double *tr, const double *n,
                                 double *f, double *speed) {
  const double p = tr[1];
  if (bits_negative(p)) return false;
  const double rinv = tr[0], e = c[4];
  double mn = c[1] * n[0] + c[2] * n[1] + c[3] * n[2];
  double un = mn * rinv;
  f[0] = mn;
  f[1] = c[1] * un + p * n[0];
  f[2] = c[2] * un + p * n[1];
  f[3] = c[3] * un + p * n[2];
  f[4] = (e + p) * un;
  speed[0] = tr[2];
  speed[1] = fabs(un);
  return true;
}

// w * Rusanov(n) from both sides' traces (flux_rusanov_cons_weighted below).
MCFD_HD void flux_rusanov_traced_weighted(const double *cl, const double *trl,
                                          const double *cr, const double *trr,
                                          const double *n, double w, double *f);

MCFD_HD void flux_rusanov_cons(const double *cl, const double *cr,
                               const double *n, double *f);
template <bool FAST_SQRT = false>
MCFD_HD void flux_rusanov_cons_weighted(const double *cl, const double *cr,
                                        const double *n, double w, double *f);

// Local Lax-Friedrichs (python/riemann.py:457-476): average flux minus
// lambda_max / 2 * (U_R - U_L), lambda_max = max(|u_n| + a) over both sides.
MCFD_HD void flux_rusanov(const Prim &l, const Prim &r, const double *n,
                          double *f) {
  double unl = l.u * n[0] + l.v * n[1] + l.w * n[2];
  double unr = r.u * n[0] + r.v * n[1] + r.w * n[2];
  double el = prim_energy(l), er = prim_energy(r);
  double fl[kK], fr[kK];
  normal_flux(l, el, n, unl, fl);
  normal_flux(r, er, n, unr, fr);
  double lam = fmax(fabs(unl) + sound_speed(l), fabs(unr) + sound_speed(r));
  double h = 0.5 * lam;
  f[0] = 0.5 * (fr[0] + fl[0]) - h * (r.rho - l.rho);
  f[1] = 0.5 * (fr[1] + fl[1]) - h * (r.rho * r.u - l.rho * l.u);
  f[2] = 0.5 * (fr[2] + fl[2]) - h * (r.rho * r.v - l.rho * l.v);
  f[3] = 0.5 * (fr[3] + fl[3]) - h * (r.rho * r.w - l.rho * l.w);
  f[4] = 0.5 * (fr[4] + fl[4]) - h * (er - el);
}

MCFD_HD void flux_rusanov_cons(const double *cl, const double *cr,
                               const double *n, double *f) {
  double fl[kK], fr[kK], sl[2], sr[2];
  if (rusanov_side(cl, n, fl, sl) && rusanov_side(cr, n, fr, sr)) {
    double h = 0.5 * fmax(sl[0] + sl[1], sr[0] + sr[1]);
#pragma unroll
    for (int k = 0; k < kK; ++k) f[k] = 0.5 * (fr[k] + fl[k]) - h * (cr[k] - cl[k]);
    return;
  }
  flux_rusanov(cons_to_prim(cl[0], cl[1], cl[2], cl[3], cl[4]),
               cons_to_prim(cr[0], cr[1], cr[2], cr[3], cr[4]), n, f);
}

MCFD_HD bool rusanov_traced_nh(const double *cl, const double *trl, const double *cr,
                               const double *trr, const double *nh, double hw, double *f);

// w * Rusanov(n) for a unit normal n and face weight w > 0, evaluated with
// the half-weighted normal nh = (w/2) n: F(nh) = (w/2) F(n) for the physical
// fluxes and |u.nh| + a|nh| = (w/2)(|u.n| + a), so
//   w F_hat = F_L(nh) + F_R(nh) - lambda(nh) (U_R - U_L)
// without the separate averaging and weighting multiplies.
template <bool FAST_SQRT>
MCFD_HD void flux_rusanov_cons_weighted(const double *cl, const double *cr,
                                        const double *n, double w, double *f) {
  // both sides' {1/rho, p, sound speed} as the node traces form them, then the
  // traced flux (summed side fluxes); a marked side (rho <= 0, E < 0 or
  // p < 0) takes the primitive form
  double trl[3], trr[3];
  node_trace<FAST_SQRT>(cl, trl);
  node_trace<FAST_SQRT>(cr, trr);
  const double hw = 0.5 * w;
  const double nh[3] = {hw * n[0], hw * n[1], hw * n[2]};
  if (rusanov_traced_nh(cl, trl, cr, trr, nh, hw, f)) return;
  flux_rusanov(cons_to_prim(cl[0], cl[1], cl[2], cl[3], cl[4]),
               cons_to_prim(cr[0], cr[1], cr[2], cr[3], cr[4]), n, f);
#pragma unroll
  for (int k = 0; k < kK; ++k) f[k] *= w;
}

// The two sides' physical fluxes are summed as they are formed and the
// dissipation shares each side's velocity factor:
//   F_L + F_R - lambda (U_R - U_L) = U_L (u_nL + lambda) + U_R (u_nR - lambda)
//       + (p_L + p_R) nh in the momentum rows, + p_L u_nL + p_R u_nR in the energy row,
// so a face point takes 28 FP64 operations (40 with the jump formed
// separately, 46 side by side).  From the half-weighted normal nh = (w/2) n
// and hw = w/2 (the face kernels of Rusanov handles read them precomputed);
// false when a side's trace is marked (the caller takes the primitive
// fallback).  The larger of the two wave speeds (both >= 0) is chosen on the
// bit patterns.
MCFD_HD bool rusanov_traced_nh(const double *cl, const double *trl, const double *cr,
                               const double *trr, const double *nh, double hw, double *f) {
  const double pl = trl[1], pr = trr[1];
  if (bits_negative(pl) || bits_negative(pr)) return false;
  const double mnl = cl[1] * nh[0] + cl[2] * nh[1] + cl[3] * nh[2];
  const double mnr = cr[1] * nh[0] + cr[2] * nh[1] + cr[3] * nh[2];
  const double unl = mnl * trl[0], unr = mnr * trr[0];
  const double sl = fma(trl[2], hw, abs_bits(unl)), sr = fma(trr[2], hw, abs_bits(unr));
  const double lam = le_nonneg(sr, sl) ? sl : sr;
  const double al = unl + lam, ar = unr - lam;
  const double ps = pl + pr;
  f[0] = fma(cr[0], ar, cl[0] * al);
#pragma unroll
  for (int d = 0; d < 3; ++d) f[1 + d] = fma(cr[1 + d], ar, fma(cl[1 + d], al, ps * nh[d]));
  f[4] = fma(cr[4], ar, fma(cl[4], al, fma(pr, unr, pl * unl)));
  return true;
}

MCFD_HD void flux_rusanov_traced_weighted(const double *cl, const double *trl,
                                          const double *cr, const double *trr,
                                          const double *n, double w, double *f) {
  const double hw = 0.5 * w;
  const double nh[3] = {hw * n[0], hw * n[1], hw * n[2]};
  if (rusanov_traced_nh(cl, trl, cr, trr, nh, hw, f)) return;
  flux_rusanov(cons_to_prim(cl[0], cl[1], cl[2], cl[3], cl[4]),
               cons_to_prim(cr[0], cr[1], cr[2], cr[3], cr[4]), n, f);
#pragma unroll
  for (int k = 0; k < kK; ++k) f[k] *= w;
}

// ---------------------------------------------------------------- HLLC
// hllc.hpp:30-109 with the star state's tangential velocity carried from
// the side it is built on.
MCFD_HD double hllc_q(double p_estimate, double p_k) {
  if (p_estimate <= p_k) return 1.0;
  double temp = 1 + kGp1Over2 * (p_estimate * rcp_newton(p_k) - 1) * kOneOverGamma;
  return sqrt(temp);
}

MCFD_HD void hllc_star(const Prim &s, double un, double e, const double *n,
                       double wave_k, double wave_star, double *f) {
  normal_flux(s, e, n, un, f);
  double temp = s.rho * (wave_k - un) * rcp_signed(wave_k - wave_star);
  double es = e * s.rinv + (wave_star - un) *
      (wave_star + s.p * rcp_signed(s.rho * (wave_k - un)));
  es *= temp;
  // star momentum = temp * (wave_star n + u_t), u_t = u - un n
  double dm = temp * (wave_star - un);
  double sm0 = temp * s.u + dm * n[0];
  double sm1 = temp * s.v + dm * n[1];
  double sm2 = temp * s.w + dm * n[2];
  f[0] += wave_k * (temp - s.rho);
  f[1] += wave_k * (sm0 - s.rho * s.u);
  f[2] += wave_k * (sm1 - s.rho * s.v);
  f[3] += wave_k * (sm2 - s.rho * s.w);
  f[4] += wave_k * (es - e);
}

MCFD_HD void flux_hllc(const Prim &l, const Prim &r, const double *n,
                       double *f) {
  double unl = l.u * n[0] + l.v * n[1] + l.w * n[2];
  double unr = r.u * n[0] + r.v * n[1] + r.w * n[2];
  double rho_average = (l.rho + r.rho) / 2;
  double a_left = sound_speed(l), a_right = sound_speed(r);
  double a_average = (a_left + a_right) / 2;
  double p_pvrs = (l.p + r.p - (unr - unl) * rho_average * a_average) / 2;
  double p_estimate = fmax(0.0, p_pvrs);
  double wave_left = unl - a_left * hllc_q(p_estimate, l.p);
  double wave_right = unr + a_right * hllc_q(p_estimate, r.p);
  double wave_star = (r.p - l.p + l.rho * unl * (wave_left - unl) -
                      r.rho * unr * (wave_right - unr)) *
                     rcp_signed(l.rho * (wave_left - unl) - r.rho * (wave_right - unr));
  if (0.0 <= wave_left) {
    normal_flux(l, prim_energy(l), n, unl, f);
  } else if (wave_right <= 0.0) {
    normal_flux(r, prim_energy(r), n, unr, f);
  } else if (0.0 <= wave_star) {
    hllc_star(l, unl, prim_energy(l), n, wave_left, wave_star, f);
  } else if (wave_star < 0.0) {
    hllc_star(r, unr, prim_energy(r), n, wave_right, wave_star, f);
  } else {
    for (int k = 0; k < kK; ++k) f[k] = NAN;
  }
}

// ---------------------------------------------------------------- AUSM
// ausm.hpp:146-187: F = rho a M+- (1, u, v, w, h) + p+- n.
MCFD_HD void ausm_signed(bool negative, const Prim &s, const double *n,
                         double *f) {
  double a = sound_speed(s);
  double h = a * a / kGm1 + kinetic(s);
  double un = s.u * n[0] + s.v * n[1] + s.w * n[2];
  double mach = un / a;
  double p = s.p;
  double signed_mach = (1 + (negative ? -mach : mach)) * 0.5;
  if (mach >= -1 && mach <= 1) {
    double m2 = signed_mach * signed_mach;
    mach = negative ? -m2 : m2;
    p *= signed_mach;
  } else if (signed_mach < 0) {
    mach = 0.0;
    p = 0.0;
  }
  double scale = s.rho * a * mach;
  f[0] += scale;
  f[1] += scale * s.u + p * n[0];
  f[2] += scale * s.v + p * n[1];
  f[3] += scale * s.w + p * n[2];
  f[4] += scale * h;
}

MCFD_HD void flux_ausm(const Prim &l, const Prim &r, const double *n,
                       double *f) {
  for (int k = 0; k < kK; ++k) f[k] = 0;
  ausm_signed(false, l, n, f);
  ausm_signed(true, r, n, f);
}

// ---------------------------------------------------------------- Roe
// python/riemann.py:405-455 in 3D: acoustic waves u_n -/+ a, the entropy
// wave and two shear waves at u_n; no entropy fix.
MCFD_HD void flux_roe(const Prim &l, const Prim &r, const double *n,
                      double *f) {
  double unl = l.u * n[0] + l.v * n[1] + l.w * n[2];
  double unr = r.u * n[0] + r.v * n[1] + r.w * n[2];
  double el = prim_energy(l), er = prim_energy(r);
  double fl[kK], fr[kK];
  normal_flux(l, el, n, unl, fl);
  normal_flux(r, er, n, unr, fr);
  for (int k = 0; k < kK; ++k) f[k] = (fl[k] + fr[k]) / 2;
  // h0 = gamma p / rho / (gamma - 1) + |u|^2 / 2 (python/equation.py): a
  // zero density (a vacuum or unconverted state) divides by zero there, so
  // the flux becomes non-finite as in the prototype
  const double il = l.rho != 0 ? l.rinv : 1.0 / l.rho;
  const double ir = r.rho != 0 ? r.rinv : 1.0 / r.rho;
  double h0_l = kGammaOverGm1 * l.p * il + kinetic(l);
  double h0_r = kGammaOverGm1 * r.p * ir + kinetic(r);
  double sl = sqrt(l.rho), sr = sqrt(r.rho);
  double inv_sum = rcp_newton(sl + sr);
  double rho = sl * sr;
  double u = (sl * l.u + sr * r.u) * inv_sum;
  double v = (sl * l.v + sr * r.v) * inv_sum;
  double w = (sl * l.w + sr * r.w) * inv_sum;
  double h0 = (sl * h0_l + sr * h0_r) * inv_sum;
  double un = u * n[0] + v * n[1] + w * n[2];
  double ke = (u * u + v * v + w * w) / 2;
  double aa = kGm1 * (h0 - ke);
  double a = sqrt(aa);
  double ua = un * a;
  double p_jump = r.p - l.p;
  double u_jump = unr - unl;
  double inv_2aa = rcp_newton(2 * aa);
  // wave u_n - a: r = (1, u - a n, h0 - u_n a)
  double s1 = 0.5 * ((p_jump - rho * a * u_jump) * inv_2aa) * fabs(un - a);
  // entropy wave u_n: r = (1, u, ke)
  double s2 = 0.5 * ((r.rho - l.rho) - p_jump * (2 * inv_2aa)) * fabs(un);
  // wave u_n + a: r = (1, u + a n, h0 + u_n a)
  double s5 = 0.5 * ((p_jump + rho * a * u_jump) * inv_2aa) * fabs(un + a);
  // shear waves u_n: tangential velocity jump times rho
  double dv0 = r.u - l.u, dv1 = r.v - l.v, dv2 = r.w - l.w;
  double dvn = dv0 * n[0] + dv1 * n[1] + dv2 * n[2];
  double st = 0.5 * rho * fabs(un);
  double t0 = st * (dv0 - dvn * n[0]);
  double t1 = st * (dv1 - dvn * n[1]);
  double t2 = st * (dv2 - dvn * n[2]);
  f[0] -= s1 + s2 + s5;
  f[1] -= s1 * (u - a * n[0]) + s2 * u + s5 * (u + a * n[0]) + t0;
  f[2] -= s1 * (v - a * n[1]) + s2 * v + s5 * (v + a * n[1]) + t1;
  f[3] -= s1 * (w - a * n[2]) + s2 * w + s5 * (w + a * n[2]) + t2;
  f[4] -= s1 * (h0 - ua) + s2 * ke + s5 * (h0 + ua) +
          (t0 * u + t1 * v + t2 * w);
}

// HLLC on conservative inputs for two states with rho > 0, E >= 0 and
// p > 0 on both sides (false otherwise: the caller takes flux_hllc on the
// converted primitives).  The same flux as flux_hllc with the energy and
// momenta taken from the inputs instead of being rebuilt from primitives;
// FAST_SQRT (the mixed form) takes the sound speeds and the pressure-ratio
// roots from sqrt_seeded.
template <bool FAST_SQRT>
MCFD_HD double sqrt_form(double x) {
  if constexpr (FAST_SQRT) return sqrt_seeded(x);
  else return sqrt(x);
}

// (gamma + 1) / (2 gamma): the pressure ratio's weight in the wave-speed factor
constexpr double kHllcQ = kGp1Over2 * kOneOverGamma;

// HLLC times the face weight w, from both sides' conservative variables,
// 1/rho, pressure and sound speed (p > 0 on both).
// The wave speeds of hllc.hpp, u_n -/+ a_k q_k with
// q_k = sqrt(1 + (gamma+1)/(2 gamma) (p*/p_k - 1)) for p* > p_k, are formed as
// a_k q_k = sqrt(gamma / rho_k (p_k + (gamma+1)/(2 gamma) (p* - p_k))): the same
// number without the reciprocal of p_k.
// The flux of the side that the reference's four cases pick (left, right,
// left star, right star), with S_k that side's wave speed and S* the contact
// speed, is
//   F*_k = (S* (S_k U_k - F_k) + S_k p*_k D) / (S_k - S*),  D = (0, n, S*),
//   p*_k = p_k + rho_k (S_k - u_k) (S* - u_k),
// which is F_k + S_k (U*_k - U_k) with the star state of hllc.hpp: the jump
// conditions across the S_k wave (S_k U* - F* = S_k U - F) and across the
// contact (F* = S* U* + p* D) give it.  A supersonic side (no star
// correction) takes the same arithmetic with S_k = 0, S* = 1, which yields
// F_k.  Per component, with g = w / (S_k - S*),
//   rho:  rho A,   m_i:  m_i A + n_i B,   E:  E A + g S* (S_k p*_k - p_k u_k),
//   A = g S* (S_k - u_k),   B = g (S_k p*_k - S* p_k),
// so neither F_k nor U*_k is formed: 23 FP64 operations after the wave
// speeds (the side flux, the star correction and the weight took 50), and
// lanes of a warp in different cases share one pass through them.
template <bool FAST_SQRT>
MCFD_HD void hllc_core_weighted(const double *cl, const double *cr, double il, double ir,
                                double pl, double pr, double al, double ar, const double *n,
                                double w, double *f) {
  const double rl = cl[0], rr = cr[0];
  const double mnl = cl[1] * n[0] + cl[2] * n[1] + cl[3] * n[2];
  const double mnr = cr[1] * n[0] + cr[2] * n[1] + cr[3] * n[2];
  const double unl = mnl * il, unr = mnr * ir;
  // (p_L + p_R - (u_R - u_L) rho_average a_average) / 2 with the averages'
  // halves taken out as one exact factor 1/8
  const double p_pvrs = fma(((unr - unl) * (rl + rr)) * (al + ar), -0.125, 0.5 * (pl + pr));
  // fmax(0, p_pvrs) and the wave-sign tests on the bit patterns (integer
  // pipes; the same results, NaN included)
  const double p_estimate = gt_zero(p_pvrs) ? p_pvrs : 0.0;
  double aql = al, aqr = ar;  // a_k q_k, q_k = 1 unless p* > p_k (both >= 0 here)
  if (!le_nonneg(p_estimate, pl)) aql = sqrt_form<FAST_SQRT>(kGamma * il * fma(kHllcQ, p_estimate - pl, pl));
  if (!le_nonneg(p_estimate, pr)) aqr = sqrt_form<FAST_SQRT>(kGamma * ir * fma(kHllcQ, p_estimate - pr, pr));
  const double wave_left = unl - aql;
  const double wave_right = unr + aqr;
  const double dl = wave_left - unl, dr = wave_right - unr;  // S_k - u_k
  const double rdl = rl * dl, rdr = rr * dr;                  // rho_k (S_k - u_k)
  const double wave_star = fma(unl, rdl, fma(-unr, rdr, pr - pl)) * rcp_signed(rdl - rdr);
  const bool sup_l = ge_zero(wave_left), sup_r = le_zero(wave_right);
  const bool star = !sup_l && !sup_r;
  if (star && !ge_zero(wave_star) && !lt_zero(wave_star)) {  // wave_star is NaN
    for (int k = 0; k < kK; ++k) f[k] = NAN;
    return;
  }
  const bool left = sup_l || (!sup_r && ge_zero(wave_star));
  // the side's values (integer selects); S_k = 0, S* = 1 without the star
  // correction, where S_k - u_k is then -u_k
  double c[kK];
#pragma unroll
  for (int k = 0; k < kK; ++k) c[k] = left ? cl[k] : cr[k];
  const double p = left ? pl : pr, un = left ? unl : unr;
  const double sk = star ? (left ? wave_left : wave_right) : 0.0;
  const double ss = star ? wave_star : 1.0;
  const double skun = star ? (left ? dl : dr) : neg_bits(un);
  const double g = w * rcp_signed(sk - ss);
  // p*_k = p_k + rho_k (S_k - u_k)(S* - u_k) (used only with the star correction)
  const double pstar = fma(left ? rdl : rdr, ss - un, p);
  const double sp = star ? sk * pstar : 0.0;  // S_k p*_k
  const double gs = g * ss;
  const double A = gs * skun;
  const double B = g * fma(-ss, p, sp);
  f[0] = c[0] * A;
  f[1] = fma(c[1], A, n[0] * B);
  f[2] = fma(c[2], A, n[1] * B);
  f[3] = fma(c[3], A, n[2] * B);
  f[4] = fma(c[4], A, gs * fma(-p, un, sp));
}

template <bool FAST_SQRT>
MCFD_HD bool flux_hllc_cons_weighted(const double *cl, const double *cr, const double *n,
                                     double w, double *f) {
  const double rl = cl[0], rr = cr[0];
  if (!bits_positive(rl) || !bits_positive(rr) || bits_negative(cl[4]) || bits_negative(cr[4])) return false;
  // the mixed form: one Newton step (relative error below 4e-14, as its node
  // traces take it, beside the seeded square roots' 1.4e-13)
  const double il = FAST_SQRT ? rcp_newton1(rl) : rcp_newton(rl);
  const double ir = FAST_SQRT ? rcp_newton1(rr) : rcp_newton(rr);
  // p = (E - |m|^2 / (2 rho)) (gamma - 1)
  const double ml = cl[1] * cl[1] + cl[2] * cl[2] + cl[3] * cl[3];
  const double mr = cr[1] * cr[1] + cr[2] * cr[2] + cr[3] * cr[3];
  const double pl = fma(-0.5 * ml, il, cl[4]) * kGm1;
  const double pr = fma(-0.5 * mr, ir, cr[4]) * kGm1;
  if (!bits_positive(pl) || !bits_positive(pr)) return false;
  const double al = sqrt_form<FAST_SQRT>(kGamma * pl * il), ar = sqrt_form<FAST_SQRT>(kGamma * pr * ir);
  hllc_core_weighted<FAST_SQRT>(cl, cr, il, ir, pl, pr, al, ar, n, w, f);
  return true;
}

// flux_hllc_cons_weighted with both sides' node traces {1/rho, p, sound
// speed}: false (primitive fallback) unless p > 0 on both sides.
template <bool FAST_SQRT>
MCFD_HD bool flux_hllc_traced_weighted(const double *cl, const double *trl, const double *cr,
                                       const double *trr, const double *n, double w, double *f) {
  if (!bits_positive(trl[1]) || !bits_positive(trr[1])) return false;
  hllc_core_weighted<FAST_SQRT>(cl, cr, trl[0], trr[0], trl[1], trr[1], trl[2], trr[2], n, w, f);
  return true;
}

// Roe on conservative inputs, times the face weight w, for two admissible
// states (rho > 0, E >= 0, p >= 0 on both sides; false otherwise and the
// caller takes flux_roe on the converted primitives).  The same flux as
// flux_roe, regrouped: the physical flux from the conservative variables
// (m u_n + p n, (E + p) u_n), the total enthalpy as (E + p) / rho, the Roe
// weights from lambda = sqrt(rho_R / rho_L) (u~ = (u_L + lambda u_R) /
// (1 + lambda), rho~ = lambda rho_L: one square root instead of two), and the
// acoustic pair combined as (a1 + a5) (u, h0) + (a5 - a1) a (n, u_n).
// The reference's average 0.5 (F_L + F_R) - 0.5 sum_k |l_k| alpha_k r_k is
// taken in its upwind form F_L + sum_k min(l_k, 0) alpha_k r_k: with Roe
// averages the wave strengths decompose the jumps exactly,
// F_R - F_L = sum_k l_k alpha_k r_k (Roe's property), so the two are the
// same flux, and the right state's physical flux and normal velocity are
// never formed (u_n,R - u_n,L is the normal part of the velocity jump that
// the shear waves need anyway).
// FAST_SQRT (the mixed form) takes both square roots from sqrt_seeded.
// Roe from both sides' 1/rho and pressure and lambda = sqrt(rho_R / rho_L).
template <bool FAST_SQRT>
MCFD_HD void roe_core_weighted(const double *cl, const double *cr, double il, double ir,
                               double pl, double pr, double lam, const double *n, double w,
                               double *f) {
  const double rl = cl[0], rr = cr[0], el = cl[4], er = cr[4];
  const double ul = cl[1] * il, vl = cl[2] * il, wl = cl[3] * il;
  const double ur = cr[1] * ir, vr = cr[2] * ir, wr = cr[3] * ir;
  const double unl = ul * n[0] + vl * n[1] + wl * n[2];
  // F(U_L)
  const double hl = el + pl;
  const double s0 = rl * unl;
  const double s1 = cl[1] * unl + pl * n[0];
  const double s2 = cl[2] * unl + pl * n[1];
  const double s3 = cl[3] * unl + pl * n[2];
  const double s4 = hl * unl;
  // Roe averages
  const double inv = rcp_newton(1 + lam);
  const double rho = lam * rl;
  const double u = (ul + lam * ur) * inv, v = (vl + lam * vr) * inv, ww = (wl + lam * wr) * inv;
  const double h0 = (hl * il + lam * ((er + pr) * ir)) * inv;
  const double un = u * n[0] + v * n[1] + ww * n[2];
  const double ke = 0.5 * (u * u + v * v + ww * ww);
  const double aa = kGm1 * (h0 - ke);
  double a;
  if constexpr (FAST_SQRT) a = sqrt_seeded(aa);
  else a = sqrt(aa);
  const double i2aa = rcp_newton(2 * aa);
  // min(l_k, 0) on the bit patterns (integer selects; NaN stays NaN)
  const double l1 = un - a, l5 = un + a;
  const double m1 = gt_zero(l1) ? 0.0 : l1, m2 = gt_zero(un) ? 0.0 : un, m5 = gt_zero(l5) ? 0.0 : l5;
  const double dv0 = ur - ul, dv1 = vr - vl, dv2 = wr - wl;
  const double dvn = dv0 * n[0] + dv1 * n[1] + dv2 * n[2];  // u_n,R - u_n,L
  // the wave strengths times min(l_k, 0)
  const double dp = pr - pl, rau = rho * a * dvn;
  const double a1 = ((dp - rau) * i2aa) * m1;
  const double a2 = ((rr - rl) - dp * (2 * i2aa)) * m2;
  const double a5 = ((dp + rau) * i2aa) * m5;
  const double st = rho * m2;
  const double t0 = st * (dv0 - dvn * n[0]), t1 = st * (dv1 - dvn * n[1]), t2 = st * (dv2 - dvn * n[2]);
  const double S = a1 + a5, Sa = S + a2, D = (a5 - a1) * a;
  f[0] = w * (s0 + Sa);
  f[1] = w * (s1 + (Sa * u + D * n[0] + t0));
  f[2] = w * (s2 + (Sa * v + D * n[1] + t1));
  f[3] = w * (s3 + (Sa * ww + D * n[2] + t2));
  f[4] = w * (s4 + (S * h0 + D * un + a2 * ke + (t0 * u + t1 * v + t2 * ww)));
}

template <bool FAST_SQRT>
MCFD_HD bool flux_roe_cons_weighted(const double *cl, const double *cr, const double *n,
                                    double w, double *f) {
  const double rl = cl[0], rr = cr[0], el = cl[4], er = cr[4];
  if (!bits_positive(rl) || !bits_positive(rr) || bits_negative(el) || bits_negative(er)) return false;
  const double il = rcp_newton(rl), ir = rcp_newton(rr);
  const double ul = cl[1] * il, vl = cl[2] * il, wl = cl[3] * il;
  const double ur = cr[1] * ir, vr = cr[2] * ir, wr = cr[3] * ir;
  const double pl = (el - 0.5 * (cl[1] * ul + cl[2] * vl + cl[3] * wl)) * kGm1;
  const double pr = (er - 0.5 * (cr[1] * ur + cr[2] * vr + cr[3] * wr)) * kGm1;
  if (bits_negative(pl) || bits_negative(pr)) return false;
  double lam;
  if constexpr (FAST_SQRT) lam = sqrt_seeded(rr * il);
  else lam = sqrt(rr * il);
  roe_core_weighted<FAST_SQRT>(cl, cr, il, ir, pl, pr, lam, n, w, f);
  return true;
}

// flux_roe_cons_weighted with both sides' node traces {1/rho, p, sqrt(rho)}:
// lambda = sqrt(rho_R) sqrt(rho_L) / rho_L without a square root; false
// (primitive fallback) when a side is marked (p = -1).
template <bool FAST_SQRT>
MCFD_HD bool flux_roe_traced_weighted(const double *cl, const double *trl, const double *cr,
                                      const double *trr, const double *n, double w, double *f) {
  if (bits_negative(trl[1]) || bits_negative(trr[1])) return false;
  const double lam = (trr[2] * trl[2]) * trl[0];
  roe_core_weighted<FAST_SQRT>(cl, cr, trl[0], trr[0], trl[1], trr[1], lam, n, w, f);
  return true;
}

// ---------------------------------------------------------------- Exact
// exact.hpp:62-320 on the normal component; the tangential velocity comes
// from the left state if u* > 0 else the right (SetPassiveScalars).  The
// reference keeps u* as solver state across calls and leaves it untouched in
// vacuum branches; here (as for a freshly built solver) it is 0 there.
// The root finder is capped at kExactMaxIter iterations per loop; reaching
// the cap sets *not_converged.
constexpr int kExactMaxIter = 256;

struct Exact1D {
  double rho, u, p;  // normal-frame state on the t axis
};

MCFD_HD double ex_sound(double rho, double p) {
  return (rho > 0 && p > 0) ? sqrt(kGamma * p / rho) : 0.0;
}

// The Exact solver's powers have rational exponents for gamma = 1.4:
// (gamma - 1) / (2 gamma) = 1/7 and gamma = 7/5.  On the device they come
// from inverse roots z = x^(-1/K) (K = 7, 5): an FP32 seed exp2(-log2(x) / K)
// (relative error below 1e-6), then two Newton steps on z^-K = x in the
// division-free form z <- z + z (1 - x z^K) / K, each taking a relative error
// e to about (K + 1) / 2 e^2 (1e-12, then the FP64 rounding level).  Outside
// x in [2^-120, 2^120] (FP32 cannot seed it) pow is taken.
#ifdef __CUDA_ARCH__
template <int K>
__device__ __forceinline__ double zpow(double z) {
  const double z2 = z * z;
  if constexpr (K == 5) return (z2 * z2) * z;
  const double z3 = z2 * z;
  return (z3 * z3) * z;  // K == 7
}
template <int K>
__device__ __forceinline__ bool inv_root(double x, double *z_out) {
  const int e = (int)((bits64(x) >> 52) & 0x7ff) - 1023;
  if (e < -120 || e > 120 || (long long)bits64(x) < 0) return false;
  const float xf = f64_to_f32(x);
  double z = f32_to_f64(exp2f(log2f(xf) * (-1.0f / K)));
#pragma unroll
  for (int i = 0; i < 2; ++i) {
    const double err = fma(-x, zpow<K>(z), 1.0);
    z = fma(z * err, 1.0 / K, z);
  }
  *z_out = z;
  return true;
}
#endif

// r^(1/7) for the expansion branch (r = p_after / p_before >= 0); with
// *r67 = r^(-6/7) = r^(1/7) / r for its derivative when asked.
MCFD_HD double ex_root7(double r, double *r67 = nullptr) {
#ifdef __CUDA_ARCH__
  double z;
  if (inv_root<7>(r, &z)) {
    const double z3 = (z * z) * z, z6 = z3 * z3;
    if (r67) *r67 = z6;
    return r * z6;
  }
#endif
  const double s = pow(r, kGm1Over2 / kGamma);
  if (r67) *r67 = s / r;
  return s;
}

// p / rho^gamma (the isentrope constant of ex_near_expansion and the vacuum
// cases), rho^-gamma = (rho^(-1/5))^7.
MCFD_HD double ex_isentrope(double p, double rho) {
#ifdef __CUDA_ARCH__
  double z;
  if (inv_root<5>(rho, &z)) return p * zpow<7>(z);
#endif
  return p / pow(rho, kGamma);
}

struct SpeedChange {
  double rho_before, p_before, a_before, p_const;
  // 1 / p_before and 1 / (rho_before a_before), once per side (IEEE
  // reciprocals: a zero gives the infinity the reference's quotients give)
  double inv_p, inv_rho_a;
  MCFD_HD SpeedChange(double rho, double p)
      : rho_before(rho), p_before(p),
        a_before(rho == 0 ? 0 : ex_sound(rho, p)),
        p_const(p * kGm1Over2),
        inv_p(1.0 / p), inv_rho_a(1.0 / (rho * a_before)) {}
  MCFD_HD double P(double p_after) const { return kGp1Over2 * p_after + p_const; }
  MCFD_HD double value(double p_after) const {
    if (p_after >= p_before) {
      double divisor = sqrt(rho_before * P(p_after));
      return (p_after - p_before) / divisor;
    }
    // pow(+0, y > 0) is +0: the vacuum test at p = 0 needs no power
    double v = (p_after == 0 ? 0.0 : ex_root7(p_after * inv_p)) - 1;
    return v * (kGm1Under2 * a_before);
  }
  // value and prime at the same pressure: in the shock branch one reciprocal
  // of the square root D = sqrt(rho P) serves both (1 / P = rho / D^2); in the
  // expansion branch r^(1/7) and r^(-6/7) = r^(1/7) / r of r = p_after /
  // p_before come from one inverse root.
  MCFD_HD void value_prime(double p_after, double *v, double *d) const {
    if (p_after >= p_before) {
      const double divisor = sqrt(rho_before * P(p_after));
      const double inv = 1.0 / divisor;
      *v = (p_after - p_before) * inv;
      const double w = kGp1Over4 * (p_before - p_after);
      *d = fma(w * rho_before, inv * inv, 1.0) * inv;
      return;
    }
    double r67;
    const double s = ex_root7(p_after * inv_p, &r67);
    *v = (s - 1) * (kGm1Under2 * a_before);
    *d = r67 * inv_rho_a;
  }
};

MCFD_HD Exact1D ex_inside_expansion(double gri_1, double gri_2) {
  constexpr double r = kGm1 / kGp1;
  double a = r * gri_2;
  double a_square = a * a;
  // q^(1 / (gamma - 1)) = q^(5/2) = q^2 sqrt(q)
  const double q = a_square / gri_1 * kOneOverGamma;
  double rho = (q * q) * sqrt(q);
  return Exact1D{rho, a, a_square * rho * kOneOverGamma};
}

MCFD_HD Exact1D ex_near_shock(int field, const Exact1D &before,
                              Exact1D after) {
  double u = before.u;
  double divisor = (after.u - before.u) * before.rho;
  u += (divisor != 0 ? (after.p - before.p) / divisor : before.u);
  bool after_shock = field == 1 ? (u < 0) : (u > 0);
  if (after_shock) {
    after.rho = before.rho * ((before.u - u) / (after.u - u));
    return after;
  }
  return before;
}

MCFD_HD Exact1D ex_near_expansion(int field, const Exact1D &before,
                                  Exact1D after) {
  double a_before = ex_sound(before.rho, before.p);
  double gri_1 = ex_isentrope(before.p, before.rho);
  double gri_2, a_after;
  if (field == 1) {
    gri_2 = before.u + kGm1Under2 * a_before;
    a_after = a_before + kGm1Over2 * (before.u - after.u);
  } else {
    gri_2 = before.u - kGm1Under2 * a_before;
    a_after = a_before - kGm1Over2 * (before.u - after.u);
  }
  bool after_wave = field == 1 ? (after.u - a_after < 0) : (after.u + a_after > 0);
  bool before_wave = field == 1 ? (before.u - a_before > 0)
                                : (before.u + a_before < 0);
  if (after_wave) {
    after.rho = kGamma * after.p / (a_after * a_after);
    return after;
  } else if (before_wave) {
    return before;
  }
  return ex_inside_expansion(gri_1, gri_2);
}

MCFD_HD Exact1D ex_near_vacuum(const Exact1D &l, const Exact1D &r) {
  double left_a = ex_sound(l.rho, l.p);
  if (l.u > left_a) return l;
  double right_a = ex_sound(r.rho, r.p);
  if (r.u + right_a < 0) return r;
  double gri_1 = ex_isentrope(l.p, l.rho);
  double gri_2 = l.u + left_a * kGm1Under2;
  if (gri_2 >= 0) return ex_inside_expansion(gri_1, gri_2);
  gri_1 = ex_isentrope(r.p, r.rho);
  gri_2 = r.u - right_a * kGm1Under2;
  if (gri_2 < 0) return ex_inside_expansion(gri_1, gri_2);
  return Exact1D{0, 0, 0};
}

MCFD_HD Exact1D exact_upwind(const Exact1D &l, const Exact1D &r,
                             double *star_u, bool *not_converged) {
  *star_u = 0.0;
  if (l.rho > 0) {
    if (!(r.rho > 0)) {
      double a_left = ex_sound(l.rho, l.p);
      if (l.u >= a_left) return l;
      double u_star = l.u + a_left * kGm1Under2;
      if (u_star <= 0) return Exact1D{0, 0, 0};
      return ex_inside_expansion(ex_isentrope(l.p, l.rho), u_star);
    }
  } else {
    if (r.rho > 0) {
      double a_right = ex_sound(r.rho, r.p);
      if (r.u + a_right <= 0) return r;
      double u_star = r.u - a_right * kGm1Under2;
      if (u_star >= 0) return Exact1D{0, 0, 0};
      return ex_inside_expansion(ex_isentrope(r.p, r.rho), u_star);
    }
    return Exact1D{0, 0, 0};
  }
  double du = r.u - l.u;
  SpeedChange cl(l.rho, l.p), cr(r.rho, r.p);
  if (cl.value(0) + cr.value(0) + du < 0) {
    // FindRoot (exact.hpp:140-152), both loops capped
    double x = l.p;
    int it = 0;
    while (cl.value(x) + cr.value(x) + du > 0 && it < kExactMaxIter) {
      x *= 0.5;
      ++it;
    }
    if (it == kExactMaxIter) *not_converged = true;
    it = 0;
    // Newton: value and prime of both sides at each x together
    double vl, dl, vr, dr;
    cl.value_prime(x, &vl, &dl);
    cr.value_prime(x, &vr, &dr);
    double fx = vl + vr + du;
    while (fx < -1e-8 && it < kExactMaxIter) {
      x -= fx / (dl + dr);
      ++it;
      cl.value_prime(x, &vl, &dl);
      cr.value_prime(x, &vr, &dr);
      fx = vl + vr + du;
    }
    if (it == kExactMaxIter) *not_converged = true;
    Exact1D star{0, 0, x};
    star.u = 0.5 * (r.u + vr + l.u - vl);
    *star_u = star.u;
    if (0 < star.u) {
      return star.p >= l.p ? ex_near_shock(1, l, star)
                           : ex_near_expansion(1, l, star);
    }
    return star.p >= r.p ? ex_near_shock(3, r, star)
                         : ex_near_expansion(3, r, star);
  }
  return ex_near_vacuum(l, r);
}

MCFD_HD void flux_exact(const Prim &l, const Prim &r, const double *n,
                        double *f, bool *not_converged) {
  double unl = l.u * n[0] + l.v * n[1] + l.w * n[2];
  double unr = r.u * n[0] + r.v * n[1] + r.w * n[2];
  double star_u;
  Exact1D s = exact_upwind(Exact1D{l.rho, unl, l.p}, Exact1D{r.rho, unr, r.p},
                           &star_u, not_converged);
  const Prim &t = star_u > 0 ? l : r;
  double untan = star_u > 0 ? unl : unr;
  // velocity = s.u n + (u_t of the passive side)
  Prim w;
  w.rho = s.rho;
  w.rinv = s.rho > 0 ? 1.0 / s.rho : 0.0;
  w.p = s.p;
  w.u = t.u + (s.u - untan) * n[0];
  w.v = t.v + (s.u - untan) * n[1];
  w.w = t.w + (s.u - untan) * n[2];
  normal_flux(w, prim_energy(w), n, s.u, f);
}

// Upwind flux F(U_L, U_R; n) of a rotated solver (rotated/euler.hpp:153-159).
template <int R>
MCFD_HD void flux_upwind(const Prim &l, const Prim &r, const double *n,
                         double *f, bool *not_converged) {
  if constexpr (R == kRusanov) {
    flux_rusanov(l, r, n, f);
  } else if constexpr (R == kHllc) {
    flux_hllc(l, r, n, f);
  } else if constexpr (R == kAusm) {
    flux_ausm(l, r, n, f);
  } else if constexpr (R == kRoe) {
    flux_roe(l, r, n, f);
  } else {
    flux_exact(l, r, n, f, not_converged);
  }
}

// Interior face flux of the face kernels times the face weight w, from the
// two conservative states: Rusanov, Roe and HLLC take their conservative-
// input forms, which return false on degenerate states (rho <= 0, E < 0,
// p < 0; HLLC also p == 0); those states, and the Exact and AUSM solvers,
// take flux_upwind on the clamped primitives (ConservativeToPrimitive with
// SetZeroIfNegative).  FAST_SQRT selects the mixed form's seeded roots.
template <int R, bool FAST_SQRT>
MCFD_HD void interior_flux_weighted(const double *cl, const double *cr, const double *n,
                                    double w, double *f, bool *not_converged) {
  if constexpr (R == kRusanov) {
    flux_rusanov_cons_weighted<FAST_SQRT>(cl, cr, n, w, f);
    return;
  }
  if constexpr (R == kRoe) {
    if (flux_roe_cons_weighted<FAST_SQRT>(cl, cr, n, w, f)) return;
  }
  if constexpr (R == kHllc) {
    if (flux_hllc_cons_weighted<FAST_SQRT>(cl, cr, n, w, f)) return;
  }
  if constexpr (R != kRusanov) {
    Prim l = cons_to_prim(cl[0], cl[1], cl[2], cl[3], cl[4]);
    Prim r = cons_to_prim(cr[0], cr[1], cr[2], cr[3], cr[4]);
    flux_upwind<R>(l, r, n, f, not_converged);
#pragma unroll
    for (int k = 0; k < kK; ++k) f[k] *= w;
  }
}

// Boundary fluxes (rotated/euler.hpp:144-318) for the holder side state `in`
// and the given value `g` at the face point.
template <int R>
MCFD_HD void flux_boundary(int kind, const Prim &in, const double *g,
                           const double *n, double *f, bool *not_converged) {
  switch (kind) {
    case kBcInviscidWall:
      f[0] = 0;
      f[1] = in.p * n[0];
      f[2] = in.p * n[1];
      f[3] = in.p * n[2];
      f[4] = 0;
      break;
    case kBcSupersonicInlet: {
      Prim w = cons_to_prim(g[0], g[1], g[2], g[3], g[4]);
      double un = w.u * n[0] + w.v * n[1] + w.w * n[2];
      normal_flux(w, prim_energy(w), n, un, f);
      break;
    }
    case kBcSupersonicOutlet: {
      double un = in.u * n[0] + in.v * n[1] + in.w * n[2];
      normal_flux(in, prim_energy(in), n, un, f);
      break;
    }
    case kBcSubsonicInlet: {
      // Carlson (2011) 2.7 as in rotated/euler.hpp:181-236
      double c_interior = sound_speed(in);
      double un_in = in.u * n[0] + in.v * n[1] + in.w * n[2];
      double riemann_interior = -un_in - c_interior * kGm1Under2;
      double A = n[0] * g[1] + n[1] * g[2] + n[2] * g[3];
      double sa = A * A;
      double gamma_times_r = kGamma * kGasR;
      double qa = sa + kGm1Under2;
      double qb = riemann_interior;
      double qc = kGm1Over2 * (riemann_interior * riemann_interior) -
                  sa * gamma_times_r * g[4];
      double sd = sqrt(qb * qb - qa * qc);
      double c_b = fmax((-qb + sd) / qa, (-qb - sd) / qa);
      double t_b = (c_b * c_b) / gamma_times_r;
      double mach = sqrt((g[4] / t_b - 1) / kGm1Over2);
      double p_b = g[0] / pow(1 + kGm1Over2 * mach * mach, kGammaOverGm1);
      double speed = mach * c_b;
      Prim w = make_prim(p_b / kGasR / t_b, g[1] * speed, g[2] * speed, g[3] * speed, p_b);
      double un = w.u * n[0] + w.v * n[1] + w.w * n[2];
      normal_flux(w, prim_energy(w), n, un, f);
      break;
    }
    case kBcSubsonicOutlet: {
      double rt = in.p / in.rho;
      Prim w = in;
      w.p = g[4];
      w.rho = w.p / rt;
      w.rinv = w.rho > 0 ? 1.0 / w.rho : 0.0;
      double un = w.u * n[0] + w.v * n[1] + w.w * n[2];
      normal_flux(w, prim_energy(w), n, un, f);
      break;
    }
    case kBcSmart: {
      Prim w = cons_to_prim(g[0], g[1], g[2], g[3], g[4]);
      flux_upwind<R>(in, w, n, f, not_converged);
      break;
    }
    default:
      for (int k = 0; k < kK; ++k) f[k] = 0;
  }
}

}  // namespace mcfd
