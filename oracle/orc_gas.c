/*
 * ORACLE (test infrastructure only): ideal gas, 1D normal-frame Riemann
 * solvers, rotated-frame wrapper and boundary fluxes, restated from the
 * reference project.  Parity checker and CPU baseline; never shipped.
 *
 * Reference sources restated here (pvcStillInGradSchool/pvcRiemannSolvers):
 *   include/mini/riemann/euler/types.hpp:186-334   IdealGas<double, 1.4>
 *   include/mini/riemann/euler/exact.hpp:44-320    Exact
 *   include/mini/riemann/euler/hllc.hpp:30-109     HartenLaxLeerContact
 *   include/mini/riemann/euler/ausm.hpp:146-187    AdvectionUpstreamSplitting
 *   python/riemann.py:405-455                      Roe (1D, no entropy fix)
 *   python/riemann.py:457-476                      LaxFriedrichs (Rusanov)
 *   include/mini/riemann/rotated/euler.hpp:42-345  rotated::Euler
 */
#include <math.h>
#include <string.h>

#include "orc.h"

/* Constants evaluated the way the reference's constexpr helpers do
 * (types.hpp:206-247): each is computed from Gamma() in double arithmetic. */
#define G_GAMMA 1.4
static const double kR = 287.05;
#define G_GM1 (G_GAMMA - 1.0)
#define G_GP1 (G_GAMMA + 1.0)

static double one_over_gamma(void) { return 1.0 / G_GAMMA; }
static double gp1_over_2(void) { return G_GP1 / 2; }
static double gp1_over_4(void) { return G_GP1 / 4; }
static double one_over_gm1(void) { return 1.0 / G_GM1; }
static double gamma_over_gm1(void) { return G_GAMMA / G_GM1; }
static double gm1_over_gamma(void) { return G_GM1 / G_GAMMA; }
static double gm1_over_2(void) { return G_GM1 / 2; }
static double gm1_under_2(void) { return 2 / G_GM1; }

/* SetZeroIfNegative (types.hpp:194-202). */
static void set_zero_if_negative(double *w) {
  if (w[0] < 0) memset(w, 0, sizeof(double) * ORC_K);
  if (w[4] < 0) memset(w, 0, sizeof(double) * ORC_K);
}

static double kinetic_energy(const double *w) {
  return 0.5 * (w[1] * w[1] + w[2] * w[2] + w[3] * w[3]);
}

/* ConservativeToPrimitive (types.hpp:288-301). */
void orc_cons_to_prim(const double *cons, double *w) {
  memcpy(w, cons, sizeof(double) * ORC_K);
  set_zero_if_negative(w);
  if (w[0] != 0) {
    w[1] /= w[0];
    w[2] /= w[0];
    w[3] /= w[0];
    w[4] -= w[0] * kinetic_energy(w);
    w[4] *= G_GM1;
    set_zero_if_negative(w);
  }
}

/* PrimitiveToConservative (types.hpp:302-311). */
void orc_prim_to_cons(const double *w, double *cons) {
  memcpy(cons, w, sizeof(double) * ORC_K);
  cons[1] *= w[0];
  cons[2] *= w[0];
  cons[3] *= w[0];
  cons[4] *= one_over_gm1();
  cons[4] += w[0] * kinetic_energy(w);
}

/* PrimitiveToFlux along x (types.hpp:312-321). */
static void prim_to_flux(const double *w, double *flux) {
  orc_prim_to_cons(w, flux);
  for (int k = 0; k < ORC_K; ++k) flux[k] *= w[1];
  flux[1] += w[4];
  flux[4] += w[4] * w[1];
}

/* GetFluxMatrix (types.hpp:322-333), row-major 5x3. */
void orc_flux_matrix(const double *cv, double *mat) {
  double pv[ORC_K];
  orc_cons_to_prim(cv, pv);
  double u = pv[1], v = pv[2], w = pv[3], p = pv[4];
  double rho_u = cv[1], rho_v = cv[2], rho_w = cv[3];
  double rho_h0 = cv[4] + p;
  double col0[5] = {rho_u, rho_u * u + p, rho_v * u, rho_w * u, rho_h0 * u};
  double col1[5] = {rho_v, rho_u * v, rho_v * v + p, rho_w * v, rho_h0 * v};
  double col2[5] = {rho_w, rho_u * w, rho_v * w, rho_w * w + p, rho_h0 * w};
  for (int r = 0; r < 5; ++r) {
    mat[r * 3 + 0] = col0[r];
    mat[r * 3 + 1] = col1[r];
    mat[r * 3 + 2] = col2[r];
  }
}

/* GetSpeedOfSound(rho, p) (types.hpp:252-254). */
static double speed_of_sound(const double *w) {
  return (w[0] > 0 && w[4] > 0) ? sqrt(G_GAMMA * w[4] / w[0]) : 0;
}

/* rotated::Euler::GetMaximumSpeed (rotated/euler.hpp:340-345). */
double orc_max_speed(const double *cons) {
  double w[ORC_K];
  orc_cons_to_prim(cons, w);
  double c = speed_of_sound(w);
  double u = sqrt(w[1] * w[1] + w[2] * w[2] + w[3] * w[3]);
  return fmax(c + u, c - u);
}

/* ------------------------------------------------------------------ */
/* Exact solver (exact.hpp).                                           */

typedef struct {
  double rho_before, p_before, a_before, p_const;
} speed_change;

static speed_change speed_change_make(const double *before) {
  speed_change s;
  s.rho_before = before[0];
  s.p_before = before[4];
  s.a_before = before[0] == 0 ? 0 : speed_of_sound(before);
  s.p_const = before[4] * gm1_over_2();
  return s;
}

static double sc_P(const speed_change *s, double p_after) {
  return gp1_over_2() * p_after + s->p_const;
}

static double sc_value(const speed_change *s, double p_after) {
  double value;
  if (p_after >= s->p_before) {
    double divisor = sqrt(s->rho_before * sc_P(s, p_after));
    value = (p_after - s->p_before) / divisor;
  } else {
    double exponent = gm1_over_2() / G_GAMMA;
    value = pow(p_after / s->p_before, exponent) - 1;
    value *= gm1_under_2() * s->a_before;
  }
  return value;
}

static double sc_prime(const speed_change *s, double p_after) {
  double value;
  if (p_after >= s->p_before) {
    double p = sc_P(s, p_after);
    value = gp1_over_4() * (s->p_before - p_after);
    double divisor = sqrt(s->rho_before * p);
    value = (1 + value / p) / divisor;
  } else {
    double exponent = -gp1_over_2() / G_GAMMA;
    double divisor = s->rho_before * s->a_before;
    value = pow(p_after / s->p_before, exponent) / divisor;
  }
  return value;
}

/* The Newton loop of exact.hpp:140-152 has no iteration cap; the restatement
 * caps both loops at 4096 iterations (a converged case needs < 30). */
static double exact_find_root(const speed_change *l, const speed_change *r,
                              double du, double x) {
  const double eps = 1e-8;
#define F_OF(p) (sc_value(l, (p)) + sc_value(r, (p)) + du)
  for (int it = 0; F_OF(x) > 0 && it < 4096; ++it) x *= 0.5;
  for (int it = 0; F_OF(x) < -eps && it < 4096; ++it) {
    double divisor = sc_prime(l, x) + sc_prime(r, x);
    x -= F_OF(x) / divisor;
  }
#undef F_OF
  return x;
}

static void prim_inside_expansion(double gri_1, double gri_2, double *axis) {
  double r = G_GM1 / G_GP1;
  double a = r * gri_2;
  double a_square = a * a;
  double rho = pow(a_square / gri_1 * one_over_gamma(), one_over_gm1());
  memset(axis, 0, sizeof(double) * ORC_K);
  axis[0] = rho;
  axis[1] = a;
  axis[4] = a_square * rho * one_over_gamma();
}

/* Shock<kField> (exact.hpp:202-234) */
static void prim_near_shock(int field, const double *before, double *after,
                            double *result) {
  double u = before[1];
  double divisor = (after[1] - before[1]) * before[0];
  u += (divisor != 0 ? (after[4] - before[4]) / divisor : before[1]);
  int after_shock = field == 1 ? (u < 0) : (u > 0);
  if (after_shock) {
    after[0] = before[0];
    double d = after[1] - u;
    after[0] *= (before[1] - u) / d;
    memcpy(result, after, sizeof(double) * ORC_K);
  } else {
    memcpy(result, before, sizeof(double) * ORC_K);
  }
}

/* Expansion<kField> (exact.hpp:236-292) */
static void prim_near_expansion(int field, const double *before, double *after,
                                double *result) {
  double a_before = speed_of_sound(before);
  double gri_1 = before[4] / pow(before[0], G_GAMMA);
  double gri_2, a_after;
  if (field == 1) {
    gri_2 = before[1] + gm1_under_2() * a_before;
    a_after = a_before + gm1_over_2() * (before[1] - after[1]);
  } else {
    gri_2 = before[1] - gm1_under_2() * a_before;
    a_after = a_before - gm1_over_2() * (before[1] - after[1]);
  }
  int after_wave = field == 1 ? (after[1] - a_after < 0)
                              : (after[1] + a_after > 0);
  int before_wave = field == 1 ? (before[1] - a_before > 0)
                               : (before[1] + a_before < 0);
  if (after_wave) {
    double divisor = a_after * a_after;
    after[0] = G_GAMMA * after[4] / divisor;
    memcpy(result, after, sizeof(double) * ORC_K);
  } else if (before_wave) {
    memcpy(result, before, sizeof(double) * ORC_K);
  } else {
    prim_inside_expansion(gri_1, gri_2, result);
  }
}

/* PrimitiveNearVacuum (exact.hpp:293-320) */
static void prim_near_vacuum(const double *left, const double *right,
                             double *result) {
  double left_a = speed_of_sound(left);
  if (left[1] > left_a) {
    memcpy(result, left, sizeof(double) * ORC_K);
    return;
  }
  double right_a = speed_of_sound(right);
  if (right[1] + right_a < 0) {
    memcpy(result, right, sizeof(double) * ORC_K);
    return;
  }
  double gri_1 = left[4] / pow(left[0], G_GAMMA);
  double gri_2 = left[1] + left_a * gm1_under_2();
  if (gri_2 >= 0) {
    prim_inside_expansion(gri_1, gri_2, result);
  } else {
    gri_1 = right[4] / pow(right[0], G_GAMMA);
    gri_2 = right[1] - right_a * gm1_under_2();
    if (gri_2 < 0) {
      prim_inside_expansion(gri_1, gri_2, result);
    } else {
      memset(result, 0, sizeof(double) * ORC_K);
    }
  }
}

/* Exact::GetPrimitiveUpwind (exact.hpp:36-42, 62-138).  The reference keeps
 * star_u as member state across calls; vacuum branches leave it untouched.
 * The restatement uses a fresh solver's value (0) there, i.e. the passive
 * scalars come from the right state in vacuum cases. */
static void exact_prim_upwind(const double *left, const double *right,
                              double *result) {
  double star_u = 0.0;
  memset(result, 0, sizeof(double) * ORC_K);
  int done = 0;
  if (left[0] > 0) {
    if (!(right[0] > 0)) {  /* only right vacuum */
      double a_left = speed_of_sound(left);
      if (left[1] >= a_left) {
        memcpy(result, left, sizeof(double) * ORC_K);
      } else {
        double u_star = left[1] + a_left * gm1_under_2();
        if (u_star <= 0) {
          memset(result, 0, sizeof(double) * ORC_K);
        } else {
          double gri_1 = left[4] / pow(left[0], G_GAMMA);
          prim_inside_expansion(gri_1, u_star, result);
        }
      }
      done = 1;
    }
  } else {
    if (right[0] > 0) {  /* only left vacuum */
      double a_right = speed_of_sound(right);
      if (right[1] + a_right <= 0) {
        memcpy(result, right, sizeof(double) * ORC_K);
      } else {
        double u_star = right[1] - a_right * gm1_under_2();
        if (u_star >= 0) {
          memset(result, 0, sizeof(double) * ORC_K);
        } else {
          double gri_1 = right[4] / pow(right[0], G_GAMMA);
          prim_inside_expansion(gri_1, u_star, result);
        }
      }
    } else {
      memset(result, 0, sizeof(double) * ORC_K);
    }
    done = 1;
  }
  if (!done) {
    double u_change_given = right[1] - left[1];
    speed_change l = speed_change_make(left), r = speed_change_make(right);
    double f0 = sc_value(&l, 0) + sc_value(&r, 0) + u_change_given;
    if (f0 < 0) {
      double star[ORC_K] = {0, 0, 0, 0, 0};
      star[4] = exact_find_root(&l, &r, u_change_given, left[4]);
      star[1] = 0.5 * (right[1] + sc_value(&r, star[4]) + left[1] -
                       sc_value(&l, star[4]));
      star_u = star[1];
      if (0 < star[1]) {
        if (star[4] >= left[4])
          prim_near_shock(1, left, star, result);
        else
          prim_near_expansion(1, left, star, result);
      } else {
        if (star[4] >= right[4])
          prim_near_shock(3, right, star, result);
        else
          prim_near_expansion(3, right, star, result);
      }
    } else {
      prim_near_vacuum(left, right, result);
    }
  }
  /* SetPassiveScalars (exact.hpp:56-60) */
  result[2] = star_u > 0 ? left[2] : right[2];
  result[3] = star_u > 0 ? left[3] : right[3];
}

static void exact_flux(const double *left, const double *right, double *flux) {
  double w[ORC_K];
  exact_prim_upwind(left, right, w);
  prim_to_flux(w, flux);
}

/* ------------------------------------------------------------------ */
/* HLLC (hllc.hpp:30-109).                                             */

static double hllc_q(double p_estimate, double p_k) {
  if (p_estimate <= p_k) return 1.0;
  double temp = 1 + gp1_over_2() * (p_estimate / p_k - 1) / G_GAMMA;
  return sqrt(temp);
}

static void hllc_star_flux(const double *state, double wave_k,
                           double wave_star, double *flux) {
  double u_k[ORC_K], u_star[ORC_K];
  prim_to_flux(state, flux);
  orc_prim_to_cons(state, u_k);
  double energy = u_k[4];
  double temp = state[0] * (wave_k - state[1]) / (wave_k - wave_star);
  u_star[0] = temp;
  u_star[1] = temp * wave_star;
  u_star[2] = temp * state[2];
  u_star[3] = temp * state[3];
  u_star[4] = energy / state[0] + (wave_star - state[1]) *
      (wave_star + state[4] / (state[0] * (wave_k - state[1])));
  u_star[4] *= temp;
  for (int k = 0; k < ORC_K; ++k) {
    u_star[k] -= u_k[k];
    u_star[k] *= wave_k;
    flux[k] += u_star[k];
  }
}

static void hllc_flux(const double *left, const double *right, double *flux) {
  double rho_average = (left[0] + right[0]) / 2;
  double a_left = speed_of_sound(left);
  double a_right = speed_of_sound(right);
  double a_average = (a_left + a_right) / 2;
  double p_pvrs = (left[4] + right[4] -
                   (right[1] - left[1]) * rho_average * a_average) / 2;
  double p_estimate = fmax(0.0, p_pvrs);
  double wave_left = left[1] - a_left * hllc_q(p_estimate, left[4]);
  double wave_right = right[1] + a_right * hllc_q(p_estimate, right[4]);
  double wave_star = (right[4] - left[4] +
                      left[0] * left[1] * (wave_left - left[1]) -
                      right[0] * right[1] * (wave_right - right[1])) /
                     (left[0] * (wave_left - left[1]) -
                      right[0] * (wave_right - right[1]));
  if (0.0 <= wave_left) {
    prim_to_flux(left, flux);
  } else if (wave_right <= 0.0) {
    prim_to_flux(right, flux);
  } else if (0.0 <= wave_star) {
    hllc_star_flux(left, wave_left, wave_star, flux);
  } else if (wave_star < 0.0) {
    hllc_star_flux(right, wave_right, wave_star, flux);
  } else {
    /* NaN wave speeds: the reference returns an unset flux. */
    for (int k = 0; k < ORC_K; ++k) flux[k] = NAN;
  }
}

/* ------------------------------------------------------------------ */
/* AUSM (ausm.hpp:146-187).                                            */

static void ausm_signed_flux(int negative, const double *state, double *flux) {
  double a = speed_of_sound(state);
  double h = a * a / G_GM1 + kinetic_energy(state);
  flux[0] = 1;
  flux[1] = state[1];
  flux[2] = state[2];
  flux[3] = state[3];
  flux[4] = h;
  double mach = state[1] / a;
  double p = state[4];
  double signed_mach = (1 + (negative ? -mach : mach)) * 0.5;
  if (mach >= -1 && mach <= 1) {
    double m2 = signed_mach * signed_mach;
    mach = negative ? -m2 : m2;
    p *= signed_mach;
  } else if (signed_mach < 0) {
    mach = 0.0;
    p = 0.0;
  }
  double scale = state[0] * a * mach;
  for (int k = 0; k < ORC_K; ++k) flux[k] *= scale;
  flux[1] += p;
}

static void ausm_flux(const double *left, const double *right, double *flux) {
  double fl[ORC_K], fr[ORC_K];
  ausm_signed_flux(0, left, fl);
  ausm_signed_flux(1, right, fr);
  for (int k = 0; k < ORC_K; ++k) flux[k] = fl[k] + fr[k];
}

/* ------------------------------------------------------------------ */
/* Roe (python/riemann.py:405-455) restated in 3D: the three waves of the
 * 1D prototype plus the two shear waves (speed u, strength rho*dv, rho*dw),
 * no entropy fix.  With v = w = 0 it is the 1D prototype's flux.          */

static void roe_flux(const double *l, const double *r, double *flux) {
  double fl[ORC_K], fr[ORC_K];
  prim_to_flux(l, fl);
  prim_to_flux(r, fr);
  for (int k = 0; k < ORC_K; ++k) flux[k] = (fl[k] + fr[k]) / 2;
  /* total enthalpy h0 = a^2/(gamma-1) + |v|^2/2 (python/equation.py:200-203) */
  double h0_l = G_GAMMA * l[4] / l[0] / G_GM1 + kinetic_energy(l);
  double h0_r = G_GAMMA * r[4] / r[0] / G_GM1 + kinetic_energy(r);
  double sl = sqrt(l[0]), sr = sqrt(r[0]);
  double ssum = sl + sr;
  double rho = sl * sr;
  double u = (sl * l[1] + sr * r[1]) / ssum;
  double v = (sl * l[2] + sr * r[2]) / ssum;
  double w = (sl * l[3] + sr * r[3]) / ssum;
  double ke = (u * u + v * v + w * w) / 2;
  double h0 = (sl * h0_l + sr * h0_r) / ssum;
  double aa = G_GM1 * (h0 - ke);
  double a = sqrt(aa);
  double ua = u * a;
  double p_jump = r[4] - l[4];
  double u_jump = r[1] - l[1];
  /* 1st wave: u - a */
  double alpha = (p_jump - rho * a * u_jump) / (2 * aa);
  double s = 0.5 * alpha * fabs(u - a);
  double r1[ORC_K] = {1, u - a, v, w, h0 - ua};
  for (int k = 0; k < ORC_K; ++k) flux[k] -= s * r1[k];
  /* 2nd wave (entropy): u */
  alpha = (r[0] - l[0]) - p_jump / aa;
  s = 0.5 * alpha * fabs(u);
  double r2[ORC_K] = {1, u, v, w, ke};
  for (int k = 0; k < ORC_K; ++k) flux[k] -= s * r2[k];
  /* shear waves: u */
  double sv = 0.5 * rho * (r[2] - l[2]) * fabs(u);
  double sw = 0.5 * rho * (r[3] - l[3]) * fabs(u);
  flux[2] -= sv;
  flux[4] -= sv * v;
  flux[3] -= sw;
  flux[4] -= sw * w;
  /* 3rd wave: u + a */
  alpha = (p_jump + rho * a * u_jump) / (2 * aa);
  s = 0.5 * alpha * fabs(u + a);
  double r3[ORC_K] = {1, u + a, v, w, h0 + ua};
  for (int k = 0; k < ORC_K; ++k) flux[k] -= s * r3[k];
}

/* ------------------------------------------------------------------ */
/* Rusanov = local Lax-Friedrichs (python/riemann.py:457-476).         */

static void rusanov_flux(const double *l, const double *r, double *flux) {
  double fl[ORC_K], fr[ORC_K], ul[ORC_K], ur[ORC_K];
  prim_to_flux(r, fr);
  prim_to_flux(l, fl);
  for (int k = 0; k < ORC_K; ++k) flux[k] = (fr[k] + fl[k]) / 2;
  double al = speed_of_sound(l), ar = speed_of_sound(r);
  double lam = fmax(fabs(l[1] - al), fabs(l[1] + al));
  lam = fmax(lam, fmax(fabs(r[1] - ar), fabs(r[1] + ar)));
  orc_prim_to_cons(l, ul);
  orc_prim_to_cons(r, ur);
  for (int k = 0; k < ORC_K; ++k) flux[k] -= lam / 2 * (ur[k] - ul[k]);
}

void orc_flux_1d(int kind, const double *l, const double *r, double *flux) {
  switch (kind) {
    case ORC_EXACT: exact_flux(l, r, flux); break;
    case ORC_HLLC: hllc_flux(l, r, flux); break;
    case ORC_AUSM: ausm_flux(l, r, flux); break;
    case ORC_ROE: roe_flux(l, r, flux); break;
    case ORC_RUSANOV: rusanov_flux(l, r, flux); break;
    default:
      for (int k = 0; k < ORC_K; ++k) flux[k] = NAN;
  }
}

/* ------------------------------------------------------------------ */
/* rotated::Euler (rotated/euler.hpp).  frame rows: a = normal, b, c.  */

static void global_to_normal(const double *f, double *v) {
  double p_a = v[1] * f[0] + v[2] * f[1] + v[3] * f[2];
  double p_b = v[1] * f[3] + v[2] * f[4] + v[3] * f[5];
  double p_c = v[1] * f[6] + v[2] * f[7] + v[3] * f[8];
  v[1] = p_a;
  v[2] = p_b;
  v[3] = p_c;
}

static void normal_to_global(const double *f, double *v) {
  double p_x = v[1] * f[0] + v[2] * f[3] + v[3] * f[6];
  double p_y = v[1] * f[1] + v[2] * f[4] + v[3] * f[7];
  double p_z = v[1] * f[2] + v[2] * f[5] + v[3] * f[8];
  v[1] = p_x;
  v[2] = p_y;
  v[3] = p_z;
}

static void global_prim_to_global_flux(const double *frame, double *w,
                                       double *flux) {
  global_to_normal(frame, w);
  prim_to_flux(w, flux);
  normal_to_global(frame, flux);
}

void orc_flux_rotated(int kind, const double *frame, const double *cons_l,
                      const double *cons_r, double *flux) {
  double wl[ORC_K], wr[ORC_K];
  orc_cons_to_prim(cons_l, wl);
  orc_cons_to_prim(cons_r, wr);
  global_to_normal(frame, wl);
  global_to_normal(frame, wr);
  orc_flux_1d(kind, wl, wr, flux);
  normal_to_global(frame, flux);
}

static void flux_subsonic_inlet(const double *frame, const double *cons_in,
                                const double *given, double *flux) {
  double w[ORC_K];
  orc_cons_to_prim(cons_in, w);
  double c_interior = speed_of_sound(w);
  global_to_normal(frame, w);
  double riemann_interior = -w[1] - c_interior * gm1_under_2();
  double u_cos = given[1], v_cos = given[2], w_cos = given[3];
  double t_total = given[4];
  double A = frame[0] * u_cos + frame[1] * v_cos + frame[2] * w_cos;
  double square_of_A = A * A;
  double gamma_times_R = G_GAMMA * kR;
  double qa = square_of_A + gm1_under_2();
  double qb_half = riemann_interior;
  double qc = gm1_over_2() * (riemann_interior * riemann_interior) -
              square_of_A * gamma_times_R * t_total;
  double sqrt_delta = sqrt(qb_half * qb_half - qa * qc);
  double x_1 = (-qb_half + sqrt_delta) / qa;
  double x_2 = (-qb_half - sqrt_delta) / qa;
  double c_boundary = fmax(x_1, x_2);
  double t_boundary = (c_boundary * c_boundary) / gamma_times_R;
  /* GetMachFromTemperature (types.hpp:273-280) */
  double ratio = t_total / t_boundary;
  double mach_boundary = sqrt((ratio - 1) / gm1_over_2());
  double p_total = given[0];
  /* TotalPressureToPressure (types.hpp:268-272) */
  double factor = pow(1 + gm1_over_2() * mach_boundary * mach_boundary,
                      gamma_over_gm1());
  double p_boundary = p_total / factor;
  double speed_boundary = mach_boundary * c_boundary;
  w[4] = p_boundary;
  w[0] = p_boundary / kR / t_boundary;
  w[1] = u_cos * speed_boundary;
  w[2] = v_cos * speed_boundary;
  w[3] = w_cos * speed_boundary;
  global_prim_to_global_flux(frame, w, flux);
}

static void flux_subsonic_outlet(const double *frame, const double *cons_in,
                                 const double *given, double *flux) {
  double w[ORC_K];
  orc_cons_to_prim(cons_in, w);
  double rt_interior = w[4] / w[0];
  double p_boundary = given[4];
  w[4] = p_boundary;
  w[0] = w[4] / rt_interior;
  global_prim_to_global_flux(frame, w, flux);
}

void orc_flux_boundary(int riemann, int bc_kind, const double *frame,
                       const double *cons_in, const double *given,
                       double *flux) {
  double w[ORC_K];
  switch (bc_kind) {
    case ORC_BC_INVISCID_WALL:  /* euler.hpp:160-174 (no Riemann problem) */
      orc_cons_to_prim(cons_in, w);
      memset(flux, 0, sizeof(double) * ORC_K);
      flux[1] = w[4];
      normal_to_global(frame, flux);
      break;
    case ORC_BC_SUPERSONIC_INLET:  /* euler.hpp:144-147 */
      orc_cons_to_prim(given, w);
      global_prim_to_global_flux(frame, w, flux);
      break;
    case ORC_BC_SUPERSONIC_OUTLET:  /* euler.hpp:148-151 */
      orc_cons_to_prim(cons_in, w);
      global_prim_to_global_flux(frame, w, flux);
      break;
    case ORC_BC_SUBSONIC_INLET:
      flux_subsonic_inlet(frame, cons_in, given, flux);
      break;
    case ORC_BC_SUBSONIC_OUTLET:
      flux_subsonic_outlet(frame, cons_in, given, flux);
      break;
    case ORC_BC_SMART:  /* euler.hpp:296-299: upwind(interior, given) */
      orc_flux_rotated(riemann, frame, cons_in, given, flux);
      break;
    default:
      memset(flux, 0, sizeof(double) * ORC_K);
  }
}
