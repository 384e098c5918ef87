// The face kernels' regrouped Riemann fluxes against the reference-ordered
// primitive forms of the same header, on the host (no GPU):
//   HLLC     the selected side's star flux (S*(S_k U - F) + S_k p* D) / (S_k - S*)
//            against F_k + S_k (U*_k - U_k) with the star state of hllc.hpp;
//   Roe      F_L + sum_k min(l_k, 0) alpha_k r_k against the average
//            (F_L + F_R) / 2 - sum_k |l_k| alpha_k r_k / 2;
//   Rusanov  the summed side fluxes with the dissipation in each side's
//            velocity factor against the averaged form.
// Every form takes the face weight w.  State pairs: mild, high pressure,
// high velocity, low density, blast waves (pressure ratio 1e5) and near
// vacuum.  Prints the worst row-scaled difference per solver and exits 1 if
// one exceeds 1e-12 or a flux is finite in one form and not in the other.
#include <cmath>
#include <cstdio>
#include <random>

#include "../../pvcriemannsolvers_gb300/csrc/euler.cuh"

using namespace mcfd;

namespace {

void make_state(std::mt19937_64 &g, int mode, bool right, double *c) {
  std::uniform_real_distribution<double> U(0, 1);
  double rho = 0.2 + U(g), p = 0.2 + U(g), vs = 1.0;
  if (mode == 1) p *= 1e3;
  if (mode == 2) vs = 5.0;
  if (mode == 3) rho *= 1e-3;
  if (mode == 4) {
    rho = right ? 0.125 + U(g) : 1 + 5 * U(g);
    p = right ? 0.01 * (0.5 + U(g)) : 1000 * (0.5 + U(g));
  }
  if (mode == 5) {
    rho = 1e-6 + 1e-3 * U(g);
    p = 1e-6 + 1e-3 * U(g);
  }
  const double u = (2 * U(g) - 1) * vs, v = (2 * U(g) - 1) * vs, w = (2 * U(g) - 1) * vs;
  c[0] = rho;
  c[1] = rho * u;
  c[2] = rho * v;
  c[3] = rho * w;
  c[4] = p / kGm1 + 0.5 * rho * (u * u + v * v + w * w);
}

template <int R>
double worst_difference(const char *name, int *mismatch) {
  std::mt19937_64 g(17 + R);
  std::uniform_real_distribution<double> U(0, 1);
  double worst = 0;
  for (int it = 0; it < 300000; ++it) {
    const int mode = it % 6;
    double cl[kK], cr[kK], f[kK], ref[kK];
    make_state(g, mode, false, cl);
    make_state(g, mode, true, cr);
    double n[3] = {2 * U(g) - 1, 2 * U(g) - 1, 2 * U(g) - 1};
    const double nn = std::sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
    for (double &x : n) x /= nn;
    const double w = 0.3 + U(g);
    bool not_converged = false;
    interior_flux_weighted<R, false>(cl, cr, n, w, f, &not_converged);
    const Prim l = cons_to_prim(cl[0], cl[1], cl[2], cl[3], cl[4]);
    const Prim r = cons_to_prim(cr[0], cr[1], cr[2], cr[3], cr[4]);
    flux_upwind<R>(l, r, n, ref, &not_converged);
    double scale = 0, diff = 0;
    for (int k = 0; k < kK; ++k) {
      ref[k] *= w;
      if (std::isfinite(f[k]) != std::isfinite(ref[k])) ++*mismatch;
      if (std::isfinite(ref[k])) {
        scale = std::fmax(scale, std::fabs(ref[k]));
        diff = std::fmax(diff, std::fabs(f[k] - ref[k]));
      }
    }
    worst = std::fmax(worst, diff / (1 + scale));
  }
  std::printf("%s %.3e\n", name, worst);
  return worst;
}

}  // namespace

int main() {
  int mismatch = 0;
  double worst = 0;
  worst = std::fmax(worst, worst_difference<kHllc>("hllc", &mismatch));
  worst = std::fmax(worst, worst_difference<kRoe>("roe", &mismatch));
  worst = std::fmax(worst, worst_difference<kRusanov>("rusanov", &mismatch));
  std::printf("finiteness mismatches %d\n", mismatch);
  return (worst <= 1e-12 && mismatch == 0) ? 0 : 1;
}
