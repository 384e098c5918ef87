// Drop-in check: a System base with the reference's four virtuals
// (include/mini/temporal/ode.hpp:17-48) and an SSP-RK3 driver making the
// reference's call sequence (include/mini/temporal/rk.hpp:31-49,
// ode.hpp:121-133) drive the GPU library through mcfd::GpuSystem, compared
// with the fused device update on a second handle.  Prints the relative L2
// difference; exits non-zero on failure.
#include <cmath>
#include <cstdio>
#include <vector>

#include "mcfd.h"
#include "mcfd_system.hpp"

namespace {

// Column with the Eigen::VectorXd operations the driver needs.
struct Column {
  std::vector<double> v;
  Column() = default;
  explicit Column(size_t n) : v(n) {}
  double *data() { return v.data(); }
  const double *data() const { return v.data(); }
  size_t size() const { return v.size(); }
  Column &operator*=(double s) { for (auto &x : v) x *= s; return *this; }
  Column &operator/=(double s) { for (auto &x : v) x /= s; return *this; }
  Column &operator+=(const Column &o) { for (size_t i = 0; i < v.size(); ++i) v[i] += o.v[i]; return *this; }
};

struct System {
  using Column = ::Column;
  virtual ~System() = default;
  virtual void SetTime(double t) = 0;
  virtual void SetSolutionColumn(Column const &) = 0;
  virtual Column GetSolutionColumn() const = 0;
  virtual Column GetResidualColumn() const = 0;
};

Column NextSolution(System *s, double t, double dt) {
  s->SetTime(t);
  Column u = s->GetSolutionColumn();
  Column r = s->GetResidualColumn();
  r *= dt;
  u += r;
  return u;
}

void Rk3Update(System *s, double t, double dt) {
  Column u_curr = s->GetSolutionColumn();
  s->SetSolutionColumn(NextSolution(s, t, dt));
  Column u_next = u_curr;
  u_next *= 3;
  u_next += NextSolution(s, t + dt, dt);
  u_next /= 4;
  s->SetSolutionColumn(u_next);
  u_next = NextSolution(s, t + dt / 2, dt);
  u_next *= 2;
  u_next += u_curr;
  u_next /= 3;
  s->SetSolutionColumn(u_next);
}

// Periodic n^3 box of unit-size cells with the face conventions of
// pvcriemannsolvers_gb300/mesh.py.
struct Box {
  std::vector<double> xyz, shift;
  std::vector<int64_t> cells, fcells;
  std::vector<int32_t> fsides, fgroup;
};

Box MakeBox(int n) {
  Box b;
  auto node = [n](int i, int j, int k) { return (int64_t)((k * (n + 1) + j) * (n + 1) + i); };
  auto cell = [n](int i, int j, int k) { return (int64_t)((k * n + j) * n + i); };
  for (int k = 0; k <= n; ++k)
    for (int j = 0; j <= n; ++j)
      for (int i = 0; i <= n; ++i) {
        b.xyz.push_back(i); b.xyz.push_back(j); b.xyz.push_back(k);
      }
  for (int k = 0; k < n; ++k)
    for (int j = 0; j < n; ++j)
      for (int i = 0; i < n; ++i) {
        int64_t c[8] = {node(i, j, k), node(i + 1, j, k), node(i + 1, j + 1, k), node(i, j + 1, k),
                        node(i, j, k + 1), node(i + 1, j, k + 1), node(i + 1, j + 1, k + 1), node(i, j + 1, k + 1)};
        b.cells.insert(b.cells.end(), c, c + 8);
      }
  const int lower[3] = {4, 1, 0}, upper[3] = {2, 3, 5};
  for (int k = 0; k < n; ++k)
    for (int j = 0; j < n; ++j)
      for (int i = 0; i < n; ++i)
        for (int ax = 0; ax < 3; ++ax) {
          int idx[3] = {i, j, k};
          int nb[3] = {i, j, k};
          nb[ax] = (idx[ax] + 1) % n;
          bool wrap = idx[ax] == n - 1;
          int64_t a = cell(i, j, k), s = cell(nb[0], nb[1], nb[2]);
          double sh[3] = {0, 0, 0};
          if (wrap) {  // holder = lower id (the cell at index 0), normal -axis
            b.fcells.push_back(s); b.fcells.push_back(a);
            b.fsides.push_back(lower[ax]); b.fsides.push_back(upper[ax]);
            sh[ax] = -n;
          } else {
            b.fcells.push_back(a); b.fcells.push_back(s);
            b.fsides.push_back(upper[ax]); b.fsides.push_back(lower[ax]);
          }
          b.fgroup.push_back(-1);
          b.shift.insert(b.shift.end(), sh, sh + 3);
        }
  return b;
}

}  // namespace

int main() {
  const int n = 4, p = 2, Q = p + 1, N = Q * Q * Q;
  Box b = MakeBox(n);
  mcfd_mesh_desc d{};
  d.n_nodes = (int64_t)b.xyz.size() / 3;
  d.xyz = b.xyz.data();
  d.n_cells = (int64_t)b.cells.size() / 8;
  d.cell_nodes = b.cells.data();
  d.n_faces = (int64_t)b.fgroup.size();
  d.face_cells = b.fcells.data();
  d.face_sides = b.fsides.data();
  d.face_group = b.fgroup.data();
  d.face_shift = b.shift.data();
  mcfd_options o{};
  o.degree = p;
  o.riemann = MCFD_HLLC;
  mcfd_handle *h1 = nullptr, *h2 = nullptr;
  if (mcfd_create(&d, &o, &h1) || mcfd_create(&d, &o, &h2)) {
    std::printf("create failed: %s\n", mcfd_last_error(nullptr));
    return 1;
  }
  mcfd::GpuSystem<System> sys(h1), fused(h2);
  // smooth initial data at the GLL nodes
  const double x3[3] = {-1, 0, 1};
  Column u(static_cast<size_t>(mcfd_column_size(h1)));
  for (int64_t c = 0; c < d.n_cells; ++c)
    for (int q = 0; q < N; ++q) {
      const int64_t *cn = &b.cells[c * 8];
      double x = b.xyz[cn[0] * 3] + 0.5 * (1 + x3[q / (Q * Q)]);
      double y = b.xyz[cn[0] * 3 + 1] + 0.5 * (1 + x3[(q / Q) % Q]);
      double rho = 1 + 0.2 * std::sin(2 * M_PI * x / n) * std::cos(2 * M_PI * y / n);
      double *s = &u.v[(c * N + q) * 5];
      s[0] = rho; s[1] = rho * 0.5; s[2] = rho * 0.3; s[3] = rho * 0.1;
      s[4] = 1.0 / 0.4 + 0.5 * rho * (0.25 + 0.09 + 0.01);
    }
  sys.SetSolutionColumn(u);
  fused.SetSolutionColumn(u);
  double t = 0;
  for (int step = 0; step < 3; ++step) {
    double dt = sys.GetTimeStep(1.0, 3);
    Rk3Update(&sys, t, dt);   // the reference's call sequence, host columns
    fused.Update(t, dt, 3);   // the fused device update
    t += dt;
  }
  Column a = sys.GetSolutionColumn(), f = fused.GetSolutionColumn();
  double num = 0, den = 0;
  for (size_t i = 0; i < a.size(); ++i) {
    num += (a.v[i] - f.v[i]) * (a.v[i] - f.v[i]);
    den += f.v[i] * f.v[i];
  }
  double rel = std::sqrt(num / den);
  std::printf("dropin_rk3: relative L2 (virtual-call RK3 vs fused RK3) = %.3e\n", rel);
  return rel <= 1e-12 ? 0 : 2;
}
