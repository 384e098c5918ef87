// mcfd_system.hpp -- header-only C++ adapter that plugs the GPU library into
// the reference's temporal layer.
//
// mini::temporal::System<Scalar> (include/mini/temporal/ode.hpp:17-48) has
// four virtuals; RungeKutta<order>::Update (include/mini/temporal/rk.hpp)
// calls only those.  GpuSystem<Base> derives from the reference's System (or
// any class with the same four virtuals and a Column type offering data(),
// size() and a size constructor, e.g. Eigen::VectorXd) and forwards each
// virtual to the C ABI, so the reference's own RungeKutta drives the GPU
// residual unchanged.  The spatial extras (GetTimeStep, boundary
// registration) and the fused update are forwarded as ordinary methods.
//
// Errors: the reference reports failures by exception (root.hpp:67); every
// non-zero status of the C ABI becomes a std::runtime_error carrying
// mcfd_last_error().
#ifndef MCFD_SYSTEM_HPP_
#define MCFD_SYSTEM_HPP_

#include <cstdint>
#include <stdexcept>
#include <string>

#include "mcfd.h"

namespace mcfd {

inline void Check(int status, const mcfd_handle *h) {
  if (status != MCFD_OK) {
    throw std::runtime_error("mcfd error " + std::to_string(status) + ": " +
                             mcfd_last_error(h));
  }
}

template <class SystemBase>
class GpuSystem : public SystemBase {
 public:
  using Column = typename SystemBase::Column;

  // Takes ownership of a handle made by mcfd_create.
  explicit GpuSystem(mcfd_handle *handle) : h_(handle) {
    if (!h_) throw std::invalid_argument("null mcfd handle");
  }
  GpuSystem(const GpuSystem &) = delete;
  GpuSystem &operator=(const GpuSystem &) = delete;
  ~GpuSystem() { mcfd_destroy(h_); }

  // ---- mini::temporal::System<Scalar>
  void SetTime(double t_curr) override { Check(mcfd_set_time(h_, t_curr), h_); }
  void SetSolutionColumn(Column const &column) override {
    Check(mcfd_set_solution(h_, column.data(), static_cast<int64_t>(column.size())), h_);
  }
  Column GetSolutionColumn() const override {
    Column column(static_cast<size_t>(mcfd_column_size(h_)));
    Check(mcfd_get_solution(h_, column.data(), static_cast<int64_t>(column.size())), h_);
    return column;
  }
  Column GetResidualColumn() const override {
    Column column(static_cast<size_t>(mcfd_column_size(h_)));
    Check(mcfd_residual(h_, column.data(), static_cast<int64_t>(column.size())), h_);
    return column;
  }

  // ---- spatial::FiniteElement extras (fem.hpp:196-222, 417-435)
  double GetTimeStep(double dt_guess, int rk_order) const {
    double dt = 0;
    Check(mcfd_time_step(h_, dt_guess, rk_order, &dt), h_);
    return dt;
  }
  void SetBoundary(int32_t group, mcfd_bc_state const &state) {
    Check(mcfd_set_bc(h_, group, &state), h_);
  }

  // ---- the fused device update: same result as RungeKutta<order>::Update
  // on this system, without host round trips between stages.
  void Update(double t_curr, double dt, int order) {
    Check(mcfd_rk_step(h_, t_curr, dt, order), h_);
  }
  // n steps of { dt = GetTimeStep(dt_guess, order); Update(t, dt); t += dt }.
  double Advance(int n_steps, double dt_guess, int order, double t_curr) {
    Check(mcfd_advance(h_, n_steps, dt_guess, order, &t_curr), h_);
    return t_curr;
  }

  mcfd_handle *handle() const { return h_; }

 private:
  mcfd_handle *h_;
};

}  // namespace mcfd

#endif  // MCFD_SYSTEM_HPP_
