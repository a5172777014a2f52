// gbfem.hpp -- C++ host-side wrappers over the C-ABI (gbfem.h), shaped after
// dune-fem's interfaces so that code written against them can use the GPU
// path unchanged:
//
//   GpuDiscreteFunction       the DiscreteFunction subset the Krylov
//                             templates use (function/common/discretefunction.hh:
//                             781-901, function/adaptivefunction/adaptivefunction.hh);
//                             dofs live in device memory.
//   GpuOperator               Operator<D,R>::operator()(u,w) const
//                             (operator/common/operator.hh:32-65).
//   GpuPreconditioner         any Operator<D,D> used as a preconditioner.
//   GpuKrylovInverseOperator  InverseOperatorInterface: bind/unbind,
//                             operator()(f,u), iterations(), info()
//                             (solver/inverseoperatorinterface.hh:33-239,
//                             solver/krylovinverseoperators.hh:46-274).
//
// Errors become exceptions (the reference throws DUNE_THROW); a
// non-converged solve is a negative iteration count, not an exception, as in
// the reference.
#ifndef GBFEM_HPP
#define GBFEM_HPP

#include <cmath>
#include <cstddef>
#include <cstdint>
#include <algorithm>
#include <limits>
#include <memory>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "gbfem.h"

namespace gbfem_cpp {

struct Error : std::runtime_error {
  int code;
  Error(int c, const std::string& m) : std::runtime_error(m), code(c) {}
};

inline void check(int rc) {
  if (rc != GBFEM_OK) throw Error(rc, gbfem_last_error());
}

// Serial communication stand-ins for the calls the reference's templates make
// on space().gridPart().comm() and space().auxiliaryDofs().
struct SerialComm {
  template <class T>
  void sum(T*, int) const {}
  template <class T>
  T sum(T x) const { return x; }
};
struct GridPartStub {
  SerialComm c;
  const SerialComm& comm() const { return c; }
};
struct AuxiliaryDofs {
  std::size_t n = 0;
  std::size_t size() const { return 1; }
  std::size_t operator[](std::size_t) const { return n; }
};
struct SpaceStub {
  GridPartStub gp;
  AuxiliaryDofs aux;
  const GridPartStub& gridPart() const { return gp; }
  const AuxiliaryDofs& auxiliaryDofs() const { return aux; }
};

// A dof vector in device memory with the DiscreteFunction operations the
// Krylov loops need.  All reductions are FP64-accumulated and deterministic.
class GpuDiscreteFunction {
 public:
  typedef double RangeFieldType;
  typedef double DofType;

  GpuDiscreteFunction(std::string name, std::int64_t size, int precision = GBFEM_F64)
      : name_(std::move(name)), n_(size), prec_(precision), space_(std::make_shared<SpaceStub>()) {
    space_->aux.n = std::size_t(size);
    void* p = nullptr;
    check(gbfem_malloc(&p, bytes()));
    data_.reset(p, [](void* q) { gbfem_free(q); });
    clear();
  }
  GpuDiscreteFunction(const GpuDiscreteFunction& o) : GpuDiscreteFunction(o.name_, o.n_, o.prec_) { assign(o); }
  GpuDiscreteFunction& operator=(const GpuDiscreteFunction& o) {
    assign(o);
    return *this;
  }

  const std::string& name() const { return name_; }
  std::int64_t size() const { return n_; }
  int precision() const { return prec_; }
  void* leakPointer() { return data_.get(); }
  const void* leakPointer() const { return data_.get(); }
  const SpaceStub& space() const { return *space_; }

  void clear() { check(gbfem_memset(data_.get(), 0, bytes())); }
  void assign(const GpuDiscreteFunction& o) { check(gbfem_copy(prec_, n_, o.data_.get(), data_.get(), nullptr)); }
  void axpy(double a, const GpuDiscreteFunction& x) { check(gbfem_axpy(prec_, n_, a, x.data_.get(), data_.get(), nullptr)); }
  GpuDiscreteFunction& operator+=(const GpuDiscreteFunction& x) { axpy(1.0, x); return *this; }
  GpuDiscreteFunction& operator-=(const GpuDiscreteFunction& x) { axpy(-1.0, x); return *this; }
  GpuDiscreteFunction& operator*=(double a) {
    check(gbfem_scal(prec_, n_, a, data_.get(), nullptr));
    return *this;
  }
  double scalarProductDofs(const GpuDiscreteFunction& x) const {
    double r = 0.0;
    check(gbfem_dot(prec_, n_, data_.get(), x.data_.get(), &r, nullptr));
    return r;
  }
  double normSquaredDofs() const { return scalarProductDofs(*this); }

  void copyFromHost(const void* h) { check(gbfem_memcpy_h2d(data_.get(), h, bytes())); }
  void copyToHost(void* h) const { check(gbfem_memcpy_d2h(h, data_.get(), bytes())); }

 private:
  std::size_t bytes() const { return std::size_t(n_) * (prec_ == GBFEM_F64 ? 8 : 4); }
  std::string name_;
  std::int64_t n_;
  int prec_;
  std::shared_ptr<SpaceStub> space_;
  std::shared_ptr<void> data_;
};

// forEachPrimaryDof over the serial auxiliary-dof list (space/common/auxiliarydofs.hh:303-315)
template <class F>
void forEachPrimaryDof(const AuxiliaryDofs& a, F&& f) {
  for (std::size_t i = 0; i < a.n; ++i) f(i);
}

// Device versions of the two free functions dune-fem's GMRES and BiCGstab
// templates call on the dof arrays (solver/linear/gmres.hh:61-85,
// solver/linear/bicgstab.hh:19-49).  They are found by argument-dependent
// lookup and, being more specialised, chosen over the host loops.
template <class Communication, class FieldType>
void gemv(const Communication&, const int m, std::vector<GpuDiscreteFunction>& v, const GpuDiscreteFunction& vjp,
          FieldType* y) {
  for (int l = 0; l < m; ++l) y[l] = vjp.scalarProductDofs(v[l]);
}
template <class FieldType>
void scalarProductVecs(const GpuDiscreteFunction& r, const GpuDiscreteFunction& s, const GpuDiscreteFunction& rs,
                       FieldType* d) {
  d[0] = r.scalarProductDofs(s);
  d[1] = r.scalarProductDofs(r);
  d[2] = s.scalarProductDofs(s);
  d[3] = s.scalarProductDofs(rs);
  d[4] = r.scalarProductDofs(rs);
}

// Operator<D,R>: w = op(u).
class GpuOperator {
 public:
  explicit GpuOperator(gbfem_operator op) : op_(op, [](gbfem_operator p) { gbfem_operator_destroy(p); }) {}
  static GpuOperator dg(const gbfem_dg_desc& d) {
    gbfem_operator op = nullptr;
    check(gbfem_dg_operator_create(&d, &op));
    return GpuOperator(op);
  }
  void operator()(const GpuDiscreteFunction& u, GpuDiscreteFunction& w) const {
    check(gbfem_operator_apply(op_.get(), u.leakPointer(), w.leakPointer(), nullptr));
  }
  bool nonlinear() const {
    int v = 0;
    check(gbfem_operator_nonlinear(op_.get(), &v));
    return v != 0;
  }
  // S(u) = A u + int r(u) v, r = linear u + cubic u^3 + exponential e^u
  static GpuOperator nonlinearDG(const gbfem_dg_desc& d, const gbfem_reaction& r) {
    gbfem_operator op = nullptr;
    check(gbfem_dg_nonlinear_operator_create(&d, &r, &op));
    return GpuOperator(op);
  }
  // DifferentiableOperator::jacobian(u, jOp): jOp from jacobianOperator()
  GpuOperator jacobianOperator() const {
    gbfem_operator j = nullptr;
    check(gbfem_operator_jacobian_create(op_.get(), &j));
    return GpuOperator(j);
  }
  void jacobian(const GpuDiscreteFunction& u, GpuOperator& jOp) const {
    check(gbfem_operator_jacobian(op_.get(), u.leakPointer(), jOp.handle(), nullptr));
  }
  // the assembled (block-sparse) copy
  GpuOperator assemble() const {
    gbfem_operator a = nullptr;
    check(gbfem_operator_assemble(op_.get(), &a));
    return GpuOperator(a);
  }
  std::int64_t size() const {
    std::int64_t n = 0;
    check(gbfem_operator_size(op_.get(), &n));
    return n;
  }
  gbfem_operator handle() const { return op_.get(); }

 private:
  std::shared_ptr<gbfem_operator_s> op_;
};

// A preconditioner z = P(r), callable like an Operator<D,D>.
class GpuPreconditioner {
 public:
  explicit GpuPreconditioner(gbfem_preconditioner pc)
      : pc_(pc, [](gbfem_preconditioner p) { gbfem_preconditioner_destroy(p); }) {}
  static GpuPreconditioner diagonal(const GpuOperator& op) {
    gbfem_preconditioner pc = nullptr;
    check(gbfem_preconditioner_diagonal_create(op.handle(), &pc));
    return GpuPreconditioner(pc);
  }
  static GpuPreconditioner blockJacobi(const GpuOperator& op, int precision = GBFEM_F64) {
    gbfem_preconditioner pc = nullptr;
    check(gbfem_preconditioner_block_jacobi_create(op.handle(), precision, &pc));
    return GpuPreconditioner(pc);
  }
  // FemPreconditioning jacobi / gauss-seidel / sor / ssor of an assembled
  // operator (GBFEM_SMOOTHER_*); the operator must outlive the preconditioner
  static GpuPreconditioner sor(const GpuOperator& assembled, int method, int n = 1, double w = 1.0) {
    gbfem_preconditioner pc = nullptr;
    check(gbfem_preconditioner_sor_create(assembled.handle(), method, n, w, &pc));
    return GpuPreconditioner(pc);
  }
  void operator()(const GpuDiscreteFunction& r, GpuDiscreteFunction& z) const {
    check(gbfem_preconditioner_apply(pc_.get(), r.leakPointer(), z.leakPointer(), nullptr));
  }
  gbfem_preconditioner handle() const { return pc_.get(); }

 private:
  std::shared_ptr<gbfem_preconditioner_s> pc_;
};

// InverseOperatorInterface-shaped Krylov solver (parameter keys as
// fem.solver.*: method, tolerance, errormeasure, maxiterations, gmres.restart).
class GpuKrylovInverseOperator {
 public:
  struct SolverInfo {  // Impl::SolverInfo (solver/inverseoperatorinterface.hh:15-30)
    bool converged;
    int linearIterations;
    int nonlinearIterations;
    std::vector<double> timing;
  };
  explicit GpuKrylovInverseOperator(int method = GBFEM_SOLVER_CG, double tolerance = 1e-8,
                                    int errorMeasure = GBFEM_TOL_ABSOLUTE) {
    check(gbfem_solver_params_default(&prm_));
    prm_.method = method;
    prm_.tolerance = tolerance;
    prm_.error_measure = errorMeasure;
  }
  void bind(const GpuOperator& op) { op_ = &op; pc_ = nullptr; }
  void bind(const GpuOperator& op, const GpuPreconditioner& pc) { op_ = &op; pc_ = &pc; }
  void unbind() { op_ = nullptr; pc_ = nullptr; }
  void setMaxIterations(int it) { prm_.max_iterations = it; }
  void setRestart(int m) { prm_.restart = m; }
  // u = op^{-1}(f); u is the initial guess.
  void operator()(const GpuDiscreteFunction& f, GpuDiscreteFunction& u) const {
    if (!op_) throw Error(GBFEM_ERR_INVALID, "GpuKrylovInverseOperator: no operator bound");
    check(gbfem_solve(op_->handle(), pc_ ? pc_->handle() : nullptr, &prm_, f.leakPointer(), u.leakPointer(), &info_));
  }
  int iterations() const { return info_.iterations; }
  SolverInfo info() const { return SolverInfo{info_.converged != 0, info_.iterations, 0, {info_.time_ms}}; }
  const gbfem_solver_info& raw() const { return info_; }

 private:
  gbfem_solver_params prm_{};
  mutable gbfem_solver_info info_{};
  const GpuOperator* op_ = nullptr;
  const GpuPreconditioner* pc_ = nullptr;
};

// NewtonInverseOperator (solver/newtoninverseoperator.hh:484-790):
// bind(op), operator()(rhs, w) with w the initial guess, iterations(),
// linearIterations(), info(); parameters as gbfem_newton_params.
class GpuNewtonInverseOperator {
 public:
  GpuNewtonInverseOperator() { check(gbfem_newton_params_default(&prm_)); }
  explicit GpuNewtonInverseOperator(const gbfem_newton_params& prm) : prm_(prm) {}
  gbfem_newton_params& parameter() { return prm_; }
  void bind(const GpuOperator& op) { op_ = &op; }
  void unbind() { op_ = nullptr; }
  void operator()(const GpuDiscreteFunction& rhs, GpuDiscreteFunction& w) const {
    if (!op_) throw Error(GBFEM_ERR_INVALID, "GpuNewtonInverseOperator: no operator bound");
    check(gbfem_newton_solve(op_->handle(), &prm_, rhs.leakPointer(), w.leakPointer(), &info_));
  }
  int iterations() const { return info_.iterations; }
  int linearIterations() const { return info_.linear_iterations; }
  bool converged() const { return info_.converged != 0; }
  int failed() const { return info_.failure; }  // NewtonFailure
  double residual() const { return info_.residual; }

 private:
  gbfem_newton_params prm_{};
  mutable gbfem_newton_info info_{};
  const GpuOperator* op_ = nullptr;
};

// TimeProvider (solver/timeprovider.hh:35-200, 403-592), single process:
// deltaT = min(factor * estimate, upper bound), re-fixed every updateStep calls
// of init/next; the estimate and bound are reset after each fix.
class TimeProvider {
 public:
  explicit TimeProvider(double startTime = 0.0, double cfl = 1.0, int updateStep = 1)
      : time_(startTime), cfl_(cfl), updateStep_(updateStep), counter_(updateStep) {
    initTimeStepEstimate();
  }
  void init() { initTimeStep(dtEstimate_); }
  void init(double timeStep) { initTimeStep(timeStep); }
  void next() {
    if (!dtEstimateValid_) throw Error(GBFEM_ERR_INVALID, "TimeProvider::next: no time step estimate provided");
    advance();
    initTimeStep(dtEstimate_);
  }
  void next(double timeStep) {
    advance();
    initTimeStep(timeStep);
  }
  double time() const { return time_; }
  int timeStep() const { return valid(), timeStep_; }
  double deltaT() const { return valid(), dt_; }
  double inverseDeltaT() const { return valid(), 1.0 / dt_; }
  double factor() const { return cfl_; }
  double timeStepEstimate() const { return dtEstimate_; }
  void provideTimeStepEstimate(double dt) {
    dtEstimate_ = std::min(dtEstimate_, dt);
    dtEstimateValid_ = true;
  }
  void provideTimeStepUpperBound(double bound) {
    dtUpperBound_ = std::min(dtUpperBound_, bound);
    dtEstimateValid_ = true;
  }
  void invalidateTimeStep() { valid_ = false; }
  bool timeStepValid() const { return valid_; }

 private:
  bool valid() const {
    if (!valid_) throw Error(GBFEM_ERR_INVALID, "TimeProvider: time step not valid");
    return true;
  }
  void advance() {
    if (valid_) {
      time_ += dt_;
      ++timeStep_;
    }
  }
  void initTimeStepEstimate() {
    dtEstimate_ = std::numeric_limits<double>::max();
    dtUpperBound_ = std::numeric_limits<double>::max();
    dtEstimateValid_ = false;
  }
  void initTimeStep(double dtEstimate) {
    if (++counter_ >= updateStep_) {
      dt_ = std::min(cfl_ * dtEstimate, dtUpperBound_);
      valid_ = dt_ > 0.0;
      counter_ = 0;
    }
    initTimeStepEstimate();
  }
  double time_ = 0.0;
  int timeStep_ = 0;
  double dt_ = 0.0;
  bool valid_ = false;
  bool dtEstimateValid_ = false;
  double dtEstimate_ = 0.0, dtUpperBound_ = 0.0;
  double cfl_;
  int updateStep_, counter_;
};

// ExplicitRungeKuttaSolver with the TVD3 table over the MOL DG operator
// (solver/rungekutta/explicit.hh:145-215): initialize() provides the
// operator's estimate, solve(u) steps by tp.deltaT() and provides it again.
class GpuExplicitRungeKuttaSolver {
 public:
  GpuExplicitRungeKuttaSolver(const GpuOperator& op, TimeProvider& tp, int powerIterations = 30)
      : tp_(tp) {
    gbfem_rk_solver rk = nullptr;
    check(gbfem_rk3_create(op.handle(), &rk));
    rk_ = std::shared_ptr<gbfem_rk_solver_s>(rk, [](gbfem_rk_solver p) { gbfem_rk3_destroy(p); });
    check(gbfem_dg_time_step_estimate(op.handle(), powerIterations, 0, &estimate_, &upperBound_));
  }
  void initialize(const GpuDiscreteFunction&) {
    provide();
    initialized_ = true;
  }
  void solve(GpuDiscreteFunction& u) {
    if (!initialized_) throw Error(GBFEM_ERR_INVALID, "ExplicitRungeKuttaSolver wasn't initialized before first call!");
    check(gbfem_rk3_step(rk_.get(), u.leakPointer(), tp_.deltaT(), nullptr));
    provide();
  }
  int stages() const { return 3; }

 private:
  void provide() {
    const double big = std::numeric_limits<double>::max();
    if (estimate_ < big) tp_.provideTimeStepEstimate(estimate_);
    if (upperBound_ < big) tp_.provideTimeStepUpperBound(upperBound_);
  }
  TimeProvider& tp_;
  std::shared_ptr<gbfem_rk_solver_s> rk_;
  double estimate_ = 0.0, upperBound_ = 0.0;
  bool initialized_ = false;
};

}  // namespace gbfem_cpp

#endif  // GBFEM_HPP
