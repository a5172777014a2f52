// Stands in for dune/fem/solver/parameter.hh when compiling dune-fem's
// NewtonInverseOperator and FemPreconditioning against the shim layer: the
// linear solver's tolerance criteria and preconditioner ids (as in the
// reference) and a minimal SolverParameter holding what the Newton loop reads
// from it (tolerance, iteration limit, error measure), with the reference's
// clone() through LocalParameter.
#ifndef GBFEM_SHIM_DG_SOLVER_PARAMETER_HH
#define GBFEM_SHIM_DG_SOLVER_PARAMETER_HH
#include <limits>
#include <string>
#include "minidune.hh"
#include <dune/fem/common/staticlistofint.hh>
namespace Dune {
namespace Fem {
namespace LinearSolver {
struct ToleranceCriteria {
  static const int absolute = 0;
  static const int relative = 1;
  static const int residualReduction = 2;
};
}  // namespace LinearSolver

struct SolverParameter : public LocalParameter<SolverParameter, SolverParameter> {
  // preconditioner ids as in the reference's Preconditioners list
  static const int none = 1, ssor = 2, sor = 3, ilu = 4, gauss_seidel = 5, jacobi = 6;
  SolverParameter(const std::string& keyPrefix = "fem.solver.",
                  const ParameterReader& parameter = Parameter::container())
      : keyPrefix_(keyPrefix), parameter_(parameter) {}
  const ParameterReader& parameter() const { return parameter_; }
  bool threading() const { return false; }
  virtual void reset() { tolerance_ = -1; errorMeasure_ = -1; }
  virtual double tolerance() const {
    if (tolerance_ < 0) tolerance_ = parameter_.getValue<double>(keyPrefix_ + "tolerance", 1e-8);
    return tolerance_;
  }
  virtual void setTolerance(double tol) { tolerance_ = tol; }
  virtual int maxIterations() const {
    return parameter_.getValue<int>(keyPrefix_ + "maxiterations", std::numeric_limits<int>::max());
  }
  virtual int errorMeasure() const { return errorMeasure_ < 0 ? defaultErrorMeasure_ : errorMeasure_; }
  virtual void setDefaultErrorMeasure(int m) { defaultErrorMeasure_ = m; }

 protected:
  std::string keyPrefix_;
  ParameterReader parameter_;
  mutable double tolerance_ = -1;
  mutable int errorMeasure_ = -1;
  int defaultErrorMeasure_ = 0;
};
}  // namespace Fem
}  // namespace Dune
#endif
