// Stands in for dune/fem/solver/inverseoperatorinterface.hh when compiling
// dune-fem's NewtonInverseOperator against the shim layer: the solver
// statistics record it returns (Impl::SolverInfo).
#ifndef GBFEM_SHIM_DG_INVERSEOPERATORINTERFACE_HH
#define GBFEM_SHIM_DG_INVERSEOPERATORINTERFACE_HH
#include <vector>
#include "minidune.hh"
namespace Dune {
namespace Fem {
namespace Impl {
struct SolverInfo {
  SolverInfo(bool c, int lin, int nonlin, const std::vector<double>& t)
      : converged(c), linearIterations(lin), nonlinearIterations(nonlin), timing(t) {}
  bool converged;
  int linearIterations;
  int nonlinearIterations;
  std::vector<double> timing;
};
}  // namespace Impl
}  // namespace Fem
}  // namespace Dune
#endif
