// Minimal stand-in for dune-fem's solver/parameter.hh: only the tolerance
// criteria constants the linear solver templates use.
#ifndef GBFEM_SHIM_DUNE_FEM_SOLVER_PARAMETER_HH
#define GBFEM_SHIM_DUNE_FEM_SOLVER_PARAMETER_HH
namespace Dune {
namespace Fem {
namespace LinearSolver {
struct ToleranceCriteria {
  static const int absolute = 0;
  static const int relative = 1;
  static const int residualReduction = 2;
};
}  // namespace LinearSolver
}  // namespace Fem
}  // namespace Dune
#endif
