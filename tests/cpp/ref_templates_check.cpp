// Compile-time drop-in check: dune-fem's own LinearSolver::cg / gmres /
// bicgstab templates, instantiated with the GPU types of include/gbfem.hpp
// as the discrete function and the operator.  Compiled (not run) by
// tests/test_dropin.py where the dune-fem sources are available.
#include <complex>
#include <vector>

#include "gbfem.hpp"
#include <dune/fem/solver/linear/bicgstab.hh>
#include <dune/fem/solver/linear/cg.hh>
#include <dune/fem/solver/linear/gmres.hh>

using gbfem_cpp::forEachPrimaryDof;

int run(const gbfem_cpp::GpuOperator& op, const gbfem_cpp::GpuPreconditioner& pc, gbfem_cpp::GpuDiscreteFunction& x,
        const gbfem_cpp::GpuDiscreteFunction& b) {
  std::vector<gbfem_cpp::GpuDiscreteFunction> t(5, gbfem_cpp::GpuDiscreteFunction("t", x.size()));
  int it = Dune::Fem::LinearSolver::cg(op, &pc, t, x, b, 1e-10, 1000, 1);
  std::vector<gbfem_cpp::GpuDiscreteFunction> v(22, gbfem_cpp::GpuDiscreteFunction("v", x.size()));
  it += Dune::Fem::LinearSolver::gmres(op, &pc, v, x, b, 20, 1e-10, 1000, 1);
  std::vector<gbfem_cpp::GpuDiscreteFunction> s(6, gbfem_cpp::GpuDiscreteFunction("s", x.size()));
  it += Dune::Fem::LinearSolver::bicgstab(op, &pc, s, x, b, 1e-10, 1000, 1);
  return it;
}
