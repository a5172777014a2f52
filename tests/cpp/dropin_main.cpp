// C++ host program driving the GPU path through include/gbfem.hpp the way a
// dune-fem user drives GalerkinOperator + KrylovInverseOperator
// (cf. dune/fem/solver/test/inverseoperatortest.cc): build the operator, bind
// it with a preconditioner, solve, check the residual.  Exit code 0 = pass.
#include <cmath>
#include <cstdio>
#include <vector>

#include "gbfem.hpp"

using namespace gbfem_cpp;

int main() {
  gbfem_dg_desc d{};
  d.grid.dim = 3;
  for (int k = 0; k < 3; ++k) {
    d.grid.cells[k] = 8;
    d.grid.lower[k] = 0.0;
    d.grid.upper[k] = 1.0;
  }
  d.order = 2;
  d.quad_points = 0;
  d.precision = GBFEM_F64;
  d.diffusion = 1.0;
  d.penalty = 90.0;
  d.weak_dirichlet = 1;
  GpuOperator op = GpuOperator::dg(d);
  const std::int64_t n = op.size();
  std::vector<double> fh(n, 0.0);
  for (std::int64_t c = 0; c < n / 27; ++c) fh[c * 27] = 1.0 / 512.0;  // int_K 1 phi_0
  GpuDiscreteFunction f("f", n), u("u", n), w("w", n);
  f.copyFromHost(fh.data());
  GpuPreconditioner bj = GpuPreconditioner::blockJacobi(op);
  for (int method : {GBFEM_SOLVER_CG, GBFEM_SOLVER_GMRES, GBFEM_SOLVER_BICGSTAB, GBFEM_SOLVER_FCG}) {
    // preconditioned CG/FCG test the preconditioned or true residual against
    // eps ||b||; 1e-11 leaves room for the difference below 1e-9
    GpuKrylovInverseOperator inv(method, 1e-11, GBFEM_TOL_RELATIVE);
    inv.bind(op, bj);
    u.clear();
    inv(f, u);
    op(u, w);
    w -= f;
    const double rel = std::sqrt(w.normSquaredDofs() / f.normSquaredDofs());
    std::printf("method %d: iterations %d, relative residual %.3e\n", method, inv.iterations(), rel);
    if (!inv.info().converged || !(rel < 1e-9)) return 1;
  }
  // explicit time loop: TimeProvider + SSP-RK3 on a periodic advection operator
  gbfem_dg_desc a = d;
  for (int k = 0; k < 3; ++k) a.grid.periodic[k] = 1;
  a.diffusion = 0.0;
  a.weak_dirichlet = 0;
  a.velocity[0] = 1.0;
  a.velocity[1] = 0.5;
  GpuOperator adv = GpuOperator::dg(a);
  TimeProvider tp(0.0, 0.2);
  GpuExplicitRungeKuttaSolver ode(adv, tp);
  GpuDiscreteFunction v("v", n);
  v.copyFromHost(fh.data());
  ode.initialize(v);
  int steps = 0;
  for (tp.init(); tp.time() < 0.05; tp.next()) {
    ode.solve(v);
    ++steps;
  }
  std::vector<double> vh(n);
  v.copyToHost(vh.data());
  double mass = 0.0;
  for (std::int64_t c = 0; c < n / 27; ++c) mass += vh[c * 27];
  std::printf("time loop: %d steps of %.4e to t = %.4f, mean %.15f\n", steps, tp.deltaT(), tp.time(), mass);
  if (steps < 1 || std::fabs(mass - 1.0) > 1e-12) return 2;
  // Newton on the Bratu problem -lap u = 3 e^u through NewtonInverseOperator
  gbfem_reaction r{0.0, 0.0, -3.0};
  GpuOperator bratu = GpuOperator::nonlinearDG(d, r);
  if (!bratu.nonlinear()) return 3;
  GpuNewtonInverseOperator newton;
  newton.parameter().tolerance = 1e-10;
  newton.parameter().max_iterations = 50;
  newton.parameter().preconditioner = GBFEM_PC_BLOCK_JACOBI;
  newton.parameter().linear.tolerance = 1e-12;
  newton.parameter().linear.error_measure = GBFEM_TOL_RELATIVE;
  newton.bind(bratu);
  GpuDiscreteFunction zero("zero", n), sol("sol", n);
  newton(zero, sol);
  std::printf("Newton (Bratu): %d iterations, %d linear, |residual| %.3e\n", newton.iterations(),
              newton.linearIterations(), newton.residual());
  if (!newton.converged() || newton.iterations() > 8) return 4;
  // jacobian(u, jOp), assembled, with an SSOR-preconditioned CG
  GpuOperator jac = bratu.jacobianOperator();
  bratu.jacobian(sol, jac);
  GpuOperator assembled = jac.assemble();
  GpuPreconditioner ssor = GpuPreconditioner::sor(assembled, GBFEM_SMOOTHER_SSOR);
  GpuKrylovInverseOperator cg(GBFEM_SOLVER_CG, 1e-12, GBFEM_TOL_RELATIVE);
  cg.bind(assembled, ssor);
  u.clear();
  cg(f, u);
  jac(u, w);
  w -= f;
  const double relj = std::sqrt(w.normSquaredDofs() / f.normSquaredDofs());
  std::printf("SSOR-CG on the assembled Jacobian: %d iterations, relative residual %.3e\n", cg.iterations(), relj);
  if (!cg.info().converged || !(relj < 1e-9)) return 5;
  return 0;
}
