// Newton's method over a (nonlinear) DG operator: NewtonInverseOperator::
// operator() (solver/newtoninverseoperator.hh:688-790), its line search
// (:588-630), failure tests (:570-586) and the Eisenstat-Walker forcing of the
// linear tolerance (:44-81, :559-564), statement by statement.  The dof
// vectors stay on the device; the scalars (|r|, eta, the line-search factor)
// are host values, as in the reference.  Each Newton step linearises the
// operator (gbfem_operator_jacobian), builds the chosen preconditioner of the
// Jacobian and calls the Krylov solver of solver.cu.
#include <cuda_runtime.h>
#include <cfloat>
#include <chrono>
#include <climits>
#include <cmath>
#include <cstdio>

#include "gbfem_internal.cuh"
#include "operator_impl.hpp"

using namespace gbfem;

namespace {

struct DevVec {
  void* p = nullptr;
  ~DevVec() {
    if (p) cudaFree(p);
  }
};

struct Newton {
  gbfem_operator op;
  gbfem_newton_params prm;
  const void* rhs;
  void* w;
  long long n;
  int prec;
  void* residual;
  double delta = 0.0;
  int iterations = 0, linear_iterations = 0;
  bool step_completed = true;
  // Eisenstat-Walker state (EisenstatWalkerStrategy)
  double previous_eta = -1.0, previous_residual = -1.0;

  int failed() const {
    if (!(delta < DBL_MAX) || std::isnan(delta)) return GBFEM_NEWTON_INVALID_RESIDUAL;
    if (iterations >= prm.max_iterations) return GBFEM_NEWTON_TOO_MANY_ITERATIONS;
    if (linear_iterations >= prm.max_linear_iterations) return GBFEM_NEWTON_TOO_MANY_LINEAR_ITERATIONS;
    if (linear_iterations < 0) return GBFEM_NEWTON_LINEAR_SOLVER_FAILED;
    if (!step_completed) return GBFEM_NEWTON_LINE_SEARCH_FAILED;
    return GBFEM_NEWTON_SUCCESS;
  }
  bool converged() const { return failed() == GBFEM_NEWTON_SUCCESS; }

  // residual = S(w) - rhs; returns |residual|
  int eval_residual(double* norm) {
    GBFEM_TRY(gbfem_operator_apply(op, w, residual, nullptr));
    GBFEM_TRY(gbfem_axpy(prec, n, -1.0, rhs, residual, nullptr));
    double rr = 0.0;
    GBFEM_TRY(gbfem_dot(prec, n, residual, residual, &rr, nullptr));
    *norm = std::sqrt(rr);
    return GBFEM_OK;
  }

  double next_linear_tolerance(double current) {
    double eta = prm.eta_max;
    if (previous_eta >= 0.0) {
      const double eta_a = prm.gamma * current * current / (previous_residual * previous_residual);
      const double indicator = prm.gamma * previous_eta * previous_eta;
      const double eta_c = indicator < 0.1 ? std::min(eta_a, prm.eta_max) : std::min(prm.eta_max, std::max(eta_a, indicator));
      eta = std::min(prm.eta_max, std::max(eta_c, 0.5 * prm.tolerance / current));
    }
    previous_residual = current;
    previous_eta = eta;
    return eta;
  }
  void update_linear_tolerance() {
    if (prm.forcing == GBFEM_FORCING_EISENSTAT_WALKER) prm.linear.tolerance = next_linear_tolerance(delta);
  }

  // returns -1 (failed), 0 (no line search configured) or 1/0 (full step taken or not)
  int line_search(const void* dw, int* ls) {
    const double delta_old = delta;
    double rr = 0.0;
    GBFEM_TRY(gbfem_dot(prec, n, residual, residual, &rr, nullptr));
    delta = std::sqrt(rr);
    if (prm.line_search == GBFEM_LINESEARCH_NONE) {
      *ls = 0;
      return GBFEM_OK;
    }
    if (failed() == GBFEM_NEWTON_INVALID_RESIDUAL) {
      double test = 0.0;
      GBFEM_TRY(gbfem_dot(prec, n, dw, dw, &test, nullptr));
      if (!(test < DBL_MAX && !std::isnan(test))) delta = 2.0 * delta_old;
    }
    double factor = 1.0;
    const int no_line_search = delta < delta_old ? 1 : 0;
    int it = 0;
    while (delta >= delta_old) {
      const double delta_prev = delta;
      factor *= 0.5;
      if (prm.verbose) std::printf("    line search: %.6e > %.6e\n", delta, delta_old);
      if (std::fabs(delta - delta_old) < 1e-5 * delta) {
        *ls = -1;
        return GBFEM_OK;
      }
      GBFEM_TRY(gbfem_axpy(prec, n, factor, dw, w, nullptr));
      GBFEM_TRY(eval_residual(&delta));
      if (std::fabs(delta - delta_prev) < 1e-15) {
        *ls = -1;
        return GBFEM_OK;
      }
      if (failed() == GBFEM_NEWTON_INVALID_RESIDUAL) delta = 2.0 * delta_old;
      if (++it >= prm.max_line_search_iterations) {
        *ls = -1;
        return GBFEM_OK;
      }
    }
    *ls = no_line_search;
    return GBFEM_OK;
  }
};

struct PcHolder {
  gbfem_preconditioner pc = nullptr;
  ~PcHolder() {
    if (pc) gbfem_preconditioner_destroy(pc);
  }
};
struct OpHolder {
  gbfem_operator op = nullptr;
  ~OpHolder() {
    if (op) gbfem_operator_destroy(op);
  }
};

}  // namespace

extern "C" {

int gbfem_newton_params_default(gbfem_newton_params* prm) {
  if (!prm) return set_error(GBFEM_ERR_INVALID, "gbfem_newton_params_default: null argument");
  *prm = gbfem_newton_params{};
  prm->tolerance = 1e-6;
  prm->max_iterations = INT_MAX;
  prm->max_linear_iterations = -1;  // = linear.max_iterations
  prm->max_line_search_iterations = INT_MAX;
  prm->line_search = GBFEM_LINESEARCH_NONE;
  prm->forcing = GBFEM_FORCING_NONE;
  prm->eta_max = 0.99;
  prm->gamma = 0.1;
  prm->simplified = 0;
  prm->preconditioner = GBFEM_PC_NONE;
  prm->verbose = 0;
  prm->assembled = 0;
  GBFEM_TRY(gbfem_solver_params_default(&prm->linear));
  return GBFEM_OK;
}

int gbfem_newton_solve(gbfem_operator op, const gbfem_newton_params* prm_in, const void* rhs, void* w,
                       gbfem_newton_info* info) {
  if (!op || !prm_in || !rhs || !w || !info) return set_error(GBFEM_ERR_INVALID, "gbfem_newton_solve: null argument");
  if (op->kind != OpKind::DG) return set_error(GBFEM_ERR_NOT_IMPLEMENTED, "gbfem_newton_solve: DG operators only");
  const auto t0 = std::chrono::steady_clock::now();
  *info = gbfem_newton_info{};
  Newton nt;
  nt.op = op;
  nt.prm = *prm_in;
  if (nt.prm.max_linear_iterations < 0) nt.prm.max_linear_iterations = nt.prm.linear.max_iterations;
  nt.rhs = rhs;
  nt.w = w;
  nt.n = op->ndofs;
  nt.prec = op->precision;
  const bool nonlinear = op->nonlinear != 0;
  const size_t bytes = size_t(nt.n) * (nt.prec == GBFEM_F64 ? 8 : 4);
  DevVec res, dw;
  GBFEM_CUDA_TRY(cudaMalloc(&res.p, bytes));
  GBFEM_CUDA_TRY(cudaMalloc(&dw.p, bytes));
  nt.residual = res.p;
  OpHolder jac;
  GBFEM_TRY(gbfem_operator_jacobian_create(op, &jac.op));
  // initial residual r = S(w) - rhs
  GBFEM_TRY(nt.eval_residual(&nt.delta));
  nt.update_linear_tolerance();
  bool compute_jacobian = true;
  int idle_solves = 0;  // consecutive linear solves that made no iteration
  PcHolder pc;
  OpHolder mat;  // the assembled Jacobian (assembled = 1)
  if (nt.prm.verbose) std::printf("Start Newton: tol = %.3e\nNewton iteration 0: |residual| = %.6e\n", nt.prm.tolerance, nt.delta);
  while (true) {
    if (compute_jacobian) {
      GBFEM_TRY(gbfem_operator_jacobian(op, w, jac.op, nullptr));
      compute_jacobian = !nt.prm.simplified;
      if (pc.pc) {
        gbfem_preconditioner_destroy(pc.pc);
        pc.pc = nullptr;
      }
      if (nt.prm.assembled) {
        if (mat.op) {
          gbfem_operator_destroy(mat.op);
          mat.op = nullptr;
        }
        GBFEM_TRY(gbfem_operator_assemble(jac.op, &mat.op));
      }
      gbfem_operator J = nt.prm.assembled ? mat.op : jac.op;
      if (nt.prm.preconditioner == GBFEM_PC_DIAGONAL) GBFEM_TRY(gbfem_preconditioner_diagonal_create(J, &pc.pc));
      else if (nt.prm.preconditioner == GBFEM_PC_BLOCK_JACOBI)
        GBFEM_TRY(gbfem_preconditioner_block_jacobi_create(J, nt.prec, &pc.pc));
    }
    if (nt.prm.max_linear_iterations - nt.linear_iterations <= 0) break;
    gbfem_solver_params lp = nt.prm.linear;
    lp.max_iterations = nt.prm.max_linear_iterations - nt.linear_iterations;
    GBFEM_CUDA_TRY(cudaMemset(dw.p, 0, bytes));
    gbfem_solver_info li{};
    GBFEM_TRY(gbfem_solve(nt.prm.assembled ? mat.op : jac.op, pc.pc, &lp, nt.residual, dw.p, &li));
    if (li.iterations < 0) {
      nt.linear_iterations = li.iterations;
      break;
    }
    // A preconditioned CG stops on <r, B r> <= eps^2 <b, b> (cg.hh:62-67), which a
    // loose forcing term can meet before the first iteration: dw = 0 and the
    // step repeats unchanged.  The reference loop would repeat it until
    // max_iterations; here two such solves in a row end Newton as a linear
    // solver failure.
    idle_solves = li.iterations == 0 ? idle_solves + 1 : 0;
    if (idle_solves >= 2 && nt.delta >= nt.prm.tolerance) {
      nt.linear_iterations = -(nt.linear_iterations > 0 ? nt.linear_iterations : 1);
      break;
    }
    nt.linear_iterations += li.iterations;
    GBFEM_TRY(gbfem_axpy(nt.prec, nt.n, -1.0, dw.p, w, nullptr));  // w -= dw
    if (!nonlinear) break;
    GBFEM_TRY(gbfem_operator_apply(op, w, nt.residual, nullptr));
    GBFEM_TRY(gbfem_axpy(nt.prec, nt.n, -1.0, rhs, nt.residual, nullptr));
    int ls = 0;
    GBFEM_TRY(nt.line_search(dw.p, &ls));
    nt.step_completed = ls >= 0;
    nt.update_linear_tolerance();
    ++nt.iterations;
    if (nt.prm.verbose)
      std::printf("Newton iteration %d: |residual| = %.6e (linear %d)\n", nt.iterations, nt.delta, nt.linear_iterations);
    if (nt.delta < nt.prm.tolerance || !nt.converged()) break;
  }
  info->iterations = nt.iterations;
  info->linear_iterations = nt.linear_iterations;
  info->residual = nt.delta;
  info->failure = nt.failed();
  info->converged = info->failure == GBFEM_NEWTON_SUCCESS ? 1 : 0;
  info->time_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
  return GBFEM_OK;
}

}  // extern "C"
