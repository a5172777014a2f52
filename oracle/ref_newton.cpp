// Runs dune-fem's own Newton solver -- NewtonInverseOperator, NewtonParameter
// and its line search (dune/fem/solver/newtoninverseoperator.hh), compiled
// unmodified -- on S(w) = f, where S is the reference's DGEllipticOperator
// (dgelliptic.hh) with a nonlinear source and its Jacobian comes from
// DifferentiableDGEllipticOperator::jacobian, on the shim grid of
// oracle/shim_dg; prints, per case, the residual norm after every Newton
// step, the tolerance set for every linear solve, the iteration counts and
// the solution as JSON golden vectors.
// The linear inverse operator is an exact dense LU solve of our own (one
// "linear iteration" per Newton step), so the golden vectors record the
// Newton loop itself.  Built and run only by oracle/make_ref_golden.sh
// where the dune-fem sources are present; test infrastructure only.
//
// Model: flux diffusion * kappa(x) grad u (kappa as in ref_dgelliptic.cpp),
// source r(u) = c1 u + c3 u^3 + ce exp(u), do-nothing or periodic boundaries.
#include <config.h>

#include <cmath>
#include <cstdio>
#include <string>
#include <vector>

#include "dgspace.hh"
#include <dune/fem/schemes/dgelliptic.hh>
#include <dune/fem/solver/newtoninverseoperator.hh>

namespace refnt {

using Dune::Fem::Cell;
using Dune::Fem::ConstLocalFunction;
using Dune::Fem::DenseLinearOperator;
using Dune::Fem::DGFunction;
using Dune::Fem::Face;
using Dune::Fem::LegendreDGSpace;

struct ReactionDiffusionModel {
  typedef LegendreDGSpace::RangeType RangeType;
  typedef LegendreDGSpace::JacobianRangeType JacobianRangeType;
  ReactionDiffusionModel(const DGFunction* kappa, double diffusion, double c1, double c3, double ce)
      : diffusion_(diffusion), c1_(c1), c3_(c3), ce_(ce) {
    if (kappa) klf_.reset(new ConstLocalFunction<DGFunction>(*kappa));
  }
  bool init(const Cell& e) const {
    if (klf_) klf_->bind(e);
    return true;
  }
  template <class Point>
  double coefficient(const Point& x) const {
    if (!klf_) return diffusion_;
    RangeType k;
    klf_->evaluate(x, k);
    return diffusion_ * k[0];
  }
  template <class Point>
  void source(const Point&, const RangeType& u, const JacobianRangeType&, RangeType& s) const {
    s[0] = c1_ * u[0] + c3_ * u[0] * u[0] * u[0] + ce_ * std::exp(u[0]);
  }
  template <class Point>
  void flux(const Point& x, const RangeType&, const JacobianRangeType& du, JacobianRangeType& f) const {
    const double k = coefficient(x);
    for (int d = 0; d < 3; ++d) f[0][d] = k * du[0][d];
  }
  template <class Point>
  RangeType penalty(const Point& x, const RangeType&) const { return RangeType(coefficient(x)); }
  template <class Point>
  void linSource(const RangeType& u0, const JacobianRangeType&, const Point&, const RangeType& phi,
                 const JacobianRangeType&, RangeType& s) const {
    s[0] = (c1_ + 3.0 * c3_ * u0[0] * u0[0] + ce_ * std::exp(u0[0])) * phi[0];
  }
  template <class Point>
  void linFlux(const RangeType&, const JacobianRangeType&, const Point& x, const RangeType&,
               const JacobianRangeType& dphi, JacobianRangeType& f) const {
    const double k = coefficient(x);
    for (int d = 0; d < 3; ++d) f[0][d] = k * dphi[0][d];
  }
  void isDirichletIntersection(const Face&, std::array<int, 1>& components) const { components[0] = 0; }
  template <class Point>
  void dirichlet(int, const Point&, RangeType& g) const { g = RangeType(0.0); }

 private:
  double diffusion_, c1_, c3_, ce_;
  std::unique_ptr<ConstLocalFunction<DGFunction>> klf_;
};

// The linear inverse operator handed to the Newton solver: an exact solve of
// the dense Jacobian by Gaussian elimination with partial pivoting.  It
// records the tolerance the Newton loop set for each solve (the
// Eisenstat-Walker forcing terms, when that forcing is on).
class DenseLUInverse {
 public:
  typedef Dune::Fem::SolverParameter SolverParameterType;
  explicit DenseLUInverse(const SolverParameterType& p) : param_(p) {}
  void bind(const DenseLinearOperator& op) { op_ = &op; }
  void unbind() { op_ = nullptr; }
  void setMaxIterations(int) {}
  int iterations() const { return iterations_; }
  SolverParameterType& parameter() const { return param_; }
  const std::vector<double>& tolerances() const { return tolerances_; }
  void operator()(const DGFunction& f, DGFunction& x) const {
    tolerances_.push_back(param_.tolerance());
    const std::size_t n = op_->size();
    std::vector<double> a(n * n), b(f.dofs());
    for (std::size_t i = 0; i < n; ++i)
      for (std::size_t j = 0; j < n; ++j) a[i * n + j] = (*op_)(i, j);
    for (std::size_t k = 0; k < n; ++k) {
      std::size_t piv = k;
      for (std::size_t i = k + 1; i < n; ++i)
        if (std::fabs(a[i * n + k]) > std::fabs(a[piv * n + k])) piv = i;
      if (piv != k) {
        for (std::size_t j = 0; j < n; ++j) std::swap(a[k * n + j], a[piv * n + j]);
        std::swap(b[k], b[piv]);
      }
      for (std::size_t i = k + 1; i < n; ++i) {
        const double m = a[i * n + k] / a[k * n + k];
        for (std::size_t j = k; j < n; ++j) a[i * n + j] -= m * a[k * n + j];
        b[i] -= m * b[k];
      }
    }
    for (std::size_t k = n; k-- > 0;) {
      double s = b[k];
      for (std::size_t j = k + 1; j < n; ++j) s -= a[k * n + j] * x.dofs()[j];
      x.dofs()[k] = s / a[k * n + k];
    }
    iterations_ = 1;
  }

 private:
  const DenseLinearOperator* op_ = nullptr;
  mutable SolverParameterType param_;
  mutable int iterations_ = 0;
  mutable std::vector<double> tolerances_;
};

typedef DifferentiableDGEllipticOperator<DenseLinearOperator, ReactionDiffusionModel> SOp;
// NewtonInverseOperator keeps its linear inverse operator protected; this
// derived class only reads the tolerances it recorded.
class Newton : public Dune::Fem::NewtonInverseOperator<DenseLinearOperator, DenseLUInverse> {
 public:
  using Dune::Fem::NewtonInverseOperator<DenseLinearOperator, DenseLUInverse>::NewtonInverseOperator;
  const std::vector<double>& linearTolerances() const { return jInv_.tolerances(); }
};
inline const std::vector<double>& newton_linear_tolerances(const Newton& n) { return n.linearTolerances(); }

struct Case {
  const char* name;
  int cells[3];
  int periodic[3];
  int order;
  bool kappa_field;
  double diffusion, penalty, c1, c3, ce;
  double rhs_scale;     // f[i] = rhs_scale * ((i * 7919 + 13) % 2003 - 1001) / 1000
  double w0_constant;   // initial guess: this constant (the first Legendre mode of every cell)
  const char* line_search;
  const char* forcing;
  double tolerance;
};

void run(const Case& k, bool last) {
  Dune::Fem::CartesianGrid g;
  for (int d = 0; d < 3; ++d) {
    g.N[d] = k.cells[d];
    g.lower[d] = 0.0;
    g.h[d] = 1.0 / k.cells[d];
    g.periodic[d] = k.periodic[d];
  }
  LegendreDGSpace space(g, k.order, k.order);
  const long long nl = (long long)space.localSize();
  DGFunction f(space), w(space), kappa(space);
  for (long long i = 0; i < (long long)space.size(); ++i)
    f.dofs()[i] = k.rhs_scale * (double((i * 7919 + 13) % 2003 - 1001) / 1000.0);
  for (long long c = 0; c < g.ncells(); ++c) {
    kappa.dofs()[c * nl] = 1.0 + double((c * 31 + 7) % 11) / 10.0;
    for (long long l = 1; l < nl; ++l) kappa.dofs()[c * nl + l] = double(((c * nl + l) * 37 + 5) % 9 - 4) / 1000.0;
    w.dofs()[c * nl] = k.w0_constant;
  }
  ReactionDiffusionModel model(k.kappa_field ? &kappa : nullptr, k.diffusion, k.c1, k.c3, k.ce);
  Dune::Fem::ParameterReader params;
  params.set("penalty", k.penalty);
  params.set("fem.solver.nonlinear.linesearch", std::string(k.line_search));
  params.set("fem.solver.nonlinear.forcing", std::string(k.forcing));
  SOp op(space, model, params);

  DGFunction r0(space);
  op(w, r0);
  r0 -= f;
  const double delta0 = std::sqrt(r0.scalarProductDofs(r0));

  Newton newton(k.tolerance, params);
  std::vector<double> residuals;
  const double eps = k.tolerance;
  newton.setErrorMeasure([&residuals, eps](const DGFunction&, const DGFunction&, double res) {
    residuals.push_back(res);
    return res < eps;
  });
  newton.bind(op);
  newton(f, w);

  std::printf("  {\"name\": \"%s\", \"cells\": [%d, %d, %d], \"periodic\": [%d, %d, %d], \"order\": %d, "
              "\"quad_points\": %d, \"kappa_field\": %s, \"diffusion\": %.17g, \"penalty\": %.17g, "
              "\"reaction\": [%.17g, %.17g, %.17g], \"rhs_scale\": %.17g, \"w0_constant\": %.17g, "
              "\"line_search\": \"%s\", \"forcing\": \"%s\", \"tolerance\": %.17g,\n   \"converged\": %s, \"iterations\": %d, "
              "\"linear_iterations\": %d, \"initial_residual\": %.17g, \"residuals\": [",
              k.name, k.cells[0], k.cells[1], k.cells[2], k.periodic[0], k.periodic[1], k.periodic[2], k.order,
              Dune::Fem::gauss_points_for_order(2 * k.order), k.kappa_field ? "true" : "false", k.diffusion,
              k.penalty, k.c1, k.c3, k.ce, k.rhs_scale, k.w0_constant, k.line_search, k.forcing, k.tolerance,
              newton.converged() ? "true" : "false", newton.iterations(), newton.linearIterations(), delta0);
  for (std::size_t i = 0; i < residuals.size(); ++i) std::printf("%s%.17g", i ? ", " : "", residuals[i]);
  std::printf("],\n   \"linear_tolerances\": [");
  const std::vector<double>& tols = newton_linear_tolerances(newton);
  for (std::size_t i = 0; i < tols.size(); ++i) std::printf("%s%.17g", i ? ", " : "", tols[i]);
  std::printf("],\n   \"w\": [");
  for (std::size_t i = 0; i < w.dofs().size(); ++i) std::printf("%s%.17g", i ? ", " : "", w.dofs()[i]);
  std::printf("]}%s\n", last ? "" : ",");
}

}  // namespace refnt

int main() {
  using refnt::Case;
  const Case cases[] = {
      {"cubic_periodic_kappa", {3, 2, 2}, {1, 1, 1}, 2, true, 1.0, 90.0, 0.5, 2.0, 0.0, 10.0, 0.0, "none", "none",
       1e-10},
      {"cubic_periodic_kappa_eisenstat_walker", {3, 2, 2}, {1, 1, 1}, 2, true, 1.0, 90.0, 0.5, 2.0, 0.0, 10.0, 0.0,
       "none", "eisenstatwalker", 1e-10},
      {"exp_periodic", {3, 3, 3}, {1, 1, 1}, 1, false, 1.0, 40.0, 1.0, 0.0, 0.3, 0.5, 0.0, "none", "none", 1e-10},
      {"allen_cahn_plain", {2, 2, 2}, {0, 0, 0}, 1, false, 1e-3, 40.0, -1.0, 1.0, 0.0, 0.0, 0.58, "none", "none",
       1e-10},
      {"allen_cahn_line_search", {2, 2, 2}, {0, 0, 0}, 1, false, 1e-3, 40.0, -1.0, 1.0, 0.0, 0.0, 0.58, "simple",
       "none", 1e-10},
  };
  const int n = int(sizeof(cases) / sizeof(cases[0]));
  std::printf("{\"source\": \"dune-fem NewtonInverseOperator (dune/fem/solver/newtoninverseoperator.hh) over "
              "DifferentiableDGEllipticOperator with a nonlinear source, compiled unmodified against oracle/shim_dg\",\n"
              " \"cases\": [\n");
  for (int i = 0; i < n; ++i) refnt::run(cases[i], i == n - 1);
  std::printf(" ]}\n");
  return 0;
}
