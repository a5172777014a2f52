// Runs dune-fem's own explicit time loop -- TimeProvider (dune/fem/solver/
// timeprovider.hh), ExplicitRungeKuttaSolver (solver/rungekutta/explicit.hh)
// with tvd3ButcherTable (butchertable.{hh,cc}), all compiled unmodified --
// over the method-of-lines operator L(u) = -M^{-1} A u, where A is the
// reference's DGEllipticOperator (dgelliptic.hh) on the shim grid of
// oracle/shim_dg and M = |K| I the mass matrix of the orthonormal Legendre
// basis on affine cells (the block that operator/1order/localmassmatrix.hh
// inverts); prints the step sizes, times and final state as JSON golden
// vectors.  Built and run only by oracle/make_ref_golden.sh where the
// dune-fem sources are present; test infrastructure, never the product.
//
// The operator's time-step estimate is a function of how often it has been
// applied, so that the minimum the TimeProvider takes over the estimates of
// one step's stages is exercised:
//   estimate(k) = 1e-3 * (3 + (7 k + 2) mod 13) / 8   after the k-th application
// (the minimum falls on different stages in different steps).
// The initial state and kappa come from the same exact integer formulas as
// in ref_dgelliptic.cpp.
#include <config.h>

#include <cstdio>
#include <vector>

#include "dgspace.hh"
#include <dune/fem/schemes/dgelliptic.hh>
#include <dune/fem/solver/timeprovider.hh>
#include <dune/fem/solver/rungekutta/explicit.hh>

namespace reftl {

using Dune::Fem::Cell;
using Dune::Fem::ConstLocalFunction;
using Dune::Fem::DGFunction;
using Dune::Fem::Face;
using Dune::Fem::LegendreDGSpace;

struct DiffusionMassModel {
  typedef LegendreDGSpace::RangeType RangeType;
  typedef LegendreDGSpace::JacobianRangeType JacobianRangeType;
  DiffusionMassModel(const DGFunction& kappa, double diffusion, double mass)
      : diffusion_(diffusion), mass_(mass), klf_(new ConstLocalFunction<DGFunction>(kappa)) {}
  bool init(const Cell& e) const { klf_->bind(e); return true; }
  template <class Point>
  double coefficient(const Point& x) const {
    RangeType k;
    klf_->evaluate(x, k);
    return diffusion_ * k[0];
  }
  template <class Point>
  void source(const Point&, const RangeType& u, const JacobianRangeType&, RangeType& s) const { s[0] = mass_ * u[0]; }
  template <class Point>
  void flux(const Point& x, const RangeType&, const JacobianRangeType& du, JacobianRangeType& f) const {
    const double k = coefficient(x);
    for (int d = 0; d < 3; ++d) f[0][d] = k * du[0][d];
  }
  template <class Point>
  RangeType penalty(const Point& x, const RangeType&) const { return RangeType(coefficient(x)); }
  void isDirichletIntersection(const Face&, std::array<int, 1>& components) const { components[0] = 0; }
  template <class Point>
  void dirichlet(int, const Point&, RangeType& g) const { g = RangeType(0.0); }

 private:
  double diffusion_, mass_;
  std::unique_ptr<ConstLocalFunction<DGFunction>> klf_;
};

typedef DGEllipticOperator<DGFunction, DiffusionMassModel> EllipticOp;

class MolOperator : public Dune::Fem::SpaceOperatorInterface<DGFunction> {
 public:
  MolOperator(const EllipticOp& a, const LegendreDGSpace& s) : a_(a), space_(s) {}
  void operator()(const DGFunction& u, DGFunction& w) const override {
    a_(u, w);
    const double s = -1.0 / space_.grid().volume();
    for (double& x : w.dofs()) x *= s;
    ++applications_;
  }
  const LegendreDGSpace& space() const override { return space_; }
  double timeStepEstimate() const override { return 1e-3 * (3 + (7 * applications_ + 2) % 13) / 8.0; }
  long applications() const { return applications_; }

 private:
  const EllipticOp& a_;
  const LegendreDGSpace& space_;
  mutable long applications_ = 0;
};

}  // namespace reftl

int main() {
  using namespace reftl;
  const int cells[3] = {3, 2, 2}, order = 2, steps = 5;
  const double upper[3] = {1.0, 1.0, 1.0}, diffusion = 0.05, mass = 0.5, penalty = 90.0, cfl = 0.9;
  Dune::Fem::CartesianGrid g;
  for (int d = 0; d < 3; ++d) {
    g.N[d] = cells[d];
    g.lower[d] = 0.0;
    g.h[d] = upper[d] / cells[d];
    g.periodic[d] = 1;
  }
  LegendreDGSpace space(g, order, order);
  const long long nl = (long long)space.localSize();
  DGFunction u(space), kappa(space);
  for (long long i = 0; i < (long long)space.size(); ++i) u.dofs()[i] = double((i * 7919 + 13) % 2003 - 1001) / 1000.0;
  for (long long c = 0; c < g.ncells(); ++c) {
    kappa.dofs()[c * nl] = 1.0 + double((c * 31 + 7) % 11) / 10.0;
    for (long long l = 1; l < nl; ++l) kappa.dofs()[c * nl + l] = double(((c * nl + l) * 37 + 5) % 9 - 4) / 1000.0;
  }
  DiffusionMassModel model(kappa, diffusion, mass);
  Dune::Fem::ParameterReader params;
  params.set("penalty", penalty);
  EllipticOp a(space, model, params);
  MolOperator L(a, space);

  Dune::Fem::TimeProvider<> tp(0.0, cfl);
  DuneODE::ExplicitRungeKuttaSolver<DGFunction> ode(L, tp, DuneODE::tvd3ButcherTable(), false);
  ode.initialize(u);
  std::vector<double> dts, times;
  for (tp.init(); tp.timeStep() < steps; tp.next()) {
    times.push_back(tp.time());
    dts.push_back(tp.deltaT());
    ode.solve(u);
  }

  const DuneODE::SimpleButcherTable<double> bt = DuneODE::tvd3ButcherTable();
  const auto A = bt.A();
  const auto b = bt.b();
  const auto c = bt.c();
  std::printf("{\"source\": \"dune-fem TimeProvider + ExplicitRungeKuttaSolver(tvd3ButcherTable) over "
              "-M^{-1} DGEllipticOperator, compiled unmodified against oracle/shim_dg\",\n");
  std::printf(" \"tvd3\": {\"A\": [");
  for (int i = 0; i < bt.stages(); ++i) {
    std::printf("%s[", i ? ", " : "");
    for (int j = 0; j < bt.stages(); ++j) std::printf("%s%.17g", j ? ", " : "", A[i][j]);
    std::printf("]");
  }
  std::printf("], \"b\": [%.17g, %.17g, %.17g], \"c\": [%.17g, %.17g, %.17g], \"order\": %d},\n", b[0], b[1], b[2], c[0],
              c[1], c[2], bt.order());
  std::printf(" \"cells\": [%d, %d, %d], \"order\": %d, \"quad_points\": %d, \"periodic\": [1, 1, 1], "
              "\"diffusion\": %.17g, \"mass\": %.17g, \"penalty\": %.17g, \"cfl\": %.17g, \"steps\": %d, "
              "\"applications\": %ld,\n",
              cells[0], cells[1], cells[2], order, Dune::Fem::gauss_points_for_order(2 * order), diffusion, mass,
              penalty, cfl, steps, L.applications());
  std::printf(" \"dt\": [");
  for (std::size_t i = 0; i < dts.size(); ++i) std::printf("%s%.17g", i ? ", " : "", dts[i]);
  std::printf("],\n \"time\": [");
  for (std::size_t i = 0; i < times.size(); ++i) std::printf("%s%.17g", i ? ", " : "", times[i]);
  std::printf("],\n \"final_time\": %.17g,\n \"u\": [", tp.time());
  for (std::size_t i = 0; i < u.dofs().size(); ++i) std::printf("%s%.17g", i ? ", " : "", u.dofs()[i]);
  std::printf("]}\n");
  return 0;
}
