// Runs dune-fem's own stationary-iteration preconditioners --
// FemPreconditioning (jacobi, gauss-seidel, sor, ssor; dune/fem/solver/
// fempreconditioning.hh) over SparseRowMatrix's forward / backward sweeps
// (dune/fem/operator/matrix/spmatrix.hh), both compiled unmodified -- on the
// assembled Jacobian of the reference's DGEllipticOperator (shim grid of
// oracle/shim_dg), and prints z = P r for each as JSON golden vectors.
// Built and run only by oracle/make_ref_golden.sh where the dune-fem sources
// are present; test infrastructure, never the product.
//
// The operator, kappa and probe r come from the same exact formulas as in
// ref_dgelliptic.cpp (r is its u).  The preconditioners are built as
// KrylovInverseOperator builds them (krylovinverseoperators.hh:226-250),
// with n = 3 iterations and relaxation 1.5 requested: FemPreconditioning's
// constructor does not pass them on (fempreconditioning.hh:184-186), so one
// sweep with relaxation 1 is what runs.
#include <config.h>

#include <cstdio>
#include <string>
#include <vector>

#include "dgspace.hh"
#include <dune/fem/schemes/dgelliptic.hh>
#include <dune/fem/operator/matrix/spmatrix.hh>
#include <dune/fem/solver/fempreconditioning.hh>

namespace refpc {

using Dune::Fem::Cell;
using Dune::Fem::ConstLocalFunction;
using Dune::Fem::DenseLinearOperator;
using Dune::Fem::DGFunction;
using Dune::Fem::Face;
using Dune::Fem::LegendreDGSpace;

struct Model {
  typedef LegendreDGSpace::RangeType RangeType;
  typedef LegendreDGSpace::JacobianRangeType JacobianRangeType;
  Model(const DGFunction& kappa, double mass) : mass_(mass), klf_(new ConstLocalFunction<DGFunction>(kappa)) {}
  bool init(const Cell& e) const { klf_->bind(e); return true; }
  template <class Point>
  double coefficient(const Point& x) const {
    RangeType k;
    klf_->evaluate(x, k);
    return k[0];
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
  template <class Point>
  void linSource(const RangeType&, const JacobianRangeType&, const Point&, const RangeType& phi,
                 const JacobianRangeType&, RangeType& s) const {
    s[0] = mass_ * phi[0];
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
  double mass_;
  std::unique_ptr<ConstLocalFunction<DGFunction>> klf_;
};

typedef Dune::Fem::SparseRowMatrix<double> Matrix;

// The assembled operator the preconditioners take: its sparse matrix and its
// diagonal (AssembledOperator: exportMatrix, extractDiagonal, rangeSpace).
class SparseOperator : public Dune::Fem::AssembledOperator<DGFunction> {
 public:
  typedef Matrix MatrixType;
  SparseOperator(const LegendreDGSpace& s, const DenseLinearOperator& J) : space_(s) {
    const std::size_t n = J.size();
    std::size_t nz = 0;
    for (std::size_t i = 0; i < n; ++i) {
      std::size_t c = 0;
      for (std::size_t j = 0; j < n; ++j) c += J(i, j) != 0.0;
      nz = std::max(nz, c);
    }
    m_.reserve(n, n, nz);
    for (std::size_t i = 0; i < n; ++i)
      for (std::size_t j = 0; j < n; ++j)
        if (J(i, j) != 0.0) m_.set(i, j, J(i, j));
  }
  void operator()(const DGFunction&, DGFunction&) const override {}
  const LegendreDGSpace& rangeSpace() const { return space_; }
  const Matrix& exportMatrix() const { return m_; }
  void extractDiagonal(DGFunction& d) const {
    for (std::size_t i = 0; i < d.dofs().size(); ++i) d.dofs()[i] = m_.get(i, i);
  }

 private:
  const LegendreDGSpace& space_;
  Matrix m_;
};

template <class P>
void print_case(const char* name, const P& pc, const DGFunction& r, bool last) {
  DGFunction z(r.space());
  pc(r, z);
  std::printf("  \"%s\": [", name);
  for (std::size_t i = 0; i < z.dofs().size(); ++i) std::printf("%s%.17g", i ? ", " : "", z.dofs()[i]);
  std::printf("]%s\n", last ? "" : ",");
}

}  // namespace refpc

int main() {
  using namespace refpc;
  const int cells[3] = {3, 2, 2}, order = 2;
  const double mass = 0.3, penalty = 90.0;
  Dune::Fem::CartesianGrid g;
  for (int d = 0; d < 3; ++d) {
    g.N[d] = cells[d];
    g.lower[d] = 0.0;
    g.h[d] = 1.0 / cells[d];
    g.periodic[d] = 0;
  }
  LegendreDGSpace space(g, order, order);
  const long long nl = (long long)space.localSize();
  DGFunction r(space), kappa(space);
  for (long long i = 0; i < (long long)space.size(); ++i) r.dofs()[i] = double((i * 7919 + 13) % 2003 - 1001) / 1000.0;
  for (long long c = 0; c < g.ncells(); ++c) {
    kappa.dofs()[c * nl] = 1.0 + double((c * 31 + 7) % 11) / 10.0;
    for (long long l = 1; l < nl; ++l) kappa.dofs()[c * nl + l] = double(((c * nl + l) * 37 + 5) % 9 - 4) / 1000.0;
  }
  Model model(kappa, mass);
  Dune::Fem::ParameterReader params;
  params.set("penalty", penalty);
  DifferentiableDGEllipticOperator<DenseLinearOperator, Model> op(space, model, params);
  DenseLinearOperator J(space);
  op.jacobian(r, J);
  SparseOperator A(space, J);

  const int n = 3;
  const double w = 1.5;
  Dune::Fem::FemJacobiPreconditioning<DGFunction, SparseOperator> jacobi(A, n, w);
  Dune::Fem::FemGaussSeidelPreconditioning<DGFunction, SparseOperator> gs(A, n, w);
  Dune::Fem::FemSORPreconditioning<DGFunction, SparseOperator> sor(A, n, w);
  Dune::Fem::FemSSORPreconditioning<DGFunction, SparseOperator> ssor(A, n, w);
  std::printf("{\"source\": \"dune-fem FemPreconditioning over SparseRowMatrix::forwardIterative/backwardIterative "
              "(fempreconditioning.hh, spmatrix.hh), compiled unmodified, on the assembled DGEllipticOperator "
              "Jacobian\",\n \"cells\": [%d, %d, %d], \"order\": %d, \"quad_points\": %d, \"mass\": %.17g, "
              "\"penalty\": %.17g, \"requested_iterations\": %d, \"requested_relaxation\": %.17g,\n",
              cells[0], cells[1], cells[2], order, Dune::Fem::gauss_points_for_order(2 * order), mass, penalty, n, w);
  print_case("jacobi", jacobi, r, false);
  print_case("gauss-seidel", gs, r, false);
  print_case("sor", sor, r, false);
  print_case("ssor", ssor, r, true);
  std::printf("}\n");
  return 0;
}
