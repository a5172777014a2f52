// Runs dune-fem's own DG elliptic operator -- DGEllipticOperator::apply and
// DefaultPenalty from dune/fem/schemes/dgelliptic.hh, over the reference's
// LegendreShapeFunctionSet (legendre.hh), LegendrePolynomials
// (legendrepolynomials.{hh,cc}) and GaussPts (gausspoints.hh), all compiled
// unmodified -- on small Cartesian grids provided by the shim layer in
// oracle/shim_dg, and prints the results as JSON golden vectors.  With the
// argument "jacobian" it assembles the operator's Jacobian instead
// (DifferentiableDGEllipticOperator::jacobian, dgelliptic.hh:456-766) and
// prints it through products, its diagonal, some diagonal blocks and the
// norms of all its nonzero cell blocks.  With "hierarchical" it prints the
// order of the hierarchically sorted LegendreShapeFunctionSet (legendre.hh:
// 236-249) as indices into the default (non-hierarchical) set, for 1-3
// dimensions and orders 0-4.  Built and run only by
// oracle/make_ref_golden.sh where the dune-fem sources are present; test
// infrastructure, never part of the product.
//
// The model below is the SIPG diffusion + mass problem of this path:
//   source(u)   = mass * u,
//   flux(du)    = diffusion * kappa(x) * du,
//   penalty     = diffusion * kappa(x)   (averaged over the two sides by the
//                                         operator, dgelliptic.hh:364-368),
// with kappa an optional Q_p field in the same Legendre basis.  Boundary
// faces are either do-nothing (no Dirichlet components, dgelliptic.hh:
// 438-443) or weak homogeneous Dirichlet (g = 0, dgelliptic.hh:393-446), or
// absent on fully periodic grids.
//
// Inputs are generated by integer formulas whose conversion to double is
// exact, so a test can rebuild them bit for bit:
//   u[i]             = ((i * 7919 + 13) % 2003 - 1001) / 1000
//   kappa[c*nl + 0]  = 1 + ((c * 31 + 7) % 11) / 10
//   kappa[c*nl + l]  = (((c*nl + l) * 37 + 5) % 9 - 4) / 1000   (l > 0)
#include <config.h>

#include <array>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <string>
#include <vector>

#include "dgspace.hh"
#include <dune/fem/schemes/dgelliptic.hh>

namespace refdg {

using Dune::Fem::Cell;
using Dune::Fem::ConstLocalFunction;
using Dune::Fem::DGFunction;
using Dune::Fem::Face;
using Dune::Fem::LegendreDGSpace;

struct SipgMassModel {
  typedef LegendreDGSpace::RangeType RangeType;
  typedef LegendreDGSpace::JacobianRangeType JacobianRangeType;

  SipgMassModel(const DGFunction* kappa, double diffusion, double mass, bool dirichlet)
      : diffusion_(diffusion), mass_(mass), dirichlet_(dirichlet), kappa_(kappa) {
    if (kappa_) klf_.reset(new ConstLocalFunction<DGFunction>(*kappa_));
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
    s[0] = mass_ * u[0];
  }
  template <class Point>
  void flux(const Point& x, const RangeType&, const JacobianRangeType& du, JacobianRangeType& f) const {
    const double k = coefficient(x);
    for (int d = 0; d < 3; ++d) f[0][d] = k * du[0][d];
  }
  template <class Point>
  RangeType penalty(const Point& x, const RangeType&) const {
    return RangeType(coefficient(x));
  }
  // linearisation (the model is linear: the same maps applied to phi, dphi)
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
  void isDirichletIntersection(const Face&, std::array<int, 1>& components) const { components[0] = dirichlet_ ? 1 : 0; }
  template <class Point>
  void dirichlet(int, const Point&, RangeType& g) const { g = RangeType(0.0); }

 private:
  double diffusion_, mass_;
  bool dirichlet_;
  const DGFunction* kappa_;
  std::unique_ptr<ConstLocalFunction<DGFunction>> klf_;
};

struct Case {
  const char* name;
  int cells[3];
  double upper[3];
  int periodic[3];
  int order;
  int reported_order;  // quadrature from order() of u plus order() of w
  bool kappa_field;
  bool dirichlet;
  double diffusion, mass, penalty;
};

Dune::Fem::CartesianGrid make_grid(const Case& k) {
  Dune::Fem::CartesianGrid g;
  for (int d = 0; d < 3; ++d) {
    g.N[d] = k.cells[d];
    g.lower[d] = 0.0;
    g.h[d] = k.upper[d] / k.cells[d];
    g.periodic[d] = k.periodic[d];
  }
  return g;
}

void fill_inputs(const LegendreDGSpace& space, DGFunction& u, DGFunction& kappa) {
  const long long nl = (long long)space.localSize();
  for (long long i = 0; i < (long long)space.size(); ++i) u.dofs()[i] = double((i * 7919 + 13) % 2003 - 1001) / 1000.0;
  for (long long c = 0; c < space.grid().ncells(); ++c) {
    kappa.dofs()[c * nl] = 1.0 + double((c * 31 + 7) % 11) / 10.0;
    for (long long l = 1; l < nl; ++l) kappa.dofs()[c * nl + l] = double(((c * nl + l) * 37 + 5) % 9 - 4) / 1000.0;
  }
}

void print_header(const Case& k, int quad_points) {
  std::printf("  {\"name\": \"%s\", \"cells\": [%d, %d, %d], \"upper\": [%.17g, %.17g, %.17g], "
              "\"periodic\": [%d, %d, %d], \"order\": %d, \"quad_points\": %d, \"kappa_field\": %s, \"dirichlet\": %s, "
              "\"diffusion\": %.17g, \"mass\": %.17g, \"penalty\": %.17g",
              k.name, k.cells[0], k.cells[1], k.cells[2], k.upper[0], k.upper[1], k.upper[2], k.periodic[0],
              k.periodic[1], k.periodic[2], k.order, quad_points, k.kappa_field ? "true" : "false",
              k.dirichlet ? "true" : "false", k.diffusion, k.mass, k.penalty);
}

void print_vector(const char* key, const std::vector<double>& v) {
  std::printf(",\n   \"%s\": [", key);
  for (std::size_t i = 0; i < v.size(); ++i) std::printf("%s%.17g", i ? ", " : "", v[i]);
  std::printf("]");
}

void run_case(const Case& k, bool last) {
  const Dune::Fem::CartesianGrid g = make_grid(k);
  LegendreDGSpace space(g, k.order, k.reported_order);
  DGFunction u(space), w(space), kappa(space);
  fill_inputs(space, u, kappa);
  SipgMassModel model(k.kappa_field ? &kappa : nullptr, k.diffusion, k.mass, k.dirichlet);
  Dune::Fem::ParameterReader params;
  params.set("penalty", k.penalty);
  DGEllipticOperator<DGFunction, SipgMassModel> op(space, model, params);
  op(u, w);

  print_header(k, Dune::Fem::gauss_points_for_order(2 * k.reported_order));
  print_vector("w", w.dofs());
  std::printf("}%s\n", last ? "" : ",");
}

// The assembled Jacobian of a case (its quadrature follows the space's true
// order: q = p+1).  Printed: J v for
// v[i] = ((i * 4243 + 7) % 1999 - 999) / 1000 (J u is the apply above); the
// diagonal; the dense
// diagonal blocks of the listed cells (row-major, rows = test functions);
// and, for every pair of cells with a nonzero block, [row cell, column cell,
// Frobenius norm].
void run_jacobian(const Case& k, const std::vector<long long>& block_cells, bool last) {
  const Dune::Fem::CartesianGrid g = make_grid(k);
  LegendreDGSpace space(g, k.order, k.order);
  DGFunction u(space), kappa(space);
  fill_inputs(space, u, kappa);
  SipgMassModel model(k.kappa_field ? &kappa : nullptr, k.diffusion, k.mass, k.dirichlet);
  Dune::Fem::ParameterReader params;
  params.set("penalty", k.penalty);
  DifferentiableDGEllipticOperator<Dune::Fem::DenseLinearOperator, SipgMassModel> op(space, model, params);
  Dune::Fem::DenseLinearOperator J(space);
  op.jacobian(u, J);

  const std::size_t n = space.size(), nl = space.localSize();
  std::vector<double> v(n), Jv(n, 0.0), diag(n), blocks;
  for (std::size_t i = 0; i < n; ++i) v[i] = double(((long long)i * 4243 + 7) % 1999 - 999) / 1000.0;
  for (std::size_t i = 0; i < n; ++i) {
    for (std::size_t j = 0; j < n; ++j) Jv[i] += J(i, j) * v[j];
    diag[i] = J(i, i);
  }
  for (long long c : block_cells)
    for (std::size_t i = 0; i < nl; ++i)
      for (std::size_t j = 0; j < nl; ++j) blocks.push_back(J(c * nl + i, c * nl + j));
  print_header(k, Dune::Fem::gauss_points_for_order(2 * k.order));
  print_vector("Jv", Jv);
  print_vector("diag", diag);
  std::printf(",\n   \"block_cells\": [");
  for (std::size_t i = 0; i < block_cells.size(); ++i) std::printf("%s%lld", i ? ", " : "", block_cells[i]);
  std::printf("]");
  print_vector("blocks", blocks);
  std::printf(",\n   \"block_norms\": [");
  bool first = true;
  for (long long r = 0; r < g.ncells(); ++r)
    for (long long c = 0; c < g.ncells(); ++c) {
      double s = 0.0;
      for (std::size_t i = 0; i < nl; ++i)
        for (std::size_t j = 0; j < nl; ++j) s += J(r * nl + i, c * nl + j) * J(r * nl + i, c * nl + j);
      if (s == 0.0) continue;
      std::printf("%s[%lld, %lld, %.17g]", first ? "" : ", ", r, c, std::sqrt(s));
      first = false;
    }
  std::printf("]}%s\n", last ? "" : ",");
}

// perm[h] = index in the non-hierarchical set of the h-th function of the
// hierarchical set, found by matching values at a generic point (the values
// of the (p+1)^dim functions there are distinct; checked).
template <int dim>
std::vector<int> hierarchical_order(int order) {
  typedef Dune::Fem::ScalarFunctionSpace<dim> FS;
  Dune::Fem::LegendreShapeFunctionSet<FS, false> plain(order);
  Dune::Fem::LegendreShapeFunctionSet<FS, true> hier(order);
  typename FS::DomainType x;
  const double at[3] = {0.2137, 0.6183, 0.4471};
  for (int d = 0; d < dim; ++d) x[d] = at[d];
  std::vector<double> vp(plain.size()), vh(hier.size());
  plain.evaluateEach(x, [&](std::size_t i, const typename FS::RangeType& v) { vp[i] = v[0]; });
  hier.evaluateEach(x, [&](std::size_t i, const typename FS::RangeType& v) { vh[i] = v[0]; });
  std::vector<int> perm;
  for (double v : vh) {
    int found = -1, count = 0;
    for (std::size_t i = 0; i < vp.size(); ++i)
      if (vp[i] == v) { found = int(i); ++count; }
    if (count != 1) { std::fprintf(stderr, "hierarchical_order: ambiguous value\n"); std::exit(1); }
    perm.push_back(found);
  }
  return perm;
}

template <int dim>
void print_orders(bool last) {
  for (int p = 0; p <= 4; ++p) {
    const std::vector<int> perm = hierarchical_order<dim>(p);
    std::printf("  {\"dim\": %d, \"order\": %d, \"perm\": [", dim, p);
    for (std::size_t i = 0; i < perm.size(); ++i) std::printf("%s%d", i ? ", " : "", perm[i]);
    std::printf("]}%s\n", last && p == 4 ? "" : ",");
  }
}

}  // namespace refdg

int main(int argc, char** argv) {
  using refdg::Case;
  if (argc > 1 && std::string(argv[1]) == "hierarchical") {
    std::printf("{\"source\": \"dune-fem LegendreShapeFunctionSet<FS, true> (legendre.hh) against the default "
                "ordering, compiled unmodified\",\n \"orders\": [\n");
    refdg::print_orders<1>(false);
    refdg::print_orders<2>(false);
    refdg::print_orders<3>(true);
    std::printf(" ]}\n");
    return 0;
  }
  if (argc > 1 && std::string(argv[1]) == "jacobian") {
    const Case cases[] = {
        {"q1_periodic_aniso_kappa_mass", {3, 2, 2}, {1.5, 1.0, 0.5}, {1, 1, 1}, 1, 1, true, false, 1.0, 0.7, 40.0},
        {"q2_open_z_kappa", {3, 2, 2}, {1.0, 1.0, 1.0}, {1, 1, 0}, 2, 2, true, false, 1.0, 0.0, 90.0},
        {"q2_dirichlet_kappa", {3, 2, 2}, {1.0, 1.0, 1.0}, {0, 0, 0}, 2, 2, true, true, 1.0, 0.0, 90.0},
        {"q3_periodic_const_mass", {2, 2, 2}, {1.0, 0.75, 1.25}, {1, 1, 1}, 3, 3, false, false, 0.5, 1.3, 160.0},
    };
    const std::vector<long long> block_cells[] = {{0, 5, 11}, {7}, {4}, {}};
    std::printf("{\"source\": \"dune-fem DifferentiableDGEllipticOperator::jacobian (dune/fem/schemes/dgelliptic.hh) "
                "over LegendreShapeFunctionSet and GaussPts, compiled unmodified against oracle/shim_dg\",\n"
                " \"cases\": [\n");
    for (int i = 0; i < 4; ++i) refdg::run_jacobian(cases[i], block_cells[i], i == 3);
    std::printf(" ]}\n");
    return 0;
  }
  const Case cases[] = {
      {"q1_periodic_aniso_kappa_mass", {3, 2, 2}, {1.5, 1.0, 0.5}, {1, 1, 1}, 1, 1, true, false, 1.0, 0.7, 40.0},
      {"q2_periodic_kappa_qp2", {2, 3, 2}, {1.0, 1.0, 1.0}, {1, 1, 1}, 2, 3, true, false, 1.0, 0.0, 90.0},
      {"q3_periodic_const_mass", {2, 2, 2}, {1.0, 0.75, 1.25}, {1, 1, 1}, 3, 3, false, false, 0.5, 1.3, 160.0},
      {"q2_open_z_kappa", {3, 2, 2}, {1.0, 1.0, 1.0}, {1, 1, 0}, 2, 2, true, false, 1.0, 0.0, 90.0},
      {"q4_periodic_kappa_qp2", {2, 2, 2}, {1.0, 1.0, 1.0}, {1, 1, 1}, 4, 5, true, false, 1.0, 0.2, 250.0},
      {"q3_open_const_qp2", {2, 2, 2}, {1.0, 1.0, 1.0}, {0, 0, 0}, 3, 4, false, false, 1.0, 0.0, 160.0},
      {"q2_dirichlet_kappa", {3, 2, 2}, {1.0, 1.0, 1.0}, {0, 0, 0}, 2, 2, true, true, 1.0, 0.0, 90.0},
      {"q3_dirichlet_aniso_qp2", {2, 2, 2}, {1.0, 0.5, 2.0}, {0, 1, 0}, 3, 4, false, true, 0.8, 0.4, 160.0},
  };
  const int n = int(sizeof(cases) / sizeof(cases[0]));
  std::printf("{\"source\": \"dune-fem DGEllipticOperator (dune/fem/schemes/dgelliptic.hh) over LegendreShapeFunctionSet "
              "and GaussPts, compiled unmodified against oracle/shim_dg\",\n \"cases\": [\n");
  for (int i = 0; i < n; ++i) refdg::run_case(cases[i], i == n - 1);
  std::printf(" ]}\n");
  return 0;
}
