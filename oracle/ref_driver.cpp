// Driver that runs the reference's own compiled code for the pieces of this
// path that build standalone, and prints their outputs as JSON golden
// vectors.  Built and run only by oracle/make_ref_golden.sh, in a checkout
// that has the dune-fem sources; the product never uses it.
//
// Compiled unmodified from the reference tree:
//   dune/fem/quadrature/gausspoints.hh (+ _implementation.hh)  -> Gauss rules
//   dune/fem/space/shapefunctionset/legendrepolynomials.{hh,cc} -> Legendre tables
//   dune/fem/solver/linear/{cg,gmres,bicgstab}.hh               -> Krylov iterates
// against the minimal shims in oracle/shim (visibility macros, FieldTraits,
// ToleranceCriteria).  The vector type below provides the discrete-function
// subset those templates call.
#include <cmath>
#include <complex>  // cg.hh calls std::real without including it
#include <cstdio>
#include <functional>
#include <string>
#include <vector>

#include <dune/fem/quadrature/gausspoints.hh>
#include <dune/fem/space/shapefunctionset/legendrepolynomials.hh>
#include <dune/fem/solver/linear/cg.hh>
#include <dune/fem/solver/linear/gmres.hh>
#include <dune/fem/solver/linear/bicgstab.hh>

namespace refdrv {

struct Comm {
  template <class T>
  void sum(T*, int) const {}
  template <class T>
  T sum(T x) const { return x; }
};
struct GridPart {
  Comm c;
  const Comm& comm() const { return c; }
};
// The auxiliary-dof list of a serial run: one sentinel entry equal to the
// number of dofs (space/common/auxiliarydofs.hh).
struct AuxDofs {
  size_t n;
  size_t size() const { return 1; }
  size_t operator[](size_t) const { return n; }
};
template <class F>
void forEachPrimaryDof(const AuxDofs& a, F&& f) {
  for (size_t i = 0; i < a.n; ++i) f(i);
}
struct SpaceT {
  GridPart gp;
  AuxDofs aux;
  const GridPart& gridPart() const { return gp; }
  const AuxDofs& auxiliaryDofs() const { return aux; }
};

struct Vec {
  typedef double RangeFieldType;
  typedef double DofType;
  const SpaceT* sp;
  std::vector<double> d;
  Vec(const SpaceT& s, size_t n) : sp(&s), d(n, 0.0) {}
  const SpaceT& space() const { return *sp; }
  std::vector<double>& dofVector() { return d; }
  const std::vector<double>& dofVector() const { return d; }
  void assign(const Vec& o) { d = o.d; }
  void clear() { std::fill(d.begin(), d.end(), 0.0); }
  Vec& operator-=(const Vec& o) { for (size_t i = 0; i < d.size(); ++i) d[i] -= o.d[i]; return *this; }
  Vec& operator+=(const Vec& o) { for (size_t i = 0; i < d.size(); ++i) d[i] += o.d[i]; return *this; }
  Vec& operator*=(double a) { for (auto& x : d) x *= a; return *this; }
  void axpy(double a, const Vec& o) { for (size_t i = 0; i < d.size(); ++i) d[i] += a * o.d[i]; }
  double scalarProductDofs(const Vec& o) const {
    double s = 0;
    for (size_t i = 0; i < d.size(); ++i) s += d[i] * o.d[i];
    return s;
  }
  double normSquaredDofs() const { return scalarProductDofs(*this); }
};

struct Op {
  std::function<void(const std::vector<double>&, std::vector<double>&)> f;
  void operator()(const Vec& x, Vec& y) const { f(x.d, y.d); }
};

// tridiagonal test matrices
void tri(const std::vector<double>& x, std::vector<double>& y, double lo, double up, double diag0, double dslope) {
  const size_t n = x.size();
  for (size_t i = 0; i < n; ++i) {
    double di = diag0 + dslope * double(i) / double(n);
    double s = di * x[i];
    if (i > 0) s += lo * x[i - 1];
    if (i + 1 < n) s += up * x[i + 1];
    y[i] = s;
  }
}

void print_vec(const char* name, const std::vector<double>& v, bool last = false) {
  std::printf("  \"%s\": [", name);
  for (size_t i = 0; i < v.size(); ++i) std::printf("%s%.17g", i ? ", " : "", v[i]);
  std::printf("]%s\n", last ? "" : ",");
}

}  // namespace refdrv

int main(int argc, char** argv) {
  using namespace refdrv;
  const std::string what = argc > 1 ? argv[1] : "tables";
  if (what == "tables") {
    Dune::Fem::GaussPts gp;
    std::printf("{\n  \"gauss\": {\n");
    for (int m = 1; m <= Dune::Fem::GaussPts::MAXP; ++m) {
      std::printf("    \"%d\": {\"order\": %d, \"points\": [", m, gp.order(m));
      for (int i = 0; i < m; ++i) std::printf("%s%.17g", i ? ", " : "", gp.point(m, i));
      std::printf("], \"weights\": [");
      for (int i = 0; i < m; ++i) std::printf("%s%.17g", i ? ", " : "", gp.weight(m, i));
      std::printf("]}%s\n", m < Dune::Fem::GaussPts::MAXP ? "," : "");
    }
    std::printf("  },\n  \"legendre\": {\n    \"x\": [");
    const double xs[] = {0.0, 0.0694318442029737, 0.25, 0.5, 0.7886751345948129, 0.93, 1.0};
    const int nx = sizeof(xs) / sizeof(xs[0]);
    for (int i = 0; i < nx; ++i) std::printf("%s%.17g", i ? ", " : "", xs[i]);
    std::printf("],\n    \"value\": [");
    for (int k = 0; k < Dune::Fem::LegendrePolynomials::maxOrder; ++k) {
      std::printf("%s[", k ? ", " : "");
      for (int i = 0; i < nx; ++i) std::printf("%s%.17g", i ? ", " : "", Dune::Fem::LegendrePolynomials::evaluate(k, xs[i]));
      std::printf("]");
    }
    std::printf("],\n    \"jacobian\": [");
    for (int k = 0; k < Dune::Fem::LegendrePolynomials::maxOrder; ++k) {
      std::printf("%s[", k ? ", " : "");
      for (int i = 0; i < nx; ++i) std::printf("%s%.17g", i ? ", " : "", Dune::Fem::LegendrePolynomials::jacobian(k, xs[i]));
      std::printf("]");
    }
    std::printf("]\n  }\n}\n");
    return 0;
  }
  // Krylov golden vectors
  const size_t n = 60;
  SpaceT sp;
  sp.aux.n = n;
  Vec b(sp, n);
  for (size_t i = 0; i < n; ++i) b.d[i] = std::sin(0.3 * double(i) + 0.1);
  Op spd{[](const std::vector<double>& x, std::vector<double>& y) { tri(x, y, -1.0, -1.0, 2.05, 0.5); }};
  Op nonsym{[](const std::vector<double>& x, std::vector<double>& y) { tri(x, y, -1.3, -0.7, 2.5, 0.3); }};
  // diagonal (Jacobi) preconditioner of the SPD matrix
  Op jac{[](const std::vector<double>& x, std::vector<double>& y) {
    for (size_t i = 0; i < x.size(); ++i) y[i] = x[i] / (2.05 + 0.5 * double(i) / double(x.size()));
  }};
  Op jacn{[](const std::vector<double>& x, std::vector<double>& y) {
    for (size_t i = 0; i < x.size(); ++i) y[i] = x[i] / (2.5 + 0.3 * double(i) / double(x.size()));
  }};
  const int rel = Dune::Fem::LinearSolver::ToleranceCriteria::relative;
  std::printf("{\n  \"n\": %zu,\n", n);
  print_vec("b", b.d);
  {
    std::vector<Vec> tmp(3, Vec(sp, n));
    Vec x(sp, n);
    int it = Dune::Fem::LinearSolver::cg(spd, (Op*)nullptr, tmp, x, b, 1e-10, 1000, rel);
    std::printf("  \"cg_iterations\": %d,\n", it);
    print_vec("cg_x", x.d);
  }
  {
    std::vector<Vec> tmp(5, Vec(sp, n));
    Vec x(sp, n);
    int it = Dune::Fem::LinearSolver::cg(spd, &jac, tmp, x, b, 1e-10, 1000, rel);
    std::printf("  \"pcg_iterations\": %d,\n", it);
    print_vec("pcg_x", x.d);
  }
  {
    const int m = 10;
    std::vector<Vec> v(m + 1, Vec(sp, n));
    Vec x(sp, n);
    int it = Dune::Fem::LinearSolver::gmres(nonsym, (Op*)nullptr, v, x, b, m, 1e-10, 1000, rel);
    std::printf("  \"gmres_restart\": %d,\n  \"gmres_iterations\": %d,\n", m, it);
    print_vec("gmres_x", x.d);
  }
  {
    const int m = 10;
    std::vector<Vec> v(m + 2, Vec(sp, n));
    Vec x(sp, n);
    int it = Dune::Fem::LinearSolver::gmres(nonsym, &jacn, v, x, b, m, 1e-10, 1000, rel);
    std::printf("  \"pgmres_iterations\": %d,\n", it);
    print_vec("pgmres_x", x.d);
  }
  {
    std::vector<Vec> v(5, Vec(sp, n));
    Vec x(sp, n);
    int it = Dune::Fem::LinearSolver::bicgstab(nonsym, (Op*)nullptr, v, x, b, 1e-10, 1000, rel);
    std::printf("  \"bicgstab_iterations\": %d,\n", it);
    print_vec("bicgstab_x", x.d, true);
  }
  std::printf("}\n");
  return 0;
}
