// Driver that runs the reference's own compiled code for the pieces of this
// path that build standalone, and prints their outputs as JSON golden
// vectors.  Built and run only by oracle/make_ref_golden.sh, in a checkout
// that has the dune-fem sources; the product never uses it.
//
// Compiled unmodified from the reference tree:
//   dune/fem/quadrature/gausspoints.hh (+ _implementation.hh)  -> Gauss rules
//   dune/fem/space/shapefunctionset/legendrepolynomials.{hh,cc} -> Legendre tables
//   dune/fem/solver/linear/{cg,gmres,bicgstab}.hh               -> Krylov iterates
// The "sipg" mode runs those Krylov templates over the oracle's DG SIPG
// operator (oracle.cpp, linked in) on an 8^3 Q2 grid.
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

// The oracle's DG operator (oracle.cpp, linked in): the SIPG systems on which
// the reference's Krylov templates run in the "sipg" mode below.
extern "C" int oracle_dg_apply(const int* cells, const double* lower, const double* upper, const int* periodic,
                               int order, int quad, double diffusion, double penalty, double mass,
                               const double* velocity, int weak_dirichlet, const double* kappa, const double* u,
                               double* w, int nthreads);
extern "C" int oracle_dg_block_diagonal(const int* cells, const double* lower, const double* upper,
                                        const int* periodic, int order, int quad, double diffusion, double penalty,
                                        double mass, const double* velocity, int weak_dirichlet, const double* kappa,
                                        double* blocks, int nthreads);

namespace refdrv {

// 8^3 DG Q2 on the unit cube, q = p + 2, penalty 10 (p+1)^2, weak u = 0.
struct SipgCase {
  int cells[3] = {8, 8, 8};
  double lower[3] = {0, 0, 0}, upper[3] = {1, 1, 1};
  int periodic[3] = {0, 0, 0};
  int order = 2, quad = 4;
  double diffusion = 1.0, penalty = 90.0, mass = 0.0;
  double velocity[3] = {0, 0, 0};
  size_t ndofs() const { return size_t(cells[0]) * cells[1] * cells[2] * 27; }
  void apply(const std::vector<double>& x, std::vector<double>& y) const {
    oracle_dg_apply(cells, lower, upper, periodic, order, quad, diffusion, penalty, mass, velocity, 1, nullptr,
                    x.data(), y.data(), 1);
  }
  std::vector<double> diagonal() const {
    const size_t nc = size_t(cells[0]) * cells[1] * cells[2];
    std::vector<double> blocks(nc * 27 * 27), d(nc * 27);
    oracle_dg_block_diagonal(cells, lower, upper, periodic, order, quad, diffusion, penalty, mass, velocity, 1,
                             nullptr, blocks.data(), 1);
    for (size_t c = 0; c < nc; ++c)
      for (int i = 0; i < 27; ++i) d[c * 27 + i] = blocks[(c * 27 + i) * 27 + i];
    return d;
  }
};

// Every 97th entry of x, its 2-norm and its sum: enough to pin an iterate of
// 13,824 values in a small file.
void print_sample(const char* name, const std::vector<double>& x, bool last = false) {
  double n2 = 0, sm = 0;
  for (double v : x) { n2 += v * v; sm += v; }
  std::printf("  \"%s\": {\"norm2\": %.17g, \"sum\": %.17g, \"every97\": [", name, std::sqrt(n2), sm);
  for (size_t i = 0; i < x.size(); i += 97) std::printf("%s%.17g", i ? ", " : "", x[i]);
  std::printf("]}%s\n", last ? "" : ",");
}

int run_sipg() {
  SipgCase sym;
  SipgCase adv;
  adv.diffusion = 0.1;
  adv.mass = 1.0;
  adv.velocity[0] = 1.0;
  adv.velocity[1] = 0.5;
  adv.velocity[2] = 0.25;
  const size_t n = sym.ndofs();
  SpaceT sp;
  sp.aux.n = n;
  Vec b(sp, n);
  for (size_t i = 0; i < n; ++i) b.d[i] = std::sin(0.37 * double(i) + 0.2);
  Op A{[&](const std::vector<double>& x, std::vector<double>& y) { sym.apply(x, y); }};
  Op N{[&](const std::vector<double>& x, std::vector<double>& y) { adv.apply(x, y); }};
  const std::vector<double> dg = sym.diagonal();
  // the diagonal preconditioner (solver/diagonalpreconditioner.hh: 1/diag)
  Op D{[&](const std::vector<double>& x, std::vector<double>& y) {
    for (size_t i = 0; i < x.size(); ++i) y[i] = x[i] / dg[i];
  }};
  const int rel = Dune::Fem::LinearSolver::ToleranceCriteria::relative;
  std::printf("{\n  \"problem\": \"8^3 DG Q2, q = 4, penalty 90, weak u = 0; b_i = sin(0.37 i + 0.2); "
              "gmres, bicgstab: diffusion 0.1, mass 1, velocity (1, 0.5, 0.25)\",\n  \"n\": %zu,\n", n);
  {
    std::vector<Vec> tmp(3, Vec(sp, n));
    Vec x(sp, n);
    int it = Dune::Fem::LinearSolver::cg(A, (Op*)nullptr, tmp, x, b, 1e-10, 5000, rel);
    std::printf("  \"cg_iterations\": %d,\n", it);
    print_sample("cg_x", x.d);
  }
  {
    std::vector<Vec> tmp(5, Vec(sp, n));
    Vec x(sp, n);
    int it = Dune::Fem::LinearSolver::cg(A, &D, tmp, x, b, 1e-10, 5000, rel);
    std::printf("  \"diag_pcg_iterations\": %d,\n", it);
    print_sample("diag_pcg_x", x.d);
  }
  {
    const int m = 20;
    std::vector<Vec> v(m + 1, Vec(sp, n));
    Vec x(sp, n);
    int it = Dune::Fem::LinearSolver::gmres(N, (Op*)nullptr, v, x, b, m, 1e-10, 5000, rel);
    std::printf("  \"gmres_restart\": %d,\n  \"gmres_iterations\": %d,\n", m, it);
    print_sample("gmres_x", x.d);
  }
  {
    std::vector<Vec> v(5, Vec(sp, n));
    Vec x(sp, n);
    int it = Dune::Fem::LinearSolver::bicgstab(N, (Op*)nullptr, v, x, b, 1e-10, 5000, rel);
    std::printf("  \"bicgstab_iterations\": %d,\n", it);
    print_sample("bicgstab_x", x.d, true);
  }
  std::printf("}\n");
  return 0;
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
  if (what == "sipg") return run_sipg();
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
