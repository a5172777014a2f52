// CPU oracle of the matrix-free operator apply and Krylov solve.
//
// TEST INFRASTRUCTURE ONLY.  This file is the checker the GPU path is
// compared against and the timed CPU baseline; the product library never
// links, loads or calls it.
//
// It restates, in plain C++17, the reference algorithm of dune-fem for this
// path, following (paths relative to the dune-fem source tree):
//  * Impl::GalerkinOperator::evaluateImpl (dune/fem/schemes/galerkin.hh:811-917):
//    element loop; interior integral; per intersection a two-sided skeleton
//    integral when index(inside) < index(outside), a boundary integral on the
//    boundary; scatter of the outside contribution under a lock
//    (galerkin.hh:950-991);
//  * LocalGalerkinOperator::add{Interior,Skeleton,Boundary}Integral
//    (galerkin.hh:332-537): dense evaluation of u and grad u at every
//    quadrature point from cached basis values, integrand times
//    weight * integrationElement, dense axpy back into the test functions
//    (space/basisfunctionset/default.hh:276-487);
//  * the SIPG + upwind form of pydemo/advectiondiffusion.py:33-55;
//  * LegendreShapeFunction (space/shapefunctionset/legendre.hh:30-193) with
//    the shifted orthonormal Legendre polynomials evaluated by Horner on the
//    binomial coefficient form (legendrepolynomials.hh:24-46);
//  * tensor Gauss rules with the point index x[0] fastest
//    (quadrature/femquadratures_inline.hh:33-80);
//  * ThreadIterator's contiguous element partition
//    (misc/threads/threaditerator.hh:150-175);
//  * LinearSolver::cg and ::gmres (solver/linear/cg.hh:18-117,
//    solver/linear/gmres.hh:116-299);
//  * DirichletWrapperOperator's apply for continuous Q1 (w = Au, w_D = u_D,
//    schemes/dirichletwrapper.hh:101-105).
// Its tables are pinned against the reference's own compiled tables
// (tests/golden/ref_tables.json, made by oracle/make_ref_golden.sh).
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <functional>
#include <mutex>
#include <thread>
#include <vector>

namespace {

// ---------------------------------------------------------------- tables --
// factor[n][k] = (-1)^(n+k) C(n,k) C(n+k,k): shifted Legendre P_n(2x-1) in
// monomials of x; weight[n] = sqrt(2n+1) makes them orthonormal on [0,1].
double binom(int n, int k) {
  double r = 1.0;
  for (int i = 1; i <= k; ++i) r = r * (n - k + i) / i;
  return r;
}

struct Legendre {
  double factor[12][12];
  double weight[12];
  Legendre() {
    for (int n = 0; n < 12; ++n) {
      weight[n] = std::sqrt(2.0 * n + 1.0);
      for (int k = 0; k < 12; ++k)
        factor[n][k] = k <= n ? (((n + k) % 2) ? -1.0 : 1.0) * binom(n, k) * binom(n + k, k) : 0.0;
    }
  }
  double evaluate(int num, double x) const {
    double phi = factor[num][num];
    for (int i = num - 1; i >= 0; --i) phi = phi * x + factor[num][i];
    return weight[num] * phi;
  }
  double jacobian(int num, double x) const {
    double phi = 0.0;
    if (num >= 1) {
      phi = factor[num][num] * num;
      for (int i = num - 1; i >= 1; --i) phi = phi * x + factor[num][i] * i;
    }
    return weight[num] * phi;
  }
};
const Legendre& legendre() {
  static Legendre L;
  return L;
}

// Gauss-Legendre on [0,1] by Newton on P_m in long double, ascending points.
void gauss(int m, double* pts, double* wts) {
  const long double pi = 3.141592653589793238462643383279502884L;
  for (int i = 0; i < m; ++i) {
    long double x = std::cos(pi * (i + 0.75L) / (m + 0.5L));
    long double dp = 1.0L;
    for (int it = 0; it < 200; ++it) {
      long double p0 = 1.0L, p1 = x;
      for (int j = 2; j <= m; ++j) {
        long double p2 = ((2 * j - 1) * x * p1 - (j - 1) * p0) / j;
        p0 = p1;
        p1 = p2;
      }
      if (m == 1) { p1 = x; p0 = 1.0L; }
      dp = m * (x * p1 - p0) / (x * x - 1.0L);
      long double dx = p1 / dp;
      x -= dx;
      if (std::fabs(dx) < 1e-30L) break;
    }
    {
      long double p0 = 1.0L, p1 = x;
      for (int j = 2; j <= m; ++j) {
        long double p2 = ((2 * j - 1) * x * p1 - (j - 1) * p0) / j;
        p0 = p1;
        p1 = p2;
      }
      if (m == 1) { p1 = x; p0 = 1.0L; }
      dp = m * (x * p1 - p0) / (x * x - 1.0L);
    }
    pts[m - 1 - i] = double(0.5L * (1.0L + x));
    wts[m - 1 - i] = double(1.0L / ((1.0L - x * x) * dp * dp));
  }
}

// --------------------------------------------------------------- grid ----
struct Desc {
  int cells[3];
  double lower[3], upper[3];
  int periodic[3];
  int order, quad;
  double diffusion, penalty, mass;
  double velocity[3];
  int weak_dirichlet;
};

struct Space {
  Desc d;
  int n, nloc, q;
  long long ncells;
  double h[3], vol;
  std::vector<int> mi;            // multi-index [nloc][3], i0 slowest (legendre.hh:168-193)
  std::vector<double> gp, gw;     // 1-D Gauss rule
  // cached basis values at volume points: phi[qp][l], dphi[qp][l][3] (reference gradient)
  std::vector<double> vphi, vdphi, vwt;
  // face caches: for face f = 2*dir + side, points on the face in x-fastest order
  std::vector<double> fphi[6], fdphi[6], fwt[6];
  explicit Space(const Desc& dd) : d(dd) {
    n = d.order + 1;
    nloc = n * n * n;
    q = d.quad;
    ncells = (long long)d.cells[0] * d.cells[1] * d.cells[2];
    vol = 1.0;
    for (int k = 0; k < 3; ++k) {
      h[k] = (d.upper[k] - d.lower[k]) / d.cells[k];
      vol *= h[k];
    }
    for (int i0 = 0; i0 < n; ++i0)
      for (int i1 = 0; i1 < n; ++i1)
        for (int i2 = 0; i2 < n; ++i2) { mi.push_back(i0); mi.push_back(i1); mi.push_back(i2); }
    gp.resize(q);
    gw.resize(q);
    gauss(q, gp.data(), gw.data());
    const Legendre& L = legendre();
    const int nq = q * q * q;
    vphi.resize(nq * nloc);
    vdphi.resize(nq * nloc * 3);
    vwt.resize(nq);
    for (int iq = 0; iq < nq; ++iq) {
      int ix[3] = {iq % q, (iq / q) % q, iq / (q * q)};  // x[0] fastest
      double x[3] = {gp[ix[0]], gp[ix[1]], gp[ix[2]]};
      vwt[iq] = gw[ix[0]] * gw[ix[1]] * gw[ix[2]];
      for (int l = 0; l < nloc; ++l) {
        double v[3], dv[3];
        for (int k = 0; k < 3; ++k) {
          v[k] = L.evaluate(mi[3 * l + k], x[k]);
          dv[k] = L.jacobian(mi[3 * l + k], x[k]);
        }
        vphi[iq * nloc + l] = v[0] * v[1] * v[2];
        vdphi[(iq * nloc + l) * 3 + 0] = dv[0] * v[1] * v[2];
        vdphi[(iq * nloc + l) * 3 + 1] = v[0] * dv[1] * v[2];
        vdphi[(iq * nloc + l) * 3 + 2] = v[0] * v[1] * dv[2];
      }
    }
    const int nf = q * q;
    for (int f = 0; f < 6; ++f) {
      const int dir = f / 2, side = f % 2;
      int t0 = dir == 0 ? 1 : 0, t1 = dir == 2 ? 1 : 2;
      fphi[f].resize(nf * nloc);
      fdphi[f].resize(nf * nloc * 3);
      fwt[f].resize(nf);
      for (int iq = 0; iq < nf; ++iq) {
        double x[3];
        x[dir] = side;
        x[t0] = gp[iq % q];
        x[t1] = gp[iq / q];
        fwt[f][iq] = gw[iq % q] * gw[iq / q];
        for (int l = 0; l < nloc; ++l) {
          double v[3], dv[3];
          for (int k = 0; k < 3; ++k) {
            v[k] = L.evaluate(mi[3 * l + k], x[k]);
            dv[k] = L.jacobian(mi[3 * l + k], x[k]);
          }
          fphi[f][iq * nloc + l] = v[0] * v[1] * v[2];
          fdphi[f][(iq * nloc + l) * 3 + 0] = dv[0] * v[1] * v[2];
          fdphi[f][(iq * nloc + l) * 3 + 1] = v[0] * dv[1] * v[2];
          fdphi[f][(iq * nloc + l) * 3 + 2] = v[0] * v[1] * dv[2];
        }
      }
    }
  }
  void coords(long long c, long long* x) const {
    x[0] = c % d.cells[0];
    x[1] = (c / d.cells[0]) % d.cells[1];
    x[2] = c / ((long long)d.cells[0] * d.cells[1]);
  }
  long long index(const long long* x) const { return x[0] + d.cells[0] * (x[1] + (long long)d.cells[1] * x[2]); }
  // neighbour through face f; -1 on a non-periodic boundary
  long long neighbour(long long c, int f) const {
    long long x[3];
    coords(c, x);
    const int dir = f / 2;
    x[dir] += (f % 2) ? 1 : -1;
    if (x[dir] < 0 || x[dir] >= d.cells[dir]) {
      if (!d.periodic[dir]) return -1;
      x[dir] = (x[dir] + d.cells[dir]) % d.cells[dir];
    }
    return index(x);
  }
};

// Evaluate value and physical gradient of a local function at face point iq.
inline void eval_face(const Space& S, int f, int iq, const double* ul, double* val, double* grad) {
  const double* phi = &S.fphi[f][iq * S.nloc];
  const double* dphi = &S.fdphi[f][iq * S.nloc * 3];
  double v = 0, g[3] = {0, 0, 0};
  for (int l = 0; l < S.nloc; ++l) {
    v += phi[l] * ul[l];
    for (int k = 0; k < 3; ++k) g[k] += dphi[3 * l + k] * ul[l];
  }
  *val = v;
  for (int k = 0; k < 3; ++k) grad[k] = g[k] / S.h[k];
}

// axpy of (val*phi + grad_n * n.grad phi) at face point iq into wl.
inline void axpy_face(const Space& S, int f, int iq, double val, double gn, const double* n, double* wl) {
  const double* phi = &S.fphi[f][iq * S.nloc];
  const double* dphi = &S.fdphi[f][iq * S.nloc * 3];
  for (int l = 0; l < S.nloc; ++l) {
    double dn = 0;
    for (int k = 0; k < 3; ++k) dn += n[k] * dphi[3 * l + k] / S.h[k];
    wl[l] += val * phi[l] + gn * dn;
  }
}

struct Lockset {
  std::vector<std::mutex> m;
  explicit Lockset(size_t n) : m(n) {}
  std::mutex& of(long long c) { return m[size_t(c) % m.size()]; }
};

void dg_apply_range(const Space& S, const double* u, const double* kappa, double* w, long long c0, long long c1,
                    Lockset& locks, bool threaded) {
  const Desc& d = S.d;
  const int nloc = S.nloc;
  const int nq = S.q * S.q * S.q, nf = S.q * S.q;
  std::vector<double> wl(nloc), wo(nloc);
  const bool adv = d.velocity[0] != 0 || d.velocity[1] != 0 || d.velocity[2] != 0;
  for (long long c = c0; c < c1; ++c) {
    const double* ul = u + c * nloc;
    const double* kl = kappa ? kappa + c * nloc : nullptr;
    std::fill(wl.begin(), wl.end(), 0.0);
    // interior integral (galerkin.hh:332-360)
    for (int iq = 0; iq < nq; ++iq) {
      const double* phi = &S.vphi[iq * nloc];
      const double* dphi = &S.vdphi[iq * nloc * 3];
      double uv = 0, g[3] = {0, 0, 0}, kv = kl ? 0.0 : 1.0;
      for (int l = 0; l < nloc; ++l) {
        uv += phi[l] * ul[l];
        for (int k = 0; k < 3; ++k) g[k] += dphi[3 * l + k] * ul[l];
        if (kl) kv += phi[l] * kl[l];
      }
      const double wt = S.vwt[iq] * S.vol;
      double F[3];
      for (int k = 0; k < 3; ++k) F[k] = d.diffusion * kv * g[k] / S.h[k] - (adv ? d.velocity[k] * uv : 0.0);
      const double src = d.mass * uv;
      for (int l = 0; l < nloc; ++l) {
        double t = src * phi[l];
        for (int k = 0; k < 3; ++k) t += F[k] * dphi[3 * l + k] / S.h[k];
        wl[l] += wt * t;
      }
    }
    // intersections in the order -x,+x,-y,+y,-z,+z
    for (int f = 0; f < 6; ++f) {
      const int dir = f / 2, side = f % 2;
      double n[3] = {0, 0, 0};
      n[dir] = side ? 1.0 : -1.0;
      const double area = S.vol / S.h[dir];
      const long long o = S.neighbour(c, f);
      const double bn = adv ? d.velocity[dir] * n[dir] : 0.0;
      if (o >= 0) {
        if (!(c < o)) continue;  // neighbour handled from the lower index (galerkin.hh:879)
        const int fo = 2 * dir + (1 - side);
        const double* uo = u + o * nloc;
        const double* ko = kappa ? kappa + o * nloc : nullptr;
        const double hF = S.vol / area;  // avg(CellVolume)/FacetArea on a uniform grid
        const double sigma = d.penalty / hF;
        std::fill(wo.begin(), wo.end(), 0.0);
        for (int iq = 0; iq < nf; ++iq) {
          double vi, gi[3], vo, go[3], ki = 1, ko_ = 1, gk[3];
          eval_face(S, f, iq, ul, &vi, gi);
          eval_face(S, fo, iq, uo, &vo, go);
          if (kl) { eval_face(S, f, iq, kl, &ki, gk); eval_face(S, fo, iq, ko, &ko_, gk); }
          const double W = S.fwt[f][iq] * area;
          const double J = vi - vo;
          const double kbar = 0.5 * (ki + ko_);
          double avgflux = 0;
          for (int k = 0; k < 3; ++k) avgflux += 0.5 * (ki * gi[k] + ko_ * go[k]) * n[k];
          double val = d.diffusion * (sigma * kbar * J - avgflux);
          if (adv) val += bn * (bn >= 0 ? vi : vo);
          axpy_face(S, f, iq, W * val, W * d.diffusion * (-0.5 * ki * J), n, wl.data());
          axpy_face(S, fo, iq, -W * val, W * d.diffusion * (-0.5 * ko_ * J), n, wo.data());
        }
        if (threaded) {
          std::lock_guard<std::mutex> g(locks.of(o));
          for (int l = 0; l < nloc; ++l) w[o * nloc + l] += wo[l];
        } else {
          for (int l = 0; l < nloc; ++l) w[o * nloc + l] += wo[l];
        }
      } else {
        // boundary integral (galerkin.hh:414-435): weak homogeneous Dirichlet.
        // weak_dirichlet 1: symmetric SIPG (-u kappa grad v . n in full);
        // weak_dirichlet 2: the boundary of dune-fem's DGEllipticOperator,
        // which weights that symmetry term by 1/2 (dgelliptic.hh:426-431)
        const double hB = S.vol / area;
        const double sym = d.weak_dirichlet == 2 ? 0.5 : 1.0;
        const double sigma = d.penalty / hB;
        for (int iq = 0; iq < nf; ++iq) {
          double vi, gi[3], ki = 1, gk[3];
          eval_face(S, f, iq, ul, &vi, gi);
          if (kl) eval_face(S, f, iq, kl, &ki, gk);
          const double W = S.fwt[f][iq] * area;
          double dn = 0;
          for (int k = 0; k < 3; ++k) dn += gi[k] * n[k];
          double val = 0, gn = 0;
          if (d.weak_dirichlet) {
            val = d.diffusion * (sigma * ki * vi - ki * dn);
            gn = d.diffusion * (-sym * ki * vi);
          }
          if (adv && bn > 0) val += bn * vi;
          axpy_face(S, f, iq, W * val, W * gn, n, wl.data());
        }
      }
    }
    // addLocalDofs(inside) under the lock
    if (threaded) {
      std::lock_guard<std::mutex> g(locks.of(c));
      for (int l = 0; l < nloc; ++l) w[c * nloc + l] += wl[l];
    } else {
      for (int l = 0; l < nloc; ++l) w[c * nloc + l] += wl[l];
    }
  }
}

void run_partitioned(long long n, int nthreads, const std::function<void(long long, long long)>& fn) {
  if (nthreads <= 1) { fn(0, n); return; }
  std::vector<std::thread> th;
  for (int t = 0; t < nthreads; ++t) {
    // contiguous blocks, sizes differ by at most one (threaditerator.hh:153-173)
    long long b = n * t / nthreads, e = n * (t + 1) / nthreads;
    th.emplace_back([=, &fn] { fn(b, e); });
  }
  for (auto& x : th) x.join();
}

Desc make_desc(const int* cells, const double* lower, const double* upper, const int* periodic, int order, int quad,
               double diffusion, double penalty, double mass, const double* velocity, int weak_dirichlet) {
  Desc d;
  for (int k = 0; k < 3; ++k) {
    d.cells[k] = cells[k];
    d.lower[k] = lower[k];
    d.upper[k] = upper[k];
    d.periodic[k] = periodic[k];
    d.velocity[k] = velocity ? velocity[k] : 0.0;
  }
  d.order = order;
  d.quad = quad;
  d.diffusion = diffusion;
  d.penalty = penalty;
  d.mass = mass;
  d.weak_dirichlet = weak_dirichlet;
  return d;
}

}  // namespace

extern "C" {

// 1-D tables for pinning against the reference's compiled ones.
void oracle_gauss(int m, double* pts, double* wts) { gauss(m, pts, wts); }
double oracle_legendre(int num, double x) { return legendre().evaluate(num, x); }
double oracle_legendre_d(int num, double x) { return legendre().jacobian(num, x); }

// w = A u for the DG SIPG/upwind/mass operator; nthreads threads with locked scatter.
int oracle_dg_apply(const int* cells, const double* lower, const double* upper, const int* periodic, int order,
                    int quad, double diffusion, double penalty, double mass, const double* velocity,
                    int weak_dirichlet, const double* kappa, const double* u, double* w, int nthreads) {
  Desc d = make_desc(cells, lower, upper, periodic, order, quad, diffusion, penalty, mass, velocity, weak_dirichlet);
  Space S(d);
  std::memset(w, 0, sizeof(double) * size_t(S.ncells) * S.nloc);
  Lockset locks(4096);
  run_partitioned(S.ncells, nthreads, [&](long long b, long long e) {
    dg_apply_range(S, u, kappa, w, b, e, locks, nthreads > 1);
  });
  return 0;
}

// Contributions of cells [c0, c1) only (interior, their boundary faces and
// the faces they own by the index rule), threads over that range.  Used to
// time a bounded sample of a large apply; w is not cleared.
int oracle_dg_apply_cells(const int* cells, const double* lower, const double* upper, const int* periodic, int order,
                          int quad, double diffusion, double penalty, double mass, const double* velocity,
                          int weak_dirichlet, const double* kappa, const double* u, double* w, long long c0,
                          long long c1, int nthreads) {
  Desc d = make_desc(cells, lower, upper, periodic, order, quad, diffusion, penalty, mass, velocity, weak_dirichlet);
  Space S(d);
  Lockset locks(4096);
  run_partitioned(c1 - c0, nthreads, [&](long long b, long long e) {
    dg_apply_range(S, u, kappa, w, c0 + b, c0 + e, locks, nthreads > 1);
  });
  return 0;
}

// Dense element-diagonal blocks [cell][i][j] by applying the operator to
// unit vectors with all other cells' dofs zero (the diagonal blocks of the
// assembled Jacobian, operator/linear/blockdiagonal.hh:24-135).
int oracle_dg_block_diagonal(const int* cells, const double* lower, const double* upper, const int* periodic,
                             int order, int quad, double diffusion, double penalty, double mass,
                             const double* velocity, int weak_dirichlet, const double* kappa, double* blocks,
                             int nthreads) {
  Desc d = make_desc(cells, lower, upper, periodic, order, quad, diffusion, penalty, mass, velocity, weak_dirichlet);
  Space S(d);
  const int nloc = S.nloc;
  const long long nd = S.ncells * nloc;
  run_partitioned(S.ncells, nthreads, [&](long long b, long long e) {
    std::vector<double> u(size_t(nd), 0.0), w(size_t(nd), 0.0);
    Lockset locks(1);
    for (long long c = b; c < e; ++c) {
      // cells whose faces touch c: itself and its neighbours; apply only to them
      std::vector<long long> touch = {c};
      for (int f = 0; f < 6; ++f) {
        long long o = S.neighbour(c, f);
        if (o >= 0 && std::find(touch.begin(), touch.end(), o) == touch.end()) touch.push_back(o);
      }
      for (int j = 0; j < nloc; ++j) {
        u[c * nloc + j] = 1.0;
        for (long long t : touch) std::fill(w.begin() + t * nloc, w.begin() + (t + 1) * nloc, 0.0);
        for (long long t : touch) dg_apply_range(S, u.data(), kappa, w.data(), t, t + 1, locks, false);
        for (int i = 0; i < nloc; ++i) blocks[(c * nloc + i) * nloc + j] = w[c * nloc + i];
        u[c * nloc + j] = 0.0;
      }
    }
  });
  return 0;
}

// Continuous Q1 on a 2-D grid: w = A u with strong Dirichlet rows w_D = u_D.
// Element loop with dense 2x2-Gauss element matrices (galerkin.hh:332-360).
int oracle_q1_apply(const int* cells, const double* lower, const double* upper, double diffusion, double mass,
                    const double* u, double* w, int diag_only) {
  const int nx = cells[0], ny = cells[1];
  const double hx = (upper[0] - lower[0]) / nx, hy = (upper[1] - lower[1]) / ny;
  double gp[2], gw[2];
  gauss(2, gp, gw);
  double K[4][4];
  for (int a = 0; a < 4; ++a)
    for (int b = 0; b < 4; ++b) {
      double s = 0;
      for (int iq = 0; iq < 4; ++iq) {
        double x = gp[iq % 2], y = gp[iq / 2];
        auto phi = [&](int k, double* v, double* dx, double* dy) {
          int kx = k & 1, ky = k >> 1;
          double fx = kx ? x : 1 - x, fy = ky ? y : 1 - y;
          *v = fx * fy;
          *dx = (kx ? 1.0 : -1.0) * fy / hx;
          *dy = fx * (ky ? 1.0 : -1.0) / hy;
        };
        double va, xa, ya, vb, xb, yb;
        phi(a, &va, &xa, &ya);
        phi(b, &vb, &xb, &yb);
        s += gw[iq % 2] * gw[iq / 2] * hx * hy * (diffusion * (xa * xb + ya * yb) + mass * va * vb);
      }
      K[a][b] = s;
    }
  const long long nv = (long long)(nx + 1) * (ny + 1);
  std::memset(w, 0, sizeof(double) * nv);
  for (int ey = 0; ey < ny; ++ey)
    for (int ex = 0; ex < nx; ++ex) {
      long long g[4];
      for (int k = 0; k < 4; ++k) g[k] = (long long)(ey + (k >> 1)) * (nx + 1) + ex + (k & 1);
      for (int a = 0; a < 4; ++a)
        for (int b = 0; b < 4; ++b) {
          if (diag_only) { if (a == b) w[g[a]] += K[a][a]; }
          else w[g[a]] += K[a][b] * u[g[b]];
        }
    }
  for (long long v = 0; v < nv; ++v) {
    int vx = int(v % (nx + 1)), vy = int(v / (nx + 1));
    if (vx == 0 || vy == 0 || vx == nx || vy == ny) w[v] = diag_only ? 1.0 : u[v];
  }
  return 0;
}

// L2 projection of a closed-form function onto DG Q_p (kind 0: exp of a
// Fourier sum with modes[m] = (wx, wy, wz, phi, a); 1: Gaussian bump with
// params (cx, cy, cz, width); 2: constant params[0]); direct evaluation at
// every quadrature point, dense basis (the interpolation/projection of a
// grid function into a DiscreteFunction).
int oracle_dg_project(const int* cells, const double* lower, const double* upper, int order, int quad, int kind,
                      const double* params, const double* modes, int nmodes, int scale_by_volume, double* out) {
  const int zero3[3] = {0, 0, 0};
  const double zv[3] = {0, 0, 0};
  Desc d = make_desc(cells, lower, upper, zero3, order, quad, 0, 0, 0, zv, 0);
  Space S(d);
  const double pi = 3.14159265358979323846;
  const int nq = S.q * S.q * S.q;
  for (long long c = 0; c < S.ncells; ++c) {
    long long xc[3];
    S.coords(c, xc);
    for (int l = 0; l < S.nloc; ++l) out[c * S.nloc + l] = 0.0;
    for (int iq = 0; iq < nq; ++iq) {
      const int ix[3] = {iq % S.q, (iq / S.q) % S.q, iq / (S.q * S.q)};
      double x[3];
      for (int k = 0; k < 3; ++k) x[k] = d.lower[k] + (double(xc[k]) + S.gp[ix[k]]) * S.h[k];
      double f;
      if (kind == 0) {
        double sum = 0.0;
        for (int m = 0; m < nmodes; ++m) {
          const double* md = modes + 5 * m;
          sum += md[4] * std::cos(2.0 * pi * (md[0] * x[0] + md[1] * x[1] + md[2] * x[2]) + md[3]);
        }
        f = std::exp(sum);
      } else if (kind == 1) {
        double r2 = 0.0;
        for (int k = 0; k < 3; ++k) r2 += (x[k] - params[k]) * (x[k] - params[k]);
        f = std::exp(-r2 / (params[3] * params[3]));
      } else {
        f = params[0];
      }
      const double wf = S.vwt[iq] * f * (scale_by_volume ? S.vol : 1.0);
      for (int l = 0; l < S.nloc; ++l) out[c * S.nloc + l] += wf * S.vphi[iq * S.nloc + l];
    }
  }
  return 0;
}

// One step of SSP-RK3 (TVD3 Butcher table, solver/rungekutta/butchertable.cc:
// 43-52) in the Butcher form of ExplicitRungeKuttaSolver::solve
// (solver/rungekutta/explicit.hh:160-215) for u' = L(u) = -A(u)/|K|.
int oracle_dg_rk3_step(const int* cells, const double* lower, const double* upper, const int* periodic, int order,
                       int quad, double diffusion, double penalty, double mass, const double* velocity,
                       int weak_dirichlet, const double* kappa, double* u, double dt, int nthreads) {
  Desc d = make_desc(cells, lower, upper, periodic, order, quad, diffusion, penalty, mass, velocity, weak_dirichlet);
  Space S(d);
  const long long n = S.ncells * S.nloc;
  static const double A[3][3] = {{0, 0, 0}, {1.0, 0, 0}, {0.25, 0.25, 0}};
  static const double b[3] = {1.0 / 6.0, 1.0 / 6.0, 2.0 / 3.0};
  std::vector<std::vector<double>> k(3, std::vector<double>(n));
  std::vector<double> y(n);
  Lockset locks(4096);
  auto L = [&](const double* in, double* out) {
    std::memset(out, 0, sizeof(double) * n);
    run_partitioned(S.ncells, nthreads, [&](long long bb, long long ee) {
      dg_apply_range(S, in, kappa, out, bb, ee, locks, nthreads > 1);
    });
    for (long long i = 0; i < n; ++i) out[i] *= -1.0 / S.vol;  // applyInverseMass
  };
  L(u, k[0].data());
  for (int i = 1; i < 3; ++i) {
    for (long long t = 0; t < n; ++t) {
      double v = u[t];
      for (int j = 0; j < i; ++j) v += A[i][j] * dt * k[j][t];
      y[t] = v;
    }
    L(y.data(), k[i].data());
  }
  for (int j = 0; j < 3; ++j)
    for (long long t = 0; t < n; ++t) u[t] += b[j] * dt * k[j][t];
  return 0;
}

// One SSP-RK3 step as oracle_dg_rk3_step, evaluated only where the result on
// the z-planes [z0, z1) depends on it (a bounded sample of a large step, for
// comparing whole planes at full grid size).  Stage i's operator is applied
// over the target planes widened by 3 - i planes (wrapping in z when the grid
// is periodic there, clipped otherwise): every face of a cell in the planes
// widened by 2 - i is then owned by a cell that is applied, so those rows are
// complete.  Same stage formulas and operation order as the full step.  u is
// full-size; only the target planes are updated.
int oracle_dg_rk3_step_planes(const int* cells, const double* lower, const double* upper, const int* periodic,
                              int order, int quad, double diffusion, double penalty, double mass,
                              const double* velocity, int weak_dirichlet, const double* kappa, double* u, double dt,
                              int z0, int z1, int nthreads) {
  Desc d = make_desc(cells, lower, upper, periodic, order, quad, diffusion, penalty, mass, velocity, weak_dirichlet);
  Space S(d);
  const int nz = cells[2];
  if (z0 < 0 || z1 > nz || z0 >= z1) return -1;
  const long long nxy = (long long)cells[0] * cells[1];
  const long long per = nxy * S.nloc;  // dofs per plane
  const long long n = S.ncells * S.nloc;
  // planes of the target range widened by h, each once
  auto planes = [&](int h) {
    std::vector<int> pl;
    std::vector<char> seen(nz, 0);
    for (int z = z0 - h; z < z1 + h; ++z) {
      int zz = z;
      if (zz < 0 || zz >= nz) {
        if (!periodic[2]) continue;
        zz = ((zz % nz) + nz) % nz;
      }
      if (!seen[zz]) { seen[zz] = 1; pl.push_back(zz); }
    }
    return pl;
  };
  static const double A[3][3] = {{0, 0, 0}, {1.0, 0, 0}, {0.25, 0.25, 0}};
  static const double b[3] = {1.0 / 6.0, 1.0 / 6.0, 2.0 / 3.0};
  std::vector<std::vector<double>> k(3, std::vector<double>(n, 0.0));
  std::vector<double> y(n, 0.0);
  Lockset locks(4096);
  // out = -A(in)/|K|, complete on the planes widened by h - 1
  auto L = [&](const double* in, double* out, int h) {
    for (int z : planes(h))
      run_partitioned(nxy, nthreads, [&](long long bb, long long ee) {
        dg_apply_range(S, in, kappa, out, z * nxy + bb, z * nxy + ee, locks, nthreads > 1);
      });
    for (int z : planes(h - 1))
      for (long long i = z * per; i < (z + 1) * per; ++i) out[i] *= -1.0 / S.vol;  // applyInverseMass
  };
  L(u, k[0].data(), 3);
  for (int i = 1; i < 3; ++i) {
    for (int z : planes(3 - i))
      for (long long t = z * per; t < (z + 1) * per; ++t) {
        double v = u[t];
        for (int j = 0; j < i; ++j) v += A[i][j] * dt * k[j][t];
        y[t] = v;
      }
    L(y.data(), k[i].data(), 3 - i);
  }
  for (int j = 0; j < 3; ++j)
    for (int z = z0; z < z1; ++z)
      for (long long t = z * per; t < (z + 1) * per; ++t) u[t] += b[j] * dt * k[j][t];
  return 0;
}

// ---------------------------------------------------------------- Krylov --
typedef void (*oracle_op_fn)(void* ctx, const double* x, double* y);

static double dotp(long long n, const double* x, const double* y) {
  double s = 0;  // sequential order (function/common/scalarproducts.hh:115-127)
  for (long long i = 0; i < n; ++i) s += x[i] * y[i];
  return s;
}

// LinearSolver::cg (solver/linear/cg.hh:18-117).  prec may be null.
// Returns iterations, negative if not converged.  tol_criteria: 0 absolute,
// 1 relative, 2 residual reduction (solver/parameter.hh:14-17).
int oracle_cg(long long n, oracle_op_fn op, void* opctx, oracle_op_fn prec, void* pctx, double* x, const double* b,
              double epsilon, int max_iter, int tol_criteria, double* out_residual) {
  std::vector<double> h(n), r(n), p(n), s, q;
  op(opctx, x, h.data());
  for (long long i = 0; i < n; ++i) { r[i] = h[i] - b[i]; p[i] = b[i] - h[i]; }
  double* qp = p.data();
  double* sp = p.data();
  if (prec) {
    s.resize(n);
    q.resize(n);
    prec(pctx, p.data(), q.data());
    s = q;
    qp = q.data();
    sp = s.data();
  }
  double prev = 0, residual = dotp(n, p.data(), qp);
  const double tolerance = epsilon * epsilon * (tol_criteria == 1 ? dotp(n, b, b) : tol_criteria == 2 ? residual : 1.0);
  int it = 0;
  for (it = 0; residual > tolerance && it < max_iter; ++it) {
    if (it > 0) {
      const double beta = residual / prev;
      for (long long i = 0; i < n; ++i) qp[i] *= beta;
      if (prec) for (long long i = 0; i < n; ++i) qp[i] += sp[i];
      else for (long long i = 0; i < n; ++i) p[i] -= r[i];
    }
    op(opctx, qp, h.data());
    const double qdoth = dotp(n, qp, h.data());
    const double alpha = residual / qdoth;
    for (long long i = 0; i < n; ++i) x[i] += alpha * qp[i];
    if (prec) {
      for (long long i = 0; i < n; ++i) p[i] -= alpha * h[i];
      prec(pctx, p.data(), sp);
      prev = residual;
      residual = dotp(n, p.data(), sp);
    } else {
      for (long long i = 0; i < n; ++i) r[i] += alpha * h[i];
      prev = residual;
      residual = dotp(n, r.data(), r.data());
    }
  }
  if (out_residual) *out_residual = std::sqrt(residual);
  return it < max_iter ? it : -it;
}

// LinearSolver::gmres (solver/linear/gmres.hh:116-299), restart m, right
// preconditioning.  Returns iterations, negative if not converged.
int oracle_gmres(long long n, oracle_op_fn op, void* opctx, oracle_op_fn prec, void* pctx, double* u, const double* b,
                 int m, double tolerance, int max_iter, int tol_criteria, double* out_residual) {
  std::vector<std::vector<double>> v(m + 2, std::vector<double>(n));
  std::vector<double> H((m + 1) * m, 0.0), g(m + 1), s(m), c(m), y(m);
  auto Hm = [&](int i, int j) -> double& { return H[i * m + j]; };
  auto rotate = [](double* x, double* yy, double cc, double ss) {
    double a = *x, bb = *yy;
    *x = cc * a + ss * bb;
    *yy = cc * bb - ss * a;
  };
  double tol = tolerance;
  if (tol_criteria == 1) tol *= std::sqrt(dotp(n, b, b));
  int iterations = 0;
  double res = 0;
  while (true) {
    op(opctx, u, v[0].data());
    for (long long i = 0; i < n; ++i) v[0][i] -= b[i];
    res = std::sqrt(dotp(n, v[0].data(), v[0].data()));
    if (tol_criteria == 2 && iterations == 0) tol *= res;
    if (res <= tol * (1 + 1e-15)) break;
    g[0] = -res;
    for (int i = 1; i <= m; ++i) g[i] = 0.0;
    for (long long i = 0; i < n; ++i) v[0][i] *= 1.0 / res;
    for (int j = 0; j < m; ++j) {
      if (prec) {
        prec(pctx, v[j].data(), v[m + 1].data());
        op(opctx, v[m + 1].data(), v[j + 1].data());
      } else {
        op(opctx, v[j].data(), v[j + 1].data());
      }
      std::vector<double> gd(j + 1, 0.0);
      for (int l = 0; l <= j; ++l) gd[l] = dotp(n, v[j + 1].data(), v[l].data());
      for (int i = 0; i <= j; ++i) Hm(i, j) = gd[i];
      for (int l = 0; l <= j; ++l)
        for (long long i = 0; i < n; ++i) v[j + 1][i] -= gd[l] * v[l][i];
      Hm(j + 1, j) = std::sqrt(dotp(n, v[j + 1].data(), v[j + 1].data()));
      for (long long i = 0; i < n; ++i) v[j + 1][i] *= 1.0 / Hm(j + 1, j);
      for (int i = 0; i < j; ++i) rotate(&Hm(i + 1, j), &Hm(i, j), c[i], s[i]);
      const double hjj = Hm(j, j), hjpj = Hm(j + 1, j);
      const double nrm = std::sqrt(hjj * hjj + hjpj * hjpj);
      c[j] = hjj / nrm;
      s[j] = -hjpj / nrm;
      rotate(&Hm(j + 1, j), &Hm(j, j), c[j], s[j]);
      rotate(&g[j + 1], &g[j], c[j], s[j]);
      ++iterations;
      if (std::fabs(g[j + 1]) < tol || iterations >= max_iter) break;
    }
    int last = iterations % m;
    if (last == 0) last = m;
    for (int i = last - 1; i >= 0; --i) {
      double dt = 0;
      for (int k = 0; k < last - (i + 1); ++k) dt += Hm(i, i + 1 + k) * y[i + 1 + k];
      y[i] = (g[i] - dt) / Hm(i, i);
    }
    if (prec) {
      std::vector<double>& ut = v[m];
      std::fill(ut.begin(), ut.end(), 0.0);
      for (int i = 0; i < last; ++i)
        for (long long k = 0; k < n; ++k) ut[k] += y[i] * v[i][k];
      prec(pctx, ut.data(), v[m + 1].data());
      for (long long k = 0; k < n; ++k) u[k] += v[m + 1][k];
    } else {
      for (int i = 0; i < last; ++i)
        for (long long k = 0; k < n; ++k) u[k] += y[i] * v[i][k];
    }
    if (std::fabs(g[last]) < tol) break;
    if (iterations >= max_iter) break;
  }
  if (out_residual) *out_residual = res;
  return iterations < max_iter ? iterations : -iterations;
}

}  // extern "C"
