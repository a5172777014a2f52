// One-dimensional tables of the tensor-product DG space, computed on the host
// in long double and rounded once to the kernel's precision.
//
//  * Gauss-Legendre points/weights on [0,1] (the rule of dune-fem's GaussPts,
//    quadrature/gausspoints.hh:111-114, point order ascending), computed by
//    Newton's method on the Legendre recurrence.
//  * Orthonormal shifted Legendre polynomials L_k(t) = sqrt(2k+1) P_k(2t-1)
//    and their derivatives (space/shapefunctionset/legendrepolynomials.hh:
//    24-46 evaluates the same functions from a coefficient table; here they
//    come from the three-term recurrence).
//  * The collocation derivative matrix of the Lagrange polynomials through
//    the Gauss points (barycentric formula of Berrut & Trefethen, SIAM Rev.
//    2004), used to take gradients in quadrature-point space.
#pragma once
#include <cmath>
#include <vector>

namespace gbfem {

constexpr int kMaxN = 5;  // p <= 4
constexpr int kMaxQ = 7;  // q <= p+3 <= 7

// Legendre P_k(x) and P_k'(x) on [-1,1] by recurrence.
inline void legendre_p(int k, long double x, long double* p, long double* dp) {
  long double p0 = 1.0L, p1 = x, d0 = 0.0L, d1 = 1.0L;
  if (k == 0) { *p = 1.0L; *dp = 0.0L; return; }
  for (int j = 2; j <= k; ++j) {
    long double p2 = ((2 * j - 1) * x * p1 - (j - 1) * p0) / j;
    long double d2 = d0 + (2 * j - 1) * p1;  // P_j' = P_{j-2}' + (2j-1) P_{j-1}
    p0 = p1; p1 = p2; d0 = d1; d1 = d2;
  }
  *p = p1; *dp = d1;
}

// Orthonormal shifted Legendre L_k(t) on [0,1] and derivative d/dt.
inline void legendre01(int k, long double t, long double* v, long double* dv) {
  long double p, dp;
  legendre_p(k, 2.0L * t - 1.0L, &p, &dp);
  long double s = std::sqrt((long double)(2 * k + 1));
  *v = s * p;
  *dv = s * 2.0L * dp;
}

// q-point Gauss-Legendre rule on [0,1], points ascending.
inline void gauss01(int q, long double* pts, long double* wts) {
  const long double pi = 3.141592653589793238462643383279502884L;
  for (int i = 0; i < q; ++i) {
    // Chebyshev-like initial guess for the i-th root (descending in x) of P_q.
    long double x = std::cos(pi * (i + 0.75L) / (q + 0.5L));
    for (int it = 0; it < 100; ++it) {
      long double p, dp;
      legendre_p(q, x, &p, &dp);
      long double dx = p / dp;
      x -= dx;
      if (std::fabs(dx) < 1e-30L) break;
    }
    long double p, dp;
    legendre_p(q, x, &p, &dp);
    // root i (descending) -> ascending index q-1-i on [0,1]
    pts[q - 1 - i] = 0.5L * (1.0L + x);
    wts[q - 1 - i] = 1.0L / ((1.0L - x * x) * dp * dp);  // weight on [-1,1] is 2/(..), halved
  }
}

// All tables a tensor-product kernel with n = p+1 basis functions and q
// points per direction needs, in long double.
struct Tables1D {
  int n = 0, q = 0;
  long double pts[kMaxQ], wts[kMaxQ];
  long double B[kMaxQ][kMaxN];    // B[a][i]  = L_i(x_a)
  long double G[kMaxQ][kMaxN];    // G[a][i]  = L_i'(x_a)
  long double Dc[kMaxQ][kMaxQ];   // Dc[a][b] = l_b'(x_a), Lagrange basis through the points
  long double tr[2][kMaxN];       // tr[s][i]  = L_i(s),  s = 0,1
  long double dtr[2][kMaxN];      // dtr[s][i] = L_i'(s)
};

inline Tables1D make_tables(int n, int q) {
  Tables1D t;
  t.n = n;
  t.q = q;
  gauss01(q, t.pts, t.wts);
  for (int a = 0; a < q; ++a)
    for (int i = 0; i < n; ++i) legendre01(i, t.pts[a], &t.B[a][i], &t.G[a][i]);
  for (int s = 0; s < 2; ++s)
    for (int i = 0; i < n; ++i) legendre01(i, (long double)s, &t.tr[s][i], &t.dtr[s][i]);
  // barycentric weights
  long double bw[kMaxQ];
  for (int j = 0; j < q; ++j) {
    long double prod = 1.0L;
    for (int k = 0; k < q; ++k)
      if (k != j) prod *= (t.pts[j] - t.pts[k]);
    bw[j] = 1.0L / prod;
  }
  for (int a = 0; a < q; ++a) {
    long double diag = 0.0L;
    for (int b = 0; b < q; ++b) {
      if (a == b) continue;
      t.Dc[a][b] = (bw[b] / bw[a]) / (t.pts[a] - t.pts[b]);
      diag -= t.Dc[a][b];
    }
    t.Dc[a][a] = diag;
  }
  return t;
}

// 1-D stiffness and advection matrices of the orthonormal Legendre basis on
// [0,1], by (n+1)-point Gauss quadrature (exact for the degree-2p products).
struct ConstTables1D {
  long double K1[kMaxN][kMaxN];  // int L_i' L_j'
  long double D1[kMaxN][kMaxN];  // int L_i' L_j
};
inline ConstTables1D make_const_tables(int n) {
  ConstTables1D t{};
  long double p[kMaxQ], w[kMaxQ];
  gauss01(n + 1, p, w);
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < n; ++j) {
      long double k = 0, d = 0;
      for (int a = 0; a <= n; ++a) {
        long double vi, di, vj, dj;
        legendre01(i, p[a], &vi, &di);
        legendre01(j, p[a], &vj, &dj);
        k += w[a] * di * dj;
        d += w[a] * di * vj;
      }
      t.K1[i][j] = k;
      t.D1[i][j] = d;
    }
  return t;
}

}  // namespace gbfem
