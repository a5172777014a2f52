// Coefficient-space apply of the same DG operator for constant coefficients.
//
// With kappa constant, affine Cartesian cells and the orthonormal Legendre
// basis, every integral of the form is an integral of a product of two
// polynomials of degree <= 2p in each direction.  Gauss quadrature with
// q >= p+1 points integrates those exactly, so the quadrature result equals
// the closed form below up to rounding (tested to 1e-12 against the
// quadrature oracle):
//
//  volume   w[l] += sum_d  eps |K|/h_d^2 (K1 u)_d  -  b_d |K|/h_d (D1 u)_d  +  c |K| u[l]
//           K1[i][j] = int_0^1 L_i' L_j',  D1[i][j] = int_0^1 L_i' L_j  (applied along axis d)
//  faces    the tangential mass matrices are the identity, so the face terms
//           act on the n x n trace coefficients directly:
//           J = v- - v+,  A = (dn- + dn+)/2,
//           Val = |F| (eps (sigma J - A) + (b.n) v_upwind),  Grad = -|F| eps J / 2
//           (boundary: Val = |F| (eps (sigma v- - dn-) + max(b.n,0) v-), Grad = -|F| eps v-)
//           w[i,jk] += L_i(s) Val[jk] + (n.e_d/h_d) L_i'(s) Grad[jk]
//
// Two kernels (the FP64 pipe is the binding resource, so work is traded for
// a little extra traffic, and every constant that can be is folded into a
// table):
//  1. dg_trace_kernel: every cell's face values v(s) = sum_i L_i(s) u_i and
//     one more trace per face into a buffer [cell][face][v|P][n^2].  With
//     sigma_s = -1, +1 the outward sign of face s, A1 = |F| eps sigma and
//     A2 = |F| eps / (2h):
//       constant kappa   P(s) = v(s) - sigma_s r d(s),  r = A2 / C, C = A1
//                        (C = 1 when A1 = 0), d(s) = sum_i L_i'(s) u_i;
//       kappa per cell   P(s) = sigma_s d(s), the outward normal derivative.
//     Both are sum_i c_i(s) u_i with c_i(0) = (-1)^i c_i(1) (L_i(1-x) =
//     (-1)^i L_i(x)), so both faces of a line come from one even and one odd
//     partial sum.
//  2. dg_const_kernel: numerical fluxes from the own and the neighbour's
//     traces (owner computes, no scatter).  For constant kappa, in units of C
//     for Val and of -A2 for Grad,
//       Val/C = P- - P+ + (A1/C - 1) J (+ upwind / C),   Grad/(-A2) = J,
//     two instructions per interior face coefficient; C and -A2 sit in the
//     per-axis expansion tables.  Then one pass per axis over the lines of
//     the cell: the 1-D operator M_d (a warp-uniform operand; its structural
//     zeros are skipped: the stiffness part lives on i, j >= 1 with i+j even,
//     the advection part on j < i with i+j odd) plus the face expansion,
//     again split into even and odd i.
// Every output is one thread's fixed-order sum: deterministic, independent of
// the launch shape.
#pragma once
#include <cuda_runtime.h>

#include "dg_kernel.cuh"

namespace gbfem {

template <typename T>
struct DgConstTablesT {
  T K1[kDgMaxN * kDgMaxN];  // K1[i*n+j] = int L_i' L_j'
  T D1[kDgMaxN * kDgMaxN];  // D1[i*n+j] = int L_i' L_j
  T tr[2 * kDgMaxN];        // L_i(s)
  T dtr[2 * kDgMaxN];       // L_i'(s)
  T M[3][kDgMaxN * kDgMaxN];  // per-axis line operator (filled per operator)
  // per-axis flux constants: A1 = |F| eps sigma, A2 = |F| eps / (2 h)
  T A1[3], A2[3];
  T massK;  // cellwise kappa: c |K| (the mass term, kept out of M)
  // folded constants (filled per operator with M):
  T pc[3][kDgMaxN];    // second trace: P(1) = sum_i pc[d][i] u_i, P(0) = sum_i (-1)^i pc[d][i] u_i
  T etr[3][kDgMaxN];   // constant kappa: Val expansion C_d L_i(1)
  T edtr[3][kDgMaxN];  // constant kappa: Grad expansion -A2_d L_i'(1)
  T adv[6];            // constant kappa: upwind |F| (b.n_f) / C_d for face f = 2d+s
  T am1, am2;          // A1/C - 1, A1/C - 2 (the same on every axis)
};

// traces[cell][f = 2d+s][0: v, 1: P][jk] (P as above; KC selects the kappa
// per cell form, whose c_0 = L_0'(1) = 0) for the cells [cell_begin,
// cell_begin + count).  L_0 = 1, so the constant-kappa c_0 is 1 too and both
// even sums start from u_0.  ucopy (optional): the x-lines also store the
// dofs they read there, so a u read from host memory is copied to the device
// on the way (every dof exactly once).
template <typename T, int N, bool KC = false>
__global__ void __launch_bounds__(256) dg_trace_kernel(const T* __restrict__ u, T* __restrict__ traces,
                                                       long long cell_begin, long long count,
                                                       const __grid_constant__ DgConstTablesT<T> tabs,
                                                       T* __restrict__ ucopy) {
  constexpr int N2 = N * N, N3 = N2 * N;
  // one line per item; consecutive items are consecutive lines of a cell, so
  // a warp's loads of an axis-0 line are contiguous (what reads of u from
  // host memory need)
  const long long total = count * 3 * N2;
  for (long long item = blockIdx.x * (long long)blockDim.x + threadIdx.x; item < total;
       item += (long long)gridDim.x * blockDim.x) {
    long long lc;
    int r;
    if (total <= 0x7fffffffLL) {  // 32-bit division by the constant where it fits
      const int it = int(item);
      lc = it / (3 * N2);
      r = it - int(lc) * (3 * N2);
    } else {
      lc = item / (3 * N2);
      r = int(item - lc * 3 * N2);
    }
    const long long cell = cell_begin + lc;
    const int d = r / N2, jk = r - d * N2;
    const int j = jk / N, k = jk % N;
    const int base = d == 0 ? j * N + k : (d == 1 ? j * N2 + k : j * N2 + k * N);
    const int stride = d == 0 ? N2 : (d == 1 ? N : 1);
    const T* uc = u + cell * N3 + base;
    const T* pc = tabs.pc[d];
    T ev = T(0), od = T(0), pe = T(0), po = T(0);
#pragma unroll
    for (int i = 0; i < N; ++i) {
      const T x = __ldg(uc + i * stride);
      if (ucopy && d == 0) ucopy[cell * N3 + base + i * stride] = x;
      if (i == 0) {
        ev = x;
        if (!KC) pe = x;
      } else if (i & 1) {
        od = fma(tabs.tr[N + i], x, od);
        po = fma(pc[i], x, po);
      } else {
        ev = fma(tabs.tr[N + i], x, ev);
        pe = fma(pc[i], x, pe);
      }
    }
    T* tc = traces + cell * (12 * N2);
    tc[(2 * d + 0) * 2 * N2 + jk] = ev - od;       // v(0)
    tc[(2 * d + 0) * 2 * N2 + N2 + jk] = pe - po;  // P(0)
    tc[(2 * d + 1) * 2 * N2 + jk] = ev + od;       // v(1)
    tc[(2 * d + 1) * 2 * N2 + N2 + jk] = pe + po;  // P(1)
  }
}

// KC: a constant kappa per cell (args.kcell), no advection: the diffusion
// part of M_d is scaled by the cell's kappa, the fluxes use the two cells'
// values as the quadrature of kappa_bar [u][v] - {kappa grad u}.n [v] -
// [u] {kappa grad v}.n does; the mass term is one FMA on axis 0.
template <typename T, int N, int CPB, bool ADV, bool KC = false>
__global__ void __launch_bounds__(256) dg_const_kernel(const __grid_constant__ DgArgsT<T> args,
                                                       const T* __restrict__ traces,
                                                       const __grid_constant__ DgConstTablesT<T> tabs) {
  constexpr int N2 = N * N, N3 = N * N * N;
  static_assert(!(KC && ADV), "cellwise kappa without advection");
  __shared__ T su[CPB * N3];
  __shared__ T sr[CPB * N3];
  __shared__ T sF[CPB * 6 * 2 * N2];  // [cell][face][Val/Grad][jk]
  __shared__ T sK[KC ? CPB : 1];
  __shared__ long long sNb[CPB * 6];
  const int tid = threadIdx.x;
  // output cells [cell_begin, cend); neighbours anywhere in the grid
  const long long cend = args.cell_begin + (args.cell_count > 0 ? args.cell_count : args.ncells);
  const long long c0 = args.cell_begin + (long long)blockIdx.x * CPB;
  if (c0 >= cend) return;
  for (int e = tid; e < CPB * N3; e += blockDim.x) {
    const long long v = c0 + e / N3;
    su[e] = v < cend ? __ldg(args.u + c0 * N3 + e) : T(0);
  }
  if (KC)
    for (int c = tid; c < CPB; c += blockDim.x) sK[c] = c0 + c < cend ? __ldg(args.kcell + c0 + c) : T(0);
  // neighbour of each cell through each face (-1: boundary, or past the
  // range), once per cell and face rather than per face coefficient
  for (int e = tid; e < CPB * 6; e += blockDim.x) {
    const int c = e / 6, f = e - c * 6;
    const int d = f >> 1, s = f & 1;
    const long long cell = c0 + c;
    long long ncell = -1;
    if (cell < cend) {
      const long long nxy = (long long)args.nc[0] * args.nc[1];
      const long long cz = cell / nxy, rem = cell - cz * nxy;
      const long long cy = rem / args.nc[0], cx = rem - cy * args.nc[0];
      const long long ccd = d == 0 ? cx : (d == 1 ? cy : cz);  // the cell's index along d
      const long long strd = d == 0 ? 1 : (d == 1 ? (long long)args.nc[0] : nxy);
      const int ncd = args.nc[d];
      long long nb = ccd + (s ? 1 : -1);
      bool has_nb = true;
      if (nb < 0 || nb >= ncd) {
        if (args.periodic[d]) nb = (nb + ncd) % ncd;
        else has_nb = false;
      }
      if (has_nb) ncell = cell + (nb - ccd) * strd;
    }
    sNb[e] = ncell;
  }
  __syncthreads();
  // uniform FP64 tests, taken once (a compare occupies the FP64 pipe too)
  const bool fold_alpha = tabs.am1 != T(0);
  const bool has_mass = tabs.M[0][0] != T(0);
  const bool has_massK = KC && tabs.massK != T(0);
  // ---- faces: numerical fluxes from own and neighbour traces -----------------
  for (int item = tid; item < CPB * 6 * N2; item += blockDim.x) {
    const int c = item / (6 * N2);
    const int r = item - c * 6 * N2;
    const int f = r / N2, jk = r - f * N2;
    const int d = f >> 1, s = f & 1;
    const long long cell = c0 + c;
    const long long cl = cell < cend ? cell : c0;
    const long long ncell = sNb[c * 6 + f];
    const bool has_nb = ncell >= 0;
    // own face f and the neighbour's opposite face: v and P (see the top)
    const T* own = traces + cl * (12 * N2) + f * 2 * N2;
    const T vm = __ldg(own + jk), pm = __ldg(own + N2 + jk);
    T vp = T(0), pp = T(0);
    if (has_nb) {
      const T* nbt = traces + ncell * (12 * N2) + (2 * d + 1 - s) * 2 * N2;
      vp = __ldg(nbt + jk);
      pp = __ldg(nbt + N2 + jk);
    }
    T val = T(0), grad = T(0);
    if (KC) {
      // P = outward normal derivative D (no 1/h; A2 carries it):
      //   eps |F| (sigma kbar J - {kappa dn u}) = A1 kbar J - A2 (k- D- - k+ D+)
      //   -eps |F| kappa- J / 2 = -A2 k- J
      const T km = __ldg(args.kcell + cl);
      if (has_nb) {
        const T kp = __ldg(args.kcell + ncell);
        const T J = vm - vp;
        val = fma(tabs.A1[d] * (T(0.5) * (km + kp)), J, -tabs.A2[d] * (km * pm - kp * pp));
        grad = -tabs.A2[d] * km * J;
      } else if (args.weak_dirichlet) {
        val = fma(tabs.A1[d] * km, vm, T(-2) * tabs.A2[d] * km * pm);
        grad = T(-2) * tabs.A2[d] * km * vm;
      }
    } else if (has_nb) {
      // Val/C = P- - P+ + (A1/C - 1) J,  Grad/(-A2) = J
      const T J = vm - vp;
      val = pm - pp;
      if (fold_alpha) val = fma(tabs.am1, J, val);
      grad = J;
      if (ADV) {
        const T bn = s ? args.b[d] : -args.b[d];
        val = fma(tabs.adv[f], bn >= T(0) ? vm : vp, val);
      }
    } else {
      if (args.weak_dirichlet) {
        // eps |F| (sigma u - dn u) / C = 2 P- + (A1/C - 2) v-,  -eps |F| u / (-A2) = 2 v-
        val = fma(tabs.am2, vm, pm + pm);
        grad = vm + vm;
      }
      if (ADV) {
        const T bn = s ? args.b[d] : -args.b[d];
        if (bn > T(0)) val = fma(tabs.adv[f], vm, val);
      }
    }
    sF[(c * 6 + f) * 2 * N2 + jk] = val;
    sF[(c * 6 + f) * 2 * N2 + N2 + jk] = grad;
  }
  __syncthreads();
  // ---- volume + face expansion, one line along axis d per item ---------------
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    const int stride = d == 0 ? N2 : (d == 1 ? N : 1);
    for (int item = tid; item < CPB * N2; item += blockDim.x) {
      const int c = item / N2, jk = item - c * N2;
      const int j = jk / N, k = jk % N;
      const int base = d == 0 ? j * N + k : (d == 1 ? j * N2 + k : j * N2 + k * N);
      const T* uc = su + c * N3 + base;
      T x[N];
#pragma unroll
      for (int i = 0; i < N; ++i) x[i] = uc[i * stride];
      const T* fv0 = sF + (c * 6 + 2 * d) * 2 * N2;
      const T* fv1 = fv0 + 2 * N2;
      // sum_s L_i(s) Val_s = L_i(1) (Val_1 + (-1)^i Val_0); the gradient
      // terms likewise with (n.e_d/h) L_i'(s): L_i'(1) (G_1 + (-1)^i G_0).
      // Constant kappa: the factors C_d and -A2_d (which carries the 1/h) of
      // Val and Grad are in etr and edtr; KC: Val and G carry them.
      const T v0 = fv0[jk], v1 = fv1[jk], g0 = fv0[N2 + jk], g1 = fv1[N2 + jk];
      const T vs = v1 + v0, vd = v1 - v0, gs = g1 + g0, gd = g1 - g0;
      T* rc = sr + c * N3 + base;
      if (KC) {
        const T kc = sK[c];
#pragma unroll
        for (int i = 0; i < N; ++i) {
          T acc = d == 0 ? T(0) : rc[i * stride];
          T t = T(0);
#pragma unroll
          for (int jj = 0; jj < N; ++jj)
            if (i != 0 && jj != 0 && !((i + jj) & 1)) t = fma(tabs.M[d][i * N + jj], x[jj], t);
          acc = fma(kc, t, acc);
          if (d == 0 && has_massK) acc = fma(tabs.massK, x[i], acc);
          acc = fma(tabs.tr[N + i], (i & 1) ? vd : vs, acc);
          if (i > 0) acc = fma(tabs.dtr[N + i], (i & 1) ? gd : gs, acc);
          rc[i * stride] = acc;
        }
        continue;
      }
#pragma unroll
      for (int i = 0; i < N; ++i) {
        T acc = d == 0 ? T(0) : rc[i * stride];
#pragma unroll
        for (int jj = 0; jj < N; ++jj) {
          // structural zeros of M_d = eps K1 - b D1 (+ mass on axis 0):
          // K1[i][j] = int L_i' L_j' vanishes in row and column 0 and for i+j
          // odd; D1[i][j] = int L_i' L_j vanishes for j >= i (L_i' has degree
          // i-1) and for i+j even; the mass entry (0,0) sits on axis 0
          const bool mass00 = d == 0 && i == 0 && jj == 0 && has_mass;
          const bool k1 = i != 0 && jj != 0 && !((i + jj) & 1);
          const bool d1 = jj < i && ((i + jj) & 1);
          const bool nz = k1 || mass00 || (ADV && d1);
          if (nz) acc = fma(tabs.M[d][i * N + jj], x[jj], acc);
        }
        acc = fma(tabs.etr[d][i], (i & 1) ? vd : vs, acc);
        if (i > 0) acc = fma(tabs.edtr[d][i], (i & 1) ? gd : gs, acc);  // L_0'(1) = 0
        rc[i * stride] = acc;
      }
    }
    __syncthreads();
  }
  for (int e = tid; e < CPB * N3; e += blockDim.x) {
    const long long v = c0 + e / N3;
    if (v < cend) __stcs(args.w + c0 * N3 + e, sr[e]);
  }
}

}  // namespace gbfem
