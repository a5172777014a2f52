// Run-time compiled general DG forms on the structured Cartesian grid.
//
// The counterpart of dune-fem's generated integrands: python/dune/models/
// integrands/ufl.py turns a UFL form into a C++ integrands class with
// interior / skeleton / boundary methods (and their linearisations), and
// schemes/galerkin.hh integrates them: the volume term at the element's
// quadrature points (addInteriorIntegral, galerkin.hh:332-360), the two-sided
// face term (addSkeletonIntegral, :475-537) and the boundary term
// (addBoundaryIntegral, :414-435).  Here the user's pointwise functions are
// compiled by nvcc at run time into this kernel (the Python package's
// integrands module writes the source), for M solution components:
//
//   interior(x, u, g)                       -> s, F   : int_K  s.v + F:grad v
//   skeleton(x, n, sigma, uL, gL, uR, gR)   -> s, F   : int_F  s.vL + F:grad vL
//   boundary(x, n, sigma, u, g)             -> s, F   : int_dK s.v + F:grad v
//
// u[m] and g[m][k] = du_m/dx_k at the point, s[m] the coefficient of v_m and
// F[m][k] that of dv_m/dx_k, x the physical point, n the unit outer normal of
// the own cell, sigma = penalty / h_F.  The skeleton function gives the own
// side's test coefficients; every cell evaluates all six of its faces, so an
// interior face is evaluated once from each side (no scatter, no atomics).
//
// Linearisation: the same kernel instantiated on Dual<R> values evaluates
// S(u + e du) and keeps the e-part, the exact Jacobian-vector product
// S'(u) du (galerkin.hh:1548-1643 assembles the same derivative from the
// linearised integrands).  Unit directions give the Jacobian's diagonal
// blocks, its diagonal and its neighbour couplings (assembly).
//
// Dof layout: dof = cell * M n^3 + i * M + m for the tensor Legendre index i
// (i0 the x-degree, slowest) and component m: the reference's vector-valued
// DG spaces enumerate the scalar basis index times the range dimension plus
// the component (space/basisfunctionset/vectorial.hh:139-165,
// VerticalDofAlignment).
//
// How: one CTA of 128 threads owns CPB cells (or unit-direction "virtual
// cells"); sum factorisation through shared memory as in dg_kernel.cuh,
// with the M components as extra batched arrays; full gradients on the
// faces (normal part from the derivative traces, tangential parts by the
// collocation derivative on the face points), and tangential test
// derivatives folded back through the transposed collocation derivative.
#pragma once
#include <cuda_runtime.h>

#include "dg_kernel.cuh"
#include "form_dual.cuh"

namespace gbfem {
namespace form {

template <typename R>
struct FormArgs {
  const R* u;        // argument (mode 0) or linearisation point (other modes; null = 0)
  const R* du;       // mode 1: direction
  R* w;              // modes 0, 1
  R* blocks;         // modes 2-4
  int nc[3];
  int periodic[3];
  long long ncells;
  R lower[3];
  R h[3];
  R invh[3];
  R detK;
  R faceA[3];
  R sigma[3];        // penalty / h_F for faces normal to d
  int mode;          // 0: w = S(u); 1: w = S'(u) du; 2: blocks[c][i][j] = S'(u)_cc;
                     // 3: blocks[c*nloc+j] = the diagonal; 4: neighbour couplings
                     //    blocks[((c*7 + 1 + f)*nloc + i)*nloc + j] (f = 2d + s)
  long long cell_begin;
  long long cell_count;  // 0: up to the last cell
};

__host__ __device__ constexpr int form_cells_per_block(int q, int mc) {
  return q * q * q * mc >= 128 ? 1 : (2 * q * q * q * mc >= 128 ? 2 : 4);
}
__host__ __device__ constexpr int form_table_bytes(int rbytes) {
  return ((kDgMaxQ * kDgMaxN + kDgMaxQ * kDgMaxQ + kDgMaxQ + 4 * kDgMaxN) * rbytes + 15) / 16 * 16;
}
__host__ __device__ constexpr int form_work(int n, int q, int mc, int cpb) {
  return cpb * mc * (q * n * n + q * q * n + 4 * q * q * q) > cpb * mc * 8 * (n * n + q * n + 3 * q * q)
             ? cpb * mc * (q * n * n + q * q * n + 4 * q * q * q)
             : cpb * mc * 8 * (n * n + q * n + 3 * q * q);
}
// dynamic shared memory of a form kernel, bytes
__host__ __device__ constexpr long long form_smem_bytes(int n, int q, int mc, int cpb, int vbytes, int rbytes) {
  return form_table_bytes(rbytes) + (2LL * cpb * mc * n * n * n + form_work(n, q, mc, cpb)) * vbytes;
}

// building and reading values of the kernel's type (R, or Dual<R> in the
// linearised kernel)
template <class V> struct Val;
template <> struct Val<double> {
  __device__ static double make(double x, double) { return x; }
  __device__ static double out(double v) { return v; }
};
template <> struct Val<float> {
  __device__ static float make(float x, float) { return x; }
  __device__ static float out(float v) { return v; }
};
template <class R> struct Val<Dual<R>> {
  __device__ static Dual<R> make(R x, R dx) { return Dual<R>(x, dx); }
  __device__ static R out(const Dual<R>& v) { return v.d; }
};

// NB arrays of dims [I0][I1][I2] (array strides ics / ocs) contracted along
// AX with the real matrix M: !TR out[..o..] = sum_i M[o*LDM + i] in[..i..],
// TR M[i*LDM + o]; ACC adds to out.  One thread per output, fixed order.
template <class V, class R, int AX, int I0, int I1, int I2, int OUT, int LDM, bool TR, bool ACC, int NB>
__device__ __forceinline__ void fcontract(const V* __restrict__ in, int ics, V* __restrict__ out, int ocs,
                                          const R* __restrict__ M) {
  constexpr int IN = AX == 0 ? I0 : (AX == 1 ? I1 : I2);
  constexpr int O1 = AX == 1 ? OUT : I1;
  constexpr int O2 = AX == 2 ? OUT : I2;
  constexpr int O0 = AX == 0 ? OUT : I0;
  constexpr int OSZ = O0 * O1 * O2;
  constexpr int IS0 = I1 * I2, IS1 = I2;
  constexpr int ISA = AX == 0 ? IS0 : (AX == 1 ? IS1 : 1);
  for (int item = threadIdx.x; item < NB * OSZ; item += blockDim.x) {
    const int b = item / OSZ;
    const int r = item - b * OSZ;
    const int x0 = r / (O1 * O2);
    const int x1 = (r / O2) % O1;
    const int x2 = r % O2;
    const int o = AX == 0 ? x0 : (AX == 1 ? x1 : x2);
    const int ib = b * ics + (AX == 0 ? 0 : x0 * IS0) + (AX == 1 ? 0 : x1 * IS1) + (AX == 2 ? 0 : x2);
    V acc = ACC ? out[b * ocs + r] : V(0);
#pragma unroll
    for (int i = 0; i < IN; ++i) acc = vfma(TR ? M[i * LDM + o] : M[o * LDM + i], in[ib + i * ISA], acc);
    out[b * ocs + r] = acc;
  }
}

template <class F, typename R, typename V, int N, int Q, int MC>
__device__ __forceinline__ void form_body(const FormArgs<R>& args, const DgTablesT<R>& tabs) {
  constexpr int CPB = form_cells_per_block(Q, MC);
  constexpr int N2 = N * N, N3 = N2 * N, Q2 = Q * Q, Q3 = Q2 * Q, NLOC = MC * N3;
  constexpr int NBV = CPB * MC;  // batched volume arrays
  constexpr int FB = CPB * 2;    // (cell, side) pairs of one face direction
  extern __shared__ __align__(16) unsigned char smem_raw[];
  R* sB = reinterpret_cast<R*>(smem_raw);
  R* sDc = sB + kDgMaxQ * kDgMaxN;
  R* sw = sDc + kDgMaxQ * kDgMaxQ;
  R* str = sw + kDgMaxQ;
  R* sdtr = str + 2 * kDgMaxN;
  V* su = reinterpret_cast<V*>(smem_raw + form_table_bytes(int(sizeof(R))));  // [CPB][MC][N3]
  V* sr = su + CPB * NLOC;                                                      // [CPB][MC][N3]
  V* work = sr + CPB * NLOC;

  const int tid = threadIdx.x;
  for (int i = tid; i < Q * N; i += blockDim.x) sB[i] = tabs.B[i];
  for (int i = tid; i < Q * Q; i += blockDim.x) sDc[i] = tabs.Dc[i];
  for (int i = tid; i < Q; i += blockDim.x) sw[i] = tabs.w[i];
  for (int i = tid; i < 2 * N; i += blockDim.x) {
    str[i] = tabs.tr[i];
    sdtr[i] = tabs.dtr[i];
  }

  const int mode = args.mode;
  const long long count = args.cell_count > 0 ? args.cell_count : args.ncells - args.cell_begin;
  const int vper = mode == 4 ? 6 * NLOC : (mode >= 2 ? NLOC : 1);
  const long long nvirt = count * vper;
  const long long vbase = (long long)blockIdx.x * CPB;
  if (vbase >= nvirt) return;  // uniform over the CTA
  const long long nxy = (long long)args.nc[0] * args.nc[1];
  // virtual cell c of this CTA -> (cell, unit direction index); false past the end
  auto vcell = [&](int c, long long& cell, int& sub) -> bool {
    const long long v = vbase + c;
    if (v >= nvirt) {
      cell = args.cell_begin;
      sub = 0;
      return false;
    }
    cell = args.cell_begin + v / vper;
    sub = int(v % vper);
    return true;
  };
  auto coords = [&](long long cell, long long* cc) {
    cc[2] = cell / nxy;
    const long long rem = cell - cc[2] * nxy;
    cc[1] = rem / args.nc[0];
    cc[0] = rem - cc[1] * args.nc[0];
  };

  // ---- own dofs --------------------------------------------------------------
  for (int e = tid; e < CPB * NLOC; e += blockDim.x) {
    const int c = e / NLOC, r = e - c * NLOC;
    const int m = r / N3, i = r - m * N3;
    long long cell;
    int sub;
    V val = V(0);
    if (vcell(c, cell, sub)) {
      const int ldof = i * MC + m;
      const R x = args.u ? args.u[cell * NLOC + ldof] : R(0);
      R dx = R(0);
      if (mode == 1) dx = args.du[cell * NLOC + ldof];
      else if (mode == 2 || mode == 3) dx = ldof == sub ? R(1) : R(0);
      val = Val<V>::make(x, dx);
    }
    su[e] = val;
  }
  __syncthreads();

  // ---- volume ----------------------------------------------------------------
  {
    V* t1 = work;                 // [NBV][Q][N][N]
    V* t2 = t1 + NBV * Q * N2;    // [NBV][Q][Q][N]
    V* U = t2 + NBV * Q2 * N;     // [NBV][Q3]
    V* G0 = U + NBV * Q3;
    V* G1 = G0 + NBV * Q3;
    V* G2 = G1 + NBV * Q3;
    fcontract<V, R, 0, N, N, N, Q, N, false, false, NBV>(su, N3, t1, Q * N2, sB);
    __syncthreads();
    fcontract<V, R, 1, Q, N, N, Q, N, false, false, NBV>(t1, Q * N2, t2, Q2 * N, sB);
    __syncthreads();
    fcontract<V, R, 2, Q, Q, N, Q, N, false, false, NBV>(t2, Q2 * N, U, Q3, sB);
    __syncthreads();
    fcontract<V, R, 0, Q, Q, Q, Q, Q, false, false, NBV>(U, Q3, G0, Q3, sDc);
    fcontract<V, R, 1, Q, Q, Q, Q, Q, false, false, NBV>(U, Q3, G1, Q3, sDc);
    fcontract<V, R, 2, Q, Q, Q, Q, Q, false, false, NBV>(U, Q3, G2, Q3, sDc);
    __syncthreads();
    for (int item = tid; item < CPB * Q3; item += blockDim.x) {
      const int c = item / Q3, r = item - c * Q3;
      const int a = r / Q2, b = (r / Q) % Q, k = r % Q;
      long long cell, cc[3];
      int sub;
      vcell(c, cell, sub);
      coords(cell, cc);
      const R x[3] = {args.lower[0] + (R(cc[0]) + tabs.x[a]) * args.h[0],
                      args.lower[1] + (R(cc[1]) + tabs.x[b]) * args.h[1],
                      args.lower[2] + (R(cc[2]) + tabs.x[k]) * args.h[2]};
      V u[MC], g[MC][3], s[MC], Fl[MC][3];
#pragma unroll
      for (int m = 0; m < MC; ++m) {
        const int idx = (c * MC + m) * Q3 + r;
        u[m] = U[idx];
        g[m][0] = G0[idx] * args.invh[0];
        g[m][1] = G1[idx] * args.invh[1];
        g[m][2] = G2[idx] * args.invh[2];
        s[m] = V(0);
        Fl[m][0] = Fl[m][1] = Fl[m][2] = V(0);
      }
      F::interior(x, u, g, s, Fl);
      const R W = sw[a] * sw[b] * sw[k] * args.detK;
#pragma unroll
      for (int m = 0; m < MC; ++m) {
        const int idx = (c * MC + m) * Q3 + r;
        U[idx] = s[m] * W;
        G0[idx] = Fl[m][0] * (W * args.invh[0]);
        G1[idx] = Fl[m][1] * (W * args.invh[1]);
        G2[idx] = Fl[m][2] * (W * args.invh[2]);
      }
    }
    __syncthreads();
    fcontract<V, R, 0, Q, Q, Q, Q, Q, true, true, NBV>(G0, Q3, U, Q3, sDc);
    __syncthreads();
    fcontract<V, R, 1, Q, Q, Q, Q, Q, true, true, NBV>(G1, Q3, U, Q3, sDc);
    __syncthreads();
    fcontract<V, R, 2, Q, Q, Q, Q, Q, true, true, NBV>(G2, Q3, U, Q3, sDc);
    __syncthreads();
    fcontract<V, R, 2, Q, Q, Q, N, N, true, false, NBV>(U, Q3, t2, Q2 * N, sB);
    __syncthreads();
    fcontract<V, R, 1, Q, Q, N, N, N, true, false, NBV>(t2, Q2 * N, t1, Q * N2, sB);
    __syncthreads();
    fcontract<V, R, 0, Q, N, N, N, N, true, false, NBV>(t1, Q * N2, sr, N3, sB);
    __syncthreads();
  }

  // ---- faces, one normal direction at a time ----------------------------------
#pragma unroll 1
  for (int d = 0; d < 3; ++d) {
    V* FC = work;                   // [CPB][2 s][4][MC][N2]: own value, nbr value, own d/dx_d, nbr d/dx_d
    V* FT = FC + FB * 4 * MC * N2;  // [..][Q][N]
    V* FQ = FT + FB * 4 * MC * Q * N;  // [..][Q][Q]
    V* TD = FQ + FB * 4 * MC * Q2;  // [CPB][2 s][2 t][2 own/nbr][MC][Q2]: tangential derivatives (reference)
    V* OV = TD + FB * 4 * MC * Q2;  // [CPB][2 s][2: value, d/dx_d][MC][Q2]: test coefficients
    V* OT = OV + FB * 2 * MC * Q2;  // [CPB][2 s][2 t][MC][Q2]
    const int t0 = d == 0 ? 1 : 0, t1d = d == 2 ? 1 : 2;  // tangential directions (axis order)
    // traces of the own cell and of the neighbour, coefficient space
    for (int item = tid; item < CPB * 2 * MC * N2; item += blockDim.x) {
      const int c = item / (2 * MC * N2);
      int r = item - c * 2 * MC * N2;
      const int s = r / (MC * N2);
      r -= s * MC * N2;
      const int m = r / N2, jk = r - m * N2;
      const int j = jk / N, k = jk % N;
      long long cell, cc[3];
      int sub;
      const bool ok = vcell(c, cell, sub);
      coords(cell, cc);
      long long nb = cc[d] + (s ? 1 : -1);
      bool has_nb = true;
      if (nb < 0 || nb >= args.nc[d]) {
        if (args.periodic[d]) nb = (nb + args.nc[d]) % args.nc[d];
        else has_nb = false;
      }
      cc[d] = nb;
      const long long ncell = cc[0] + args.nc[0] * (cc[1] + (long long)args.nc[1] * cc[2]);
      int base, stride;
      if (d == 0) { base = j * N + k; stride = N2; }
      else if (d == 1) { base = j * N2 + k; stride = N; }
      else { base = j * N2 + k * N; stride = 1; }
      const V* uo = su + (c * MC + m) * N3;
      V vm = V(0), nm = V(0), vp = V(0), np = V(0);
#pragma unroll
      for (int i = 0; i < N; ++i) {
        const V xv = uo[base + i * stride];
        vm = vfma(str[s * N + i], xv, vm);
        nm = vfma(sdtr[s * N + i], xv, nm);
      }
      if (ok && has_nb) {
        const int so = 1 - s;
#pragma unroll
        for (int i = 0; i < N; ++i) {
          const int ldof = (base + i * stride) * MC + m;
          const R xv = args.u ? args.u[ncell * NLOC + ldof] : R(0);
          R xd = R(0);
          if (mode == 1) xd = args.du[ncell * NLOC + ldof];
          else if (mode == 4) xd = (sub / NLOC == 2 * d + s && sub % NLOC == ldof) ? R(1) : R(0);
          const V xn = Val<V>::make(xv, xd);
          vp = vfma(str[so * N + i], xn, vp);
          np = vfma(sdtr[so * N + i], xn, np);
        }
      }
      V* fc = FC + (c * 2 + s) * 4 * MC * N2 + m * N2 + jk;
      fc[0] = vm;
      fc[MC * N2] = vp;
      fc[2 * MC * N2] = nm * args.invh[d];
      fc[3 * MC * N2] = np * args.invh[d];
    }
    __syncthreads();
    fcontract<V, R, 1, 1, N, N, Q, N, false, false, FB * 4 * MC>(FC, N2, FT, Q * N, sB);
    __syncthreads();
    fcontract<V, R, 2, 1, Q, N, Q, N, false, false, FB * 4 * MC>(FT, Q * N, FQ, Q2, sB);
    __syncthreads();
    // tangential derivatives of the two value arrays (own, neighbour)
    fcontract<V, R, 1, 2 * MC, Q, Q, Q, Q, false, false, FB>(FQ, 4 * MC * Q2, TD, 4 * MC * Q2, sDc);
    fcontract<V, R, 2, 2 * MC, Q, Q, Q, Q, false, false, FB>(FQ, 4 * MC * Q2, TD + 2 * MC * Q2, 4 * MC * Q2, sDc);
    __syncthreads();
    // pointwise face terms
    for (int item = tid; item < CPB * 2 * Q2; item += blockDim.x) {
      const int c = item / (2 * Q2);
      const int r = item - c * 2 * Q2;
      const int s = r / Q2, ab = r - s * Q2;
      const int a = ab / Q, b = ab % Q;
      long long cell, cc[3];
      int sub;
      vcell(c, cell, sub);
      coords(cell, cc);
      const bool boundary = !args.periodic[d] && (s ? cc[d] == args.nc[d] - 1 : cc[d] == 0);
      R x[3], n[3] = {R(0), R(0), R(0)};
      x[d] = args.lower[d] + R(cc[d] + s) * args.h[d];
      x[t0] = args.lower[t0] + (R(cc[t0]) + tabs.x[a]) * args.h[t0];
      x[t1d] = args.lower[t1d] + (R(cc[t1d]) + tabs.x[b]) * args.h[t1d];
      n[d] = s ? R(1) : R(-1);
      const V* fq = FQ + (c * 2 + s) * 4 * MC * Q2 + ab;
      const V* td = TD + (c * 2 + s) * 4 * MC * Q2 + ab;
      V uL[MC], gL[MC][3], uR[MC], gR[MC][3], sv[MC], Fl[MC][3];
#pragma unroll
      for (int m = 0; m < MC; ++m) {
        uL[m] = fq[m * Q2];
        uR[m] = fq[(MC + m) * Q2];
        gL[m][d] = fq[(2 * MC + m) * Q2];
        gR[m][d] = fq[(3 * MC + m) * Q2];
        gL[m][t0] = td[m * Q2] * args.invh[t0];
        gR[m][t0] = td[(MC + m) * Q2] * args.invh[t0];
        gL[m][t1d] = td[(2 * MC + m) * Q2] * args.invh[t1d];
        gR[m][t1d] = td[(3 * MC + m) * Q2] * args.invh[t1d];
        sv[m] = V(0);
        Fl[m][0] = Fl[m][1] = Fl[m][2] = V(0);
      }
      if (boundary) F::boundary(x, n, args.sigma[d], uL, gL, sv, Fl);
      else F::skeleton(x, n, args.sigma[d], uL, gL, uR, gR, sv, Fl);
      const R W = sw[a] * sw[b] * args.faceA[d];
      V* ov = OV + (c * 2 + s) * 2 * MC * Q2 + ab;
      V* ot = OT + (c * 2 + s) * 2 * MC * Q2 + ab;
#pragma unroll
      for (int m = 0; m < MC; ++m) {
        ov[m * Q2] = sv[m] * W;
        ov[(MC + m) * Q2] = Fl[m][d] * (W * args.invh[d]);
        ot[m * Q2] = Fl[m][t0] * (W * args.invh[t0]);
        ot[(MC + m) * Q2] = Fl[m][t1d] * (W * args.invh[t1d]);
      }
    }
    __syncthreads();
    // tangential test derivatives into the value part (transposed collocation derivative)
    fcontract<V, R, 1, MC, Q, Q, Q, Q, true, true, FB>(OT, 2 * MC * Q2, OV, 2 * MC * Q2, sDc);
    __syncthreads();
    fcontract<V, R, 2, MC, Q, Q, Q, Q, true, true, FB>(OT + MC * Q2, 2 * MC * Q2, OV, 2 * MC * Q2, sDc);
    __syncthreads();
    // back to tangential coefficients
    fcontract<V, R, 2, 1, Q, Q, N, N, true, false, FB * 2 * MC>(OV, Q2, FT, Q * N, sB);
    __syncthreads();
    fcontract<V, R, 1, 1, Q, N, N, N, true, false, FB * 2 * MC>(FT, Q * N, FC, N2, sB);
    __syncthreads();
    // expand into the cell's test functions, both sides in fixed order
    for (int item = tid; item < CPB * NLOC; item += blockDim.x) {
      const int c = item / NLOC;
      const int r = item - c * NLOC;
      const int m = r / N3, l = r - m * N3;
      const int i0 = l / N2, i1 = (l / N) % N, i2 = l % N;
      int i, jk;
      if (d == 0) { i = i0; jk = i1 * N + i2; }
      else if (d == 1) { i = i1; jk = i0 * N + i2; }
      else { i = i2; jk = i0 * N + i1; }
      V acc = sr[item];
#pragma unroll
      for (int s = 0; s < 2; ++s) {
        const V* fc = FC + (c * 2 + s) * 2 * MC * N2;
        acc = vfma(str[s * N + i], fc[m * N2 + jk], acc);
        acc = vfma(sdtr[s * N + i], fc[(MC + m) * N2 + jk], acc);
      }
      sr[item] = acc;
    }
    __syncthreads();
  }

  // ---- store -------------------------------------------------------------------
  for (int e = tid; e < CPB * NLOC; e += blockDim.x) {
    const int c = e / NLOC, r = e - c * NLOC;
    const int m = r / N3, i = r - m * N3;
    long long cell;
    int sub;
    if (!vcell(c, cell, sub)) continue;
    const int row = i * MC + m;
    const R val = Val<V>::out(sr[e]);
    if (mode <= 1) {
      args.w[cell * NLOC + row] = val;
    } else if (mode == 2) {
      args.blocks[((cell - args.cell_begin) * NLOC + row) * NLOC + sub] = val;
    } else if (mode == 3) {
      if (row == sub) args.blocks[cell * NLOC + sub] = val;
    } else {
      const int f = sub / NLOC, j = sub - f * NLOC;
      args.blocks[(((cell - args.cell_begin) * 7 + 1 + f) * NLOC + row) * NLOC + j] = val;
    }
  }
}

// ---- the interior-penalty form of a flux, a source and a convective flux ------
// U (generated from the user's pieces) provides, generic in the value type D:
//   flux(x, u, g, F)      diffusive flux F[m][k] (the form has int F:grad v)
//   source(x, u, g, s)    s[m] (int s.v)
//   advection(x, u, Fa)   convective flux (int -Fa:grad v + numerical flux)
//   wavespeed(x, u, n)    bound of |dFa/du . n| for the Lax-Friedrichs flux
//   dirichlet(x, gD)      boundary values (weak, by the same terms)
// and the flags kFlux, kSource, kAdvection, kDirichlet.  THETA = 1 is the
// symmetric interior penalty form (the reference's SIPG, schemes/
// integrands.hh:838-877, and the UFL form of pydemo/advectiondiffusion.py:
// 33-55 for a nonlinear flux):
//   int_F  sigma [u][v] - {F(u, grad u)}.n [v] - THETA [u] {A^T n}.grad v
// with A = dF/d(grad u) (for F = kappa(u) grad u, A^T n = kappa(u) n), and the
// local Lax-Friedrichs flux 1/2 (Fa(uL) + Fa(uR)).n + 1/2 lambda [u] for the
// convective part (the upwind flux for a linear Fa).  A^T n comes from dual
// numbers over the gradient, nested inside the linearisation's.
template <class U, int THETA>
struct Sipg {
  static constexpr int M = U::M;

  // F[m][k] += coef * sum_{m', j} jump[m'] n_j dF_{m'j}/dg_{mk} at (u, g)
  template <class D, class R>
  __device__ static void flux_transpose(const R* x, const D* u, D (*g)[3], const D* jump, const R* n, R coef,
                                        D (*F)[3]) {
#pragma unroll 1
    for (int mm = 0; mm < M; ++mm)
#pragma unroll 1
      for (int kk = 0; kk < 3; ++kk) {
        Dual<D> u2[M], g2[M][3], F2[M][3];
#pragma unroll
        for (int m = 0; m < M; ++m) {
          u2[m] = Dual<D>(u[m]);
#pragma unroll
          for (int k = 0; k < 3; ++k) {
            g2[m][k] = Dual<D>(g[m][k], D((m == mm && k == kk) ? 1 : 0));
            F2[m][k] = Dual<D>(D(0));
          }
        }
        U::flux(x, u2, g2, F2);
        D acc = D(0);
#pragma unroll
        for (int m = 0; m < M; ++m)
#pragma unroll
          for (int k = 0; k < 3; ++k) acc = acc + jump[m] * (F2[m][k].d * n[k]);
        F[mm][kk] = F[mm][kk] + acc * coef;
      }
  }

  template <class D, class R>
  __device__ static void interior(const R* x, const D* u, D (*g)[3], D* s, D (*F)[3]) {
    if (U::kFlux) U::flux(x, u, g, F);
    if (U::kSource) U::source(x, u, g, s);
    if (U::kAdvection) {
      D Fa[M][3];
#pragma unroll
      for (int m = 0; m < M; ++m) Fa[m][0] = Fa[m][1] = Fa[m][2] = D(0);
      U::advection(x, u, Fa);
#pragma unroll
      for (int m = 0; m < M; ++m)
#pragma unroll
        for (int k = 0; k < 3; ++k) F[m][k] = F[m][k] - Fa[m][k];
    }
  }

  template <class D, class R>
  __device__ static void lax_friedrichs(const R* x, const R* n, const D* uL, const D* uR, D* s) {
    D FaL[M][3], FaR[M][3];
#pragma unroll
    for (int m = 0; m < M; ++m)
#pragma unroll
      for (int k = 0; k < 3; ++k) FaL[m][k] = FaR[m][k] = D(0);
    U::advection(x, uL, FaL);
    U::advection(x, uR, FaR);
    const D lam = max(U::wavespeed(x, uL, n), U::wavespeed(x, uR, n));
#pragma unroll
    for (int m = 0; m < M; ++m) {
      D fn = D(0);
#pragma unroll
      for (int k = 0; k < 3; ++k) fn = fn + (FaL[m][k] + FaR[m][k]) * n[k];
      s[m] = s[m] + (fn + lam * (uL[m] - uR[m])) * R(0.5);
    }
  }

  template <class D, class R>
  __device__ static void skeleton(const R* x, const R* n, R sigma, const D* uL, D (*gL)[3], const D* uR,
                                  D (*gR)[3], D* s, D (*F)[3]) {
    if (U::kFlux) {
      D jump[M], FL[M][3], FR[M][3];
#pragma unroll
      for (int m = 0; m < M; ++m) {
        jump[m] = uL[m] - uR[m];
#pragma unroll
        for (int k = 0; k < 3; ++k) FL[m][k] = FR[m][k] = D(0);
      }
      U::flux(x, uL, gL, FL);
      U::flux(x, uR, gR, FR);
#pragma unroll
      for (int m = 0; m < M; ++m) {
        D fn = D(0);
#pragma unroll
        for (int k = 0; k < 3; ++k) fn = fn + (FL[m][k] + FR[m][k]) * n[k];
        s[m] = s[m] + jump[m] * sigma - fn * R(0.5);
      }
      if (THETA != 0) flux_transpose(x, uL, gL, jump, n, R(-0.5 * THETA), F);
    }
    if (U::kAdvection) lax_friedrichs(x, n, uL, uR, s);
  }

  template <class D, class R>
  __device__ static void boundary(const R* x, const R* n, R sigma, const D* u, D (*g)[3], D* s, D (*F)[3]) {
    if (U::kDirichlet) {
      R gd[M];
#pragma unroll
      for (int m = 0; m < M; ++m) gd[m] = R(0);
      U::dirichlet(x, gd);
      D ub[M], jump[M];
#pragma unroll
      for (int m = 0; m < M; ++m) {
        ub[m] = D(gd[m]);
        jump[m] = u[m] - gd[m];
      }
      if (U::kFlux) {
        D Fu[M][3];
#pragma unroll
        for (int m = 0; m < M; ++m) Fu[m][0] = Fu[m][1] = Fu[m][2] = D(0);
        U::flux(x, u, g, Fu);
#pragma unroll
        for (int m = 0; m < M; ++m) {
          D fn = D(0);
#pragma unroll
          for (int k = 0; k < 3; ++k) fn = fn + Fu[m][k] * n[k];
          s[m] = s[m] + jump[m] * sigma - fn;
        }
        if (THETA != 0) flux_transpose(x, u, g, jump, n, R(-THETA), F);
      }
      if (U::kAdvection) lax_friedrichs(x, n, u, ub, s);
    } else if (U::kAdvection) {
      // natural boundary: zero diffusive flux, the convective flux of the inner state
      D Fa[M][3];
#pragma unroll
      for (int m = 0; m < M; ++m) Fa[m][0] = Fa[m][1] = Fa[m][2] = D(0);
      U::advection(x, u, Fa);
#pragma unroll
      for (int m = 0; m < M; ++m) {
        D fn = D(0);
#pragma unroll
        for (int k = 0; k < 3; ++k) fn = fn + Fa[m][k] * n[k];
        s[m] = s[m] + fn;
      }
    }
  }
};

}  // namespace form
}  // namespace gbfem
