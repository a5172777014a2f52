// Sum-factorised matrix-free apply of the SIPG / upwind / mass DG operator on
// a structured Cartesian hexahedral grid with a tensor Legendre Q_p basis.
//
// What it computes is dune-fem's Impl::GalerkinOperator::evaluateImpl
// (schemes/galerkin.hh:811-917) with the DG integrands of the UFL form in
// pydemo/advectiondiffusion.py:33-55 (the interior part of
// schemes/integrands.hh:748-967 for the flux kappa*grad u):
//
//   w_i =  sum_K  int_K  eps*kappa grad u . grad phi_i - u b . grad phi_i + c u phi_i
//        + sum_F  int_F  eps*( sigma*avg(kappa) [u][phi_i] - {kappa grad u}.n [phi_i]
//                              - [u] {kappa grad phi_i}.n )  +  (b.n) u_upwind [phi_i]
//        + sum_dK int_F  eps*( sigma*kappa u phi_i - kappa du/dn phi_i - u kappa dphi_i/dn )
//                        + max(b.n,0) u phi_i                       (weak u = 0)
//
// with sigma = beta / h_F, h_F = avg|K| / |F|.
//
// How (GB300 design, not the reference's): one CTA owns CPB consecutive
// cells.  All per-cell work happens in shared memory in three phases.
//  1. Volume: u -> values at the q^3 Gauss points by three 1-D contractions
//     with B (q x n); gradients by the q x q collocation derivative matrix;
//     pointwise flux; the transposed chain back to the n^3 test functions.
//  2. Faces, owner-computes: each cell evaluates all six of its faces
//     itself, reading the neighbour's trace from global memory (L2-resident).
//     Each face is therefore computed twice, once per side.  In exchange there
//     is no scatter to a neighbour, no atomics and no lock (the reference
//     takes a shared_mutex, schemes/galerkin.hh:963-991), and the result is
//     bitwise independent of launch configuration.
//  3. One coalesced store of w.
// Every output value is produced by one thread with a fixed summation order,
// so the apply is deterministic.
#pragma once
#include <cuda_runtime.h>
#include <cstdint>

namespace gbfem {

constexpr int kDgMaxN = 5;
constexpr int kDgMaxQ = 7;

// Device tables in the kernel's precision (kernel parameter, copied to smem).
template <typename T>
struct DgTablesT {
  T B[kDgMaxQ * kDgMaxN];   // B[a*n+i]  = L_i(x_a)
  T Dc[kDgMaxQ * kDgMaxQ];  // Dc[a*q+b] = l_b'(x_a)
  T w[kDgMaxQ];             // Gauss weights on [0,1]
  T x[kDgMaxQ];             // Gauss points on [0,1]
  T tr[2 * kDgMaxN];        // tr[s*n+i]  = L_i(s)
  T dtr[2 * kDgMaxN];       // dtr[s*n+i] = L_i'(s)
};

template <typename T>
struct DgArgsT {
  const T* u;
  T* w;
  const T* kappa;     // DG coefficients of kappa (the source of kq, kf)
  const T* kq;        // KAPPA: kappa at the volume Gauss points [cell][a][b][c]
  const T* kf;        // KAPPA: kappa at the face Gauss points [cell][face 2d+s][a][b] (own side)
  const T* kcell;     // closed form with a constant kappa per cell: [cell]
  int nc[3];          // cells per direction
  int periodic[3];
  long long ncells;
  T detK;             // |K|
  T invh[3];          // 1/h_d
  T faceA[3];         // |F| of a face normal to d
  T sigma[3];         // beta / h_F for faces normal to d
  T eps;              // diffusion coefficient
  T mass;             // mass coefficient
  T b[3];             // advection velocity
  int advect;         // b != 0
  int weak_dirichlet; // Nitsche u = 0 on non-periodic boundary faces
  int unit_mode;      // 1: block-diagonal assembly (own dofs = e_j, neighbour u = 0); 2: diagonal only;
                      // 3: neighbour couplings (own u = 0, the neighbour through face f holds e_j)
  T* blocks;          // unit_mode 1 output blocks[cell - cell_begin][i][j]; unit_mode 2 output diag[cell][j]
  long long cell_begin;  // unit_mode 1: first cell of the batch
  long long cell_count;  // unit_mode 1: cells in the batch (0 = all)
};

// Contraction of NCELL arrays `in` (dims [I0][I1][I2], row-major, cell
// stride ics) along axis AX with the matrix M into `out` (same dims except
// OUT on axis AX, cell stride ocs):
//   !TR: out[..o..] = sum_i M[o*LDM + i] in[..i..];  TR: M[i*LDM + o];
//   ACC adds to the existing content of out.
// One thread owns a whole line along axis AX, keeps its
// IN inputs in registers and writes all OUT outputs.  M is warp-uniform (the
// same entry for every thread at each unrolled step), read from the kernel's
// parameter space, so a contraction costs IN + OUT shared-memory accesses per
// IN*OUT FMAs instead of two per FMA.  Same fixed summation order per output
// as `contract`.
template <typename T, int AX, int I0, int I1, int I2, int OUT, int LDM, bool TR, bool ACC, int NCELL>
__device__ __forceinline__ void contract_lines(const T* __restrict__ in, int ics, T* __restrict__ out, int ocs,
                                               const T* __restrict__ M) {
  constexpr int IN = AX == 0 ? I0 : (AX == 1 ? I1 : I2);
  constexpr int O0 = AX == 0 ? OUT : I0;
  constexpr int O1 = AX == 1 ? OUT : I1;
  constexpr int O2 = AX == 2 ? OUT : I2;
  // the two axes that are not contracted, in order
  constexpr int PA = AX == 0 ? 1 : 0, PB = AX == 2 ? 1 : 2;
  constexpr int DI[3] = {I0, I1, I2};
  constexpr int SI[3] = {I1 * I2, I2, 1};
  constexpr int SO[3] = {O1 * O2, O2, 1};
  constexpr int NA = DI[PA], NB = DI[PB];
  constexpr int LINES = NA * NB;
  for (int item = threadIdx.x; item < NCELL * LINES; item += blockDim.x) {
    const int cell = item / LINES;
    const int ln = item - cell * LINES;
    const int xa = ln / NB, xb = ln - xa * NB;
    const T* src = in + cell * ics + xa * SI[PA] + xb * SI[PB];
    T* dst = out + cell * ocs + xa * SO[PA] + xb * SO[PB];
    T x[IN];
#pragma unroll
    for (int i = 0; i < IN; ++i) x[i] = src[i * SI[AX]];
#pragma unroll
    for (int o = 0; o < OUT; ++o) {
      T acc = ACC ? dst[o * SO[AX]] : T(0);
#pragma unroll
      for (int i = 0; i < IN; ++i) acc = fma(TR ? M[i * LDM + o] : M[o * LDM + i], x[i], acc);
      dst[o * SO[AX]] = acc;
    }
  }
}

// Per-output variant of the same contraction: one thread per output value,
// matrix from shared memory.  The FP64 kernels use it: they are FP64-pipe
// bound, and this form issues fewer instructions per FMA than the line form.
// in  : NCELL arrays of dims [I0][I1][I2] (row-major), cell stride `ics`.
// out : NCELL arrays of the same dims except OUT on axis AX, cell stride `ocs`.
// !TR : out[..o..] = sum_i M[o*LDM + i] * in[..i..]
//  TR : out[..o..] = sum_i M[i*LDM + o] * in[..i..]
// ACC adds to the existing content of out.
template <typename T, int AX, int I0, int I1, int I2, int OUT, int LDM, bool TR, bool ACC, int NCELL>
__device__ __forceinline__ void contract_items(const T* __restrict__ in, int ics, T* __restrict__ out, int ocs,
                                         const T* __restrict__ M) {
  constexpr int IN = AX == 0 ? I0 : (AX == 1 ? I1 : I2);
  constexpr int O0 = AX == 0 ? OUT : I0;
  constexpr int O1 = AX == 1 ? OUT : I1;
  constexpr int O2 = AX == 2 ? OUT : I2;
  constexpr int OSZ = O0 * O1 * O2;
  constexpr int IS0 = I1 * I2, IS1 = I2;
  constexpr int ISA = AX == 0 ? IS0 : (AX == 1 ? IS1 : 1);
  for (int item = threadIdx.x; item < NCELL * OSZ; item += blockDim.x) {
    const int cell = item / OSZ;
    const int r = item - cell * OSZ;
    const int x0 = r / (O1 * O2);
    const int x1 = (r / O2) % O1;
    const int x2 = r % O2;
    const int o = AX == 0 ? x0 : (AX == 1 ? x1 : x2);
    const int ib = cell * ics + (AX == 0 ? 0 : x0 * IS0) + (AX == 1 ? 0 : x1 * IS1) + (AX == 2 ? 0 : x2);
    T acc = ACC ? out[cell * ocs + r] : T(0);
#pragma unroll
    for (int i = 0; i < IN; ++i) {
      const T m = TR ? M[i * LDM + o] : M[o * LDM + i];
      acc = fma(m, in[ib + i * ISA], acc);
    }
    out[cell * ocs + r] = acc;
  }
}

// Contraction with the form that suits the precision: lines (register
// inputs, warp-uniform parameter-space matrix) for FP32, which would
// otherwise be bound by shared-memory bandwidth; per-output items for FP64.
template <typename T, int AX, int I0, int I1, int I2, int OUT, int LDM, bool TR, bool ACC, int NCELL>
__device__ __forceinline__ void contract(const T* __restrict__ in, int ics, T* __restrict__ out, int ocs,
                                         const T* __restrict__ Msmem, const T* __restrict__ Mparam) {
  if (sizeof(T) == 8)
    contract_items<T, AX, I0, I1, I2, OUT, LDM, TR, ACC, NCELL>(in, ics, out, ocs, Msmem);
  else
    contract_lines<T, AX, I0, I1, I2, OUT, LDM, TR, ACC, NCELL>(in, ics, out, ocs, Mparam);
}

// Shared-memory footprint (elements of T) of one CTA.
template <int N, int Q, bool KAPPA, int CPB>
struct DgSmem {
  static constexpr int N3 = N * N * N, Q3 = Q * Q * Q, N2 = N * N, Q2 = Q * Q;
  static constexpr int MA = 4;  // face arrays: v-, v+, dn-, dn+ (kappa comes from the point cache)
  static constexpr int VOL = Q * N2 + Q2 * N + Q3 * 4;
  static constexpr int FACE = 2 * MA * (N2 + Q * N + Q2) + 4 * Q2;
  static constexpr int WORK = VOL > FACE ? VOL : FACE;
  static constexpr int TAB = kDgMaxQ * kDgMaxN + kDgMaxQ * kDgMaxQ + kDgMaxQ + 4 * kDgMaxN;
  static constexpr int PER_CELL = N3 * 2 + WORK;
  static constexpr int TOTAL = TAB + CPB * PER_CELL;
};

template <typename T, int N, int Q, bool KAPPA, int CPB>
__global__ void __launch_bounds__(256) dg_apply_kernel(const DgArgsT<T> args,
                                                       const __grid_constant__ DgTablesT<T> tabs) {
  using S = DgSmem<N, Q, KAPPA, CPB>;
  constexpr int N3 = S::N3, Q3 = S::Q3, N2 = S::N2, Q2 = S::Q2, MA = S::MA;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T* sm = reinterpret_cast<T*>(smem_raw);
  T* sB = sm;
  T* sDc = sB + kDgMaxQ * kDgMaxN;
  T* sw = sDc + kDgMaxQ * kDgMaxQ;
  T* str = sw + kDgMaxQ;
  T* sdtr = str + 2 * kDgMaxN;
  T* su = sm + S::TAB;                 // [CPB][N3]
  T* sr = su + CPB * N3;               // [CPB][N3]
  T* work = sr + CPB * N3;             // [CPB][WORK]
  constexpr int WS = S::WORK;

  const int tid = threadIdx.x;
  // tables -> smem
  for (int i = tid; i < Q * N; i += blockDim.x) sB[i] = tabs.B[i];
  for (int i = tid; i < Q * Q; i += blockDim.x) sDc[i] = tabs.Dc[i];
  for (int i = tid; i < Q; i += blockDim.x) sw[i] = tabs.w[i];
  for (int i = tid; i < 2 * N; i += blockDim.x) { str[i] = tabs.tr[i]; sdtr[i] = tabs.dtr[i]; }

  const long long ncells = args.ncells;
  // Cells [cell_begin, cell_begin + cell_count) (cell_count 0 = all).  In
  // unit mode the "virtual cells" are (cell, j) pairs: vcell = cell*N3 + j;
  // unit mode 3: (cell, f, j) = (cell*6 + f)*N3 + j.
  const long long ucount = args.cell_count > 0 ? args.cell_count : ncells;
  const int vper = args.unit_mode == 3 ? 6 * N3 : (args.unit_mode ? N3 : 1);
  const long long nvirt = (args.cell_begin + ucount) * vper;
  const long long v0 = (long long)blockIdx.x * CPB + args.cell_begin * vper;
  if (v0 >= nvirt) return;

  // ---- load own dofs --------------------------------------------------------
  for (int e = tid; e < CPB * N3; e += blockDim.x) {
    const int c = e / N3, i = e - c * N3;
    const long long v = v0 + c;
    T val = T(0);
    if (v < nvirt) {
      if (args.unit_mode) {
        const long long cell = v / vper;
        val = (args.unit_mode != 3 && i == int(v - cell * N3)) ? T(1) : T(0);
      } else {
        val = __ldg(args.u + v * N3 + i);
      }
    }
    su[e] = val;
  }
  __syncthreads();

  // ---- phase 1: volume ----------------------------------------------------
  {
    T* t1 = work;                 // [Q][N][N]
    T* t2 = t1 + Q * N2;          // [Q][Q][N]
    T* U = t2 + Q2 * N;           // [Q3]
    T* G0 = U + Q3;
    T* G1 = G0 + Q3;
    T* G2 = G1 + Q3;
    contract<T, 0, N, N, N, Q, N, false, false, CPB>(su, N3, t1, WS, sB, tabs.B);
    __syncthreads();
    contract<T, 1, Q, N, N, Q, N, false, false, CPB>(t1, WS, t2, WS, sB, tabs.B);
    __syncthreads();
    contract<T, 2, Q, Q, N, Q, N, false, false, CPB>(t2, WS, U, WS, sB, tabs.B);
    __syncthreads();
    // gradients in reference coordinates: collocation derivative along each axis
    contract<T, 0, Q, Q, Q, Q, Q, false, false, CPB>(U, WS, G0, WS, sDc, tabs.Dc);
    contract<T, 1, Q, Q, Q, Q, Q, false, false, CPB>(U, WS, G1, WS, sDc, tabs.Dc);
    contract<T, 2, Q, Q, Q, Q, Q, false, false, CPB>(U, WS, G2, WS, sDc, tabs.Dc);
    __syncthreads();
    // pointwise flux (in place: item r reads and writes only point r)
    for (int item = tid; item < CPB * Q3; item += blockDim.x) {
      const int c = item / Q3, r = item - c * Q3;
      const int a = r / Q2, b = (r / Q) % Q, cc = r % Q;
      const T uq = U[c * WS + r];
      T kq = T(1);
      if (KAPPA) {
        const long long v = v0 + c;
        const long long cell = v < nvirt ? (args.unit_mode ? v / vper : v) : 0;
        kq = __ldg(args.kq + cell * Q3 + r);
      }
      const T W = sw[a] * sw[b] * sw[cc] * args.detK;
      const T ek = args.eps * kq;
      // flux F = eps*kappa*grad u - b*u (physical), tested with grad phi = invh * ref-grad
      T f0 = ek * G0[c * WS + r] * args.invh[0];
      T f1 = ek * G1[c * WS + r] * args.invh[1];
      T f2 = ek * G2[c * WS + r] * args.invh[2];
      if (args.advect) {
        f0 -= args.b[0] * uq;
        f1 -= args.b[1] * uq;
        f2 -= args.b[2] * uq;
      }
      G0[c * WS + r] = W * f0 * args.invh[0];
      G1[c * WS + r] = W * f1 * args.invh[1];
      G2[c * WS + r] = W * f2 * args.invh[2];
      U[c * WS + r] = W * args.mass * uq;
    }
    __syncthreads();
    // V = W c u + Dc^T contractions of the fluxes, accumulated axis by axis
    contract<T, 0, Q, Q, Q, Q, Q, true, true, CPB>(G0, WS, U, WS, sDc, tabs.Dc);
    __syncthreads();
    contract<T, 1, Q, Q, Q, Q, Q, true, true, CPB>(G1, WS, U, WS, sDc, tabs.Dc);
    __syncthreads();
    contract<T, 2, Q, Q, Q, Q, Q, true, true, CPB>(G2, WS, U, WS, sDc, tabs.Dc);
    __syncthreads();
    contract<T, 2, Q, Q, Q, N, N, true, false, CPB>(U, WS, t2, WS, sB, tabs.B);
    __syncthreads();
    contract<T, 1, Q, Q, N, N, N, true, false, CPB>(t2, WS, t1, WS, sB, tabs.B);
    __syncthreads();
    contract<T, 0, Q, N, N, N, N, true, false, CPB>(t1, WS, sr, N3, sB, tabs.B);
    __syncthreads();
  }

  // ---- phase 2: faces, one normal direction at a time -----------------------
#pragma unroll 1
  for (int d = 0; d < 3; ++d) {
    T* FC = work;                      // [2][MA][N][N]
    T* FT = FC + 2 * MA * N2;          // [2][MA][Q][N]
    T* FQ = FT + 2 * MA * Q * N;       // [2][MA][Q][Q]
    T* FV = FQ + 2 * MA * Q2;          // [2][2][Q][Q]
    const T invh = args.invh[d];
    // F1: traces in coefficient space
    for (int item = tid; item < CPB * 2 * N2; item += blockDim.x) {
      const int c = item / (2 * N2);
      const int r = item - c * 2 * N2;
      const int s = r / N2;
      const int jk = r - s * N2;
      const int j = jk / N, k = jk % N;
      const T sgn = s ? T(1) : T(-1);
      const long long v = v0 + c;
      long long cell = args.unit_mode ? v / vper : v;
      bool valid = v < nvirt;
      if (!valid) cell = 0;
      // unit mode 3: the face whose neighbour carries e_j, and j
      const int uf = args.unit_mode == 3 && valid ? int((v - cell * vper) / N3) : -1;
      const int uj = args.unit_mode == 3 && valid ? int(v - cell * vper - uf * N3) : -1;
      long long cz = cell / ((long long)args.nc[0] * args.nc[1]);
      long long rem = cell - cz * (long long)args.nc[0] * args.nc[1];
      long long cy = rem / args.nc[0];
      long long cx = rem - cy * args.nc[0];
      long long cc[3] = {cx, cy, cz};
      long long nb = cc[d] + (s ? 1 : -1);
      bool has_nb = true;
      if (nb < 0 || nb >= args.nc[d]) {
        if (args.periodic[d]) nb = (nb + args.nc[d]) % args.nc[d];
        else has_nb = false;
      }
      long long ncoord[3] = {cx, cy, cz};
      ncoord[d] = nb;
      const long long ncell = ncoord[0] + (long long)args.nc[0] * (ncoord[1] + (long long)args.nc[1] * ncoord[2]);
      // dof index of (normal index i, tangential j,k)
      int base, stride;
      if (d == 0) { base = j * N + k; stride = N2; }
      else if (d == 1) { base = j * N2 + k; stride = N; }
      else { base = j * N2 + k * N; stride = 1; }
      const T* uo = su + c * N3;
      T vm = T(0), nm = T(0), vp = T(0), np = T(0);
#pragma unroll
      for (int i = 0; i < N; ++i) {
        const T x = uo[base + i * stride];
        vm = fma(str[s * N + i], x, vm);
        nm = fma(sdtr[s * N + i], x, nm);
      }
      if (has_nb && valid) {
        const int so = 1 - s;
#pragma unroll
        for (int i = 0; i < N; ++i) {
          const T x = args.unit_mode == 3 ? ((uf == 2 * d + s && base + i * stride == uj) ? T(1) : T(0))
                      : args.unit_mode ? T(0) : __ldg(args.u + ncell * N3 + base + i * stride);
          vp = fma(str[so * N + i], x, vp);
          np = fma(sdtr[so * N + i], x, np);
        }
      }
      T* fc = FC + c * WS + s * MA * N2;
      fc[0 * N2 + jk] = vm;
      fc[1 * N2 + jk] = vp;
      fc[2 * N2 + jk] = sgn * invh * nm;
      fc[3 * N2 + jk] = sgn * invh * np;
    }
    __syncthreads();
    // F2/F3: 2-D interpolation of all face arrays to the q x q face points
    contract<T, 1, 2 * MA, N, N, Q, N, false, false, CPB>(FC, WS, FT, WS, sB, tabs.B);
    __syncthreads();
    contract<T, 2, 2 * MA, Q, N, Q, N, false, false, CPB>(FT, WS, FQ, WS, sB, tabs.B);
    __syncthreads();
    // F4: pointwise numerical fluxes
    for (int item = tid; item < CPB * 2 * Q2; item += blockDim.x) {
      const int c = item / (2 * Q2);
      const int r = item - c * 2 * Q2;
      const int s = r / Q2;
      const int ab = r - s * Q2;
      const int a = ab / Q, b = ab % Q;
      const long long v = v0 + c;
      long long cell = args.unit_mode ? v / vper : v;
      if (v >= nvirt) cell = 0;
      long long cz = cell / ((long long)args.nc[0] * args.nc[1]);
      long long rem = cell - cz * (long long)args.nc[0] * args.nc[1];
      long long cy = rem / args.nc[0];
      long long cx = rem - cy * args.nc[0];
      const long long cd = d == 0 ? cx : (d == 1 ? cy : cz);
      const bool boundary = !args.periodic[d] && (s ? (cd == args.nc[d] - 1) : (cd == 0));
      const T* fq = FQ + c * WS + s * MA * Q2;
      const T vm = fq[0 * Q2 + ab], vp = fq[1 * Q2 + ab];
      const T nm = fq[2 * Q2 + ab], np = fq[3 * Q2 + ab];
      T km = T(1), kp = T(1);
      if (KAPPA) {
        // own side from this cell's face cache, the other side from the
        // neighbour's cache of the same face (its face 2d+1-s)
        km = __ldg(args.kf + (cell * 6 + 2 * d + s) * Q2 + ab);
        if (!boundary) {
          long long cc3[3] = {cx, cy, cz};
          long long nb = cc3[d] + (s ? 1 : -1);
          if (nb < 0 || nb >= args.nc[d]) nb = (nb + args.nc[d]) % args.nc[d];
          cc3[d] = nb;
          const long long ncell = cc3[0] + (long long)args.nc[0] * (cc3[1] + (long long)args.nc[1] * cc3[2]);
          kp = __ldg(args.kf + (ncell * 6 + 2 * d + 1 - s) * Q2 + ab);
        }
      }
      const T W = sw[a] * sw[b] * args.faceA[d];
      const T bn = args.advect ? (s ? args.b[d] : -args.b[d]) : T(0);
      T val = T(0), grad = T(0);
      if (!boundary) {
        const T J = vm - vp;
        const T kbar = T(0.5) * (km + kp);
        const T avgflux = T(0.5) * (km * nm + kp * np);
        val = W * args.eps * (args.sigma[d] * kbar * J - avgflux);
        grad = W * args.eps * (T(-0.5) * km * J);
        if (args.advect) val += W * bn * (bn >= T(0) ? vm : vp);
      } else {
        if (args.weak_dirichlet) {
          val = W * args.eps * (args.sigma[d] * km * vm - km * nm);
          grad = W * args.eps * (-km * vm);
        }
        if (args.advect && bn > T(0)) val += W * bn * vm;
      }
      T* fv = FV + c * WS + s * 2 * Q2;
      fv[ab] = val;
      fv[Q2 + ab] = grad;
    }
    __syncthreads();
    // F5/F6: transposed 2-D contraction back to the n x n tangential coefficients
    contract<T, 2, 4, Q, Q, N, N, true, false, CPB>(FV, WS, FT, WS, sB, tabs.B);
    __syncthreads();
    contract<T, 1, 4, Q, N, N, N, true, false, CPB>(FT, WS, FC, WS, sB, tabs.B);
    __syncthreads();
    // F7: expand into the cell's test functions, both sides in fixed order
    for (int item = tid; item < CPB * N3; item += blockDim.x) {
      const int c = item / N3, l = item - c * N3;
      const int i0 = l / N2, i1 = (l / N) % N, i2 = l % N;
      int i, jk;
      if (d == 0) { i = i0; jk = i1 * N + i2; }
      else if (d == 1) { i = i1; jk = i0 * N + i2; }
      else { i = i2; jk = i0 * N + i1; }
      const T* fc = FC + c * WS;
      T acc = sr[item];
#pragma unroll
      for (int s = 0; s < 2; ++s) {
        const T sgn = s ? T(1) : T(-1);
        acc = fma(str[s * N + i], fc[(2 * s) * N2 + jk], acc);
        acc = fma(sgn * invh * sdtr[s * N + i], fc[(2 * s + 1) * N2 + jk], acc);
      }
      sr[item] = acc;
    }
    __syncthreads();
  }

  // ---- phase 3: store -------------------------------------------------------
  for (int e = tid; e < CPB * N3; e += blockDim.x) {
    const int c = e / N3, i = e - c * N3;
    const long long v = v0 + c;
    if (v >= nvirt) continue;
    if (args.unit_mode == 3) {
      // neighbour couplings: blocks[cell - cell_begin][1 + f][i][j]
      const long long cell = v / vper;
      const int f = int((v - cell * vper) / N3);
      const int j = int(v - cell * vper - f * N3);
      args.blocks[(((cell - args.cell_begin) * 7 + 1 + f) * N3 + i) * N3 + j] = sr[e];
    } else if (args.unit_mode) {
      const long long cell = v / N3;
      const int j = int(v - cell * N3);
      if (args.unit_mode == 1) args.blocks[((cell - args.cell_begin) * N3 + i) * N3 + j] = sr[e];
      else if (i == j) args.blocks[cell * N3 + j] = sr[e];  // diagonal only
    } else {
      __stcs(args.w + v * N3 + i, sr[e]);
    }
  }
}

// kappa at the Gauss points of the operator, once per operator (and on
// gbfem_operator_update_coefficients): kq[cell][a][b][c] = sum_ijk k_ijk
// L_i(x_a) L_j(x_b) L_k(x_c); kf[cell][2d+s][a][b] the same on face (d, s),
// the normal factor L_i(s), (a, b) the tangential points in axis order, as the
// kernel's face arrays.  Direct sums, one thread per point.
template <typename T, int N, int Q>
__global__ void dg_kappa_points_kernel(const T* __restrict__ kappa, T* __restrict__ kq, T* __restrict__ kf,
                                       long long ncells, const __grid_constant__ DgTablesT<T> tabs) {
  constexpr int N2 = N * N, N3 = N2 * N, Q2 = Q * Q, Q3 = Q2 * Q, PER = Q3 + 6 * Q2;
  const long long total = ncells * PER;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total;
       e += (long long)gridDim.x * blockDim.x) {
    const long long cell = e / PER;
    const int r = int(e - cell * PER);
    const T* kc = kappa + cell * N3;
    T f0[N], f1[N], f2[N];  // the 1-D factors along x, y, z
    if (r < Q3) {
      const int a = r / Q2, b = (r / Q) % Q, c = r % Q;
#pragma unroll
      for (int i = 0; i < N; ++i) {
        f0[i] = tabs.B[a * N + i];
        f1[i] = tabs.B[b * N + i];
        f2[i] = tabs.B[c * N + i];
      }
    } else {
      const int fr = r - Q3, f = fr / Q2, ab = fr - f * Q2;
      const int d = f >> 1, sd = f & 1, a = ab / Q, b = ab % Q;
#pragma unroll
      for (int i = 0; i < N; ++i) {
        const T ts = tabs.tr[sd * N + i];
        f0[i] = d == 0 ? ts : tabs.B[a * N + i];
        f1[i] = d == 0 ? tabs.B[a * N + i] : (d == 1 ? ts : tabs.B[b * N + i]);
        f2[i] = d == 2 ? ts : tabs.B[b * N + i];
      }
    }
    T acc = T(0);
#pragma unroll
    for (int i = 0; i < N; ++i) {
      T si = T(0);
#pragma unroll
      for (int j = 0; j < N; ++j) {
        T sj = T(0);
#pragma unroll
        for (int k = 0; k < N; ++k) sj = fma(f2[k], __ldg(kc + i * N2 + j * N + k), sj);
        si = fma(f1[j], sj, si);
      }
      acc = fma(f0[i], si, acc);
    }
    if (r < Q3) kq[cell * Q3 + r] = acc;
    else kf[cell * 6 * Q2 + (r - Q3)] = acc;
  }
}

}  // namespace gbfem
