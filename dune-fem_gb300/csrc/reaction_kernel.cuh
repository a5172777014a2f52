// Volume reaction term of the nonlinear DG operator and of its Jacobian:
//
//   S(u) = A u + R(u),   R(u)_l = int_K r(u_h) phi_l,   r(u) = c1 u + c3 u^3 + ce exp(u)
//   R'(u0) d = int_K r'(u0_h) d_h phi_l
//
// evaluated with the operator's tensor Gauss rule (q points per direction),
// like the mass integrand of the quadrature kernel: u_h at the q^3 points by
// three 1-D contractions with B[a][i] = L_i(x_a), the pointwise function
// times w_a w_b w_c |K|, and the transposed contractions back to the n^3 test
// functions.  The form is the reference's UFL integrand r(u) v dx taken
// through GalerkinOperator's volume integral (schemes/galerkin.hh:332-360)
// and its linearisation (schemes/galerkin.hh:362-410).
//
// Modes of dg_reaction_kernel:
//   0  w += R(u)                         (after the linear part of the apply)
//   1  pts = w_abc |K| r'(u(x_abc))      (linearisation at u; w unused)
//   2  w += B^T (pts .* B u)             (Jacobian apply)
// dg_reaction_blocks_kernel adds the cell blocks (or only their diagonal) of
// the linearised term to the block diagonal of the Jacobian.
#pragma once
#include <cuda_runtime.h>

#include "dg_kernel.cuh"

namespace gbfem {

template <typename T>
struct ReactTabsT {
  T B[kDgMaxQ * kDgMaxN];  // B[a*n+i] = L_i(x_a)
  T w[kDgMaxQ];
  T xq[kDgMaxQ];           // Gauss points on [0, 1]
  T detK, c1, c3, ce;
  T lower[3], h[3];        // grid origin and cell size (point coordinates)
  int nc[3];               // cells per direction
};

// The built-in family r(u) = c1 u + c3 u^3 + ce e^u.
struct BuiltinReaction {
  static constexpr bool kCoordinates = false;
  template <typename T>
  __device__ static T value(const ReactTabsT<T>& t, T u, T, T, T) {
    return t.c1 * u + t.c3 * u * u * u + (t.ce != T(0) ? t.ce * exp(u) : T(0));
  }
  template <typename T>
  __device__ static T derivative(const ReactTabsT<T>& t, T u, T, T, T) {
    return t.c1 + T(3) * t.c3 * u * u + (t.ce != T(0) ? t.ce * exp(u) : T(0));
  }
};

// R: the pointwise function (value and derivative in u), given the point's
// physical coordinates when R::kCoordinates.
template <typename T, int N, int Q, int CPB, class R>
__device__ __forceinline__ void dg_reaction_body(int mode, const T* __restrict__ u, T* __restrict__ w,
                                                 T* __restrict__ pts, long long cell_begin, long long count,
                                                 const ReactTabsT<T>& tb) {
  constexpr int N3 = N * N * N, Q3 = Q * Q * Q;
  __shared__ T sX[CPB * N3];      // coefficients [i][j][k]
  __shared__ T sY1[CPB * Q * N * N];  // [a][j][k]
  __shared__ T sY2[CPB * Q * Q * N];  // [a][b][k]
  __shared__ T sP[CPB * Q3];      // [a][b][c]
  const int tid = threadIdx.x;
  const long long c0 = cell_begin + (long long)blockIdx.x * CPB;
  const long long cend = cell_begin + count;
  if (c0 >= cend) return;
  const int ncell = int(cend - c0 < CPB ? cend - c0 : CPB);
  for (int e = tid; e < CPB * N3; e += blockDim.x) sX[e] = e < ncell * N3 ? __ldg(u + c0 * N3 + e) : T(0);
  __syncthreads();
  // forward: Y1[a][j][k] = sum_i B[a][i] X[i][j][k]
  for (int e = tid; e < CPB * Q * N * N; e += blockDim.x) {
    const int c = e / (Q * N * N), r = e - c * Q * N * N;
    const int a = r / (N * N), jk = r - a * N * N;
    T s = T(0);
#pragma unroll
    for (int i = 0; i < N; ++i) s = fma(tb.B[a * N + i], sX[c * N3 + i * N * N + jk], s);
    sY1[e] = s;
  }
  __syncthreads();
  // Y2[a][b][k] = sum_j B[b][j] Y1[a][j][k]
  for (int e = tid; e < CPB * Q * Q * N; e += blockDim.x) {
    const int c = e / (Q * Q * N), r = e - c * Q * Q * N;
    const int a = r / (Q * N), b = (r / N) % Q, k = r % N;
    T s = T(0);
#pragma unroll
    for (int j = 0; j < N; ++j) s = fma(tb.B[b * N + j], sY1[c * Q * N * N + (a * N + j) * N + k], s);
    sY2[e] = s;
  }
  __syncthreads();
  // P[a][b][c] = sum_k B[c][k] Y2[a][b][k], then the pointwise function
  for (int e = tid; e < CPB * Q3; e += blockDim.x) {
    const int cl = e / Q3, r = e - cl * Q3;
    const int a = r / (Q * Q), b = (r / Q) % Q, cc = r % Q;
    T s = T(0);
#pragma unroll
    for (int k = 0; k < N; ++k) s = fma(tb.B[cc * N + k], sY2[cl * Q * Q * N + (a * Q + b) * N + k], s);
    const T W = tb.w[a] * tb.w[b] * tb.w[cc] * tb.detK;
    const long long cell = c0 + cl;
    T px = T(0), py = T(0), pz = T(0);
    if (R::kCoordinates) {
      const long long nxy = (long long)tb.nc[0] * tb.nc[1];
      const long long cz = cell / nxy, rem = cell - cz * nxy, cy = rem / tb.nc[0], cx = rem - cy * tb.nc[0];
      px = tb.lower[0] + (T(cx) + tb.xq[a]) * tb.h[0];
      py = tb.lower[1] + (T(cy) + tb.xq[b]) * tb.h[1];
      pz = tb.lower[2] + (T(cz) + tb.xq[cc]) * tb.h[2];
    }
    if (mode == 0) {
      sP[e] = W * R::value(tb, s, px, py, pz);
    } else if (mode == 1) {
      if (cl < ncell) pts[cell * Q3 + r] = W * R::derivative(tb, s, px, py, pz);
    } else {
      sP[e] = cl < ncell ? pts[cell * Q3 + r] * s : T(0);
    }
  }
  if (mode == 1) return;
  __syncthreads();
  // backward: Y2[a][b][k] = sum_c B[c][k] P[a][b][c]
  for (int e = tid; e < CPB * Q * Q * N; e += blockDim.x) {
    const int c = e / (Q * Q * N), r = e - c * Q * Q * N;
    const int ab = r / N, k = r % N;
    T s = T(0);
#pragma unroll
    for (int cc = 0; cc < Q; ++cc) s = fma(tb.B[cc * N + k], sP[c * Q3 + ab * Q + cc], s);
    sY2[e] = s;
  }
  __syncthreads();
  // Y1[a][j][k] = sum_b B[b][j] Y2[a][b][k]
  for (int e = tid; e < CPB * Q * N * N; e += blockDim.x) {
    const int c = e / (Q * N * N), r = e - c * Q * N * N;
    const int a = r / (N * N), j = (r / N) % N, k = r % N;
    T s = T(0);
#pragma unroll
    for (int b = 0; b < Q; ++b) s = fma(tb.B[b * N + j], sY2[c * Q * Q * N + (a * Q + b) * N + k], s);
    sY1[e] = s;
  }
  __syncthreads();
  // X[i][j][k] = sum_a B[a][i] Y1[a][j][k];  w += X
  for (int e = tid; e < ncell * N3; e += blockDim.x) {
    const int c = e / N3, r = e - c * N3;
    const int i = r / (N * N), jk = r - i * N * N;
    T s = T(0);
#pragma unroll
    for (int a = 0; a < Q; ++a) s = fma(tb.B[a * N + i], sY1[c * Q * N * N + a * N * N + jk], s);
    w[c0 * N3 + e] += s;
  }
}

// 128 threads per CTA, CPB cells per CTA
template <typename T, int N, int Q, int CPB, class R = BuiltinReaction>
__global__ void __launch_bounds__(128) dg_reaction_kernel(int mode, const T* __restrict__ u, T* __restrict__ w,
                                                          T* __restrict__ pts, long long cell_begin, long long count,
                                                          const __grid_constant__ ReactTabsT<T> tb) {
  dg_reaction_body<T, N, Q, CPB, R>(mode, u, w, pts, cell_begin, count, tb);
}

// blocks[cell - cell_begin][i][j] += sum_abc pts[abc] phi_i(x_abc) phi_j(x_abc)
// (diag_only: diag[cell][i] += the (i,i) entry); one CTA per cell.
template <typename T, int N, int Q>
__global__ void __launch_bounds__(256) dg_reaction_blocks_kernel(const T* __restrict__ pts, T* __restrict__ out,
                                                                 long long cell_begin, long long count, int diag_only,
                                                                 const __grid_constant__ ReactTabsT<T> tb) {
  constexpr int N3 = N * N * N, Q3 = Q * Q * Q;
  __shared__ T sP[Q3];
  const long long cell = cell_begin + blockIdx.x;
  if (blockIdx.x >= count) return;
  for (int e = threadIdx.x; e < Q3; e += blockDim.x) sP[e] = pts[cell * Q3 + e];
  __syncthreads();
  const int total = diag_only ? N3 : N3 * N3;
  for (int e = threadIdx.x; e < total; e += blockDim.x) {
    const int i = diag_only ? e : e / N3, j = diag_only ? e : e % N3;
    const int i0 = i / (N * N), i1 = (i / N) % N, i2 = i % N;
    const int j0 = j / (N * N), j1 = (j / N) % N, j2 = j % N;
    T acc = T(0);
    for (int a = 0; a < Q; ++a) {
      T sa = T(0);
      for (int b = 0; b < Q; ++b) {
        T sb = T(0);
#pragma unroll
        for (int c = 0; c < Q; ++c) sb = fma(tb.B[c * N + i2] * tb.B[c * N + j2], sP[(a * Q + b) * Q + c], sb);
        sa = fma(tb.B[b * N + i1] * tb.B[b * N + j1], sb, sa);
      }
      acc = fma(tb.B[a * N + i0] * tb.B[a * N + j0], sa, acc);
    }
    if (diag_only) out[cell * N3 + i] += acc;
    else out[((cell - cell_begin) * N3 + i) * (long long)N3 + j] += acc;
  }
}

}  // namespace gbfem
