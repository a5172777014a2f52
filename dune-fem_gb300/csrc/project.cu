// L2 projection of closed-form functions onto the DG Q_p space, for the
// coefficient fields and data of the benchmark problems:
//  * kappa = exp(sum_k a_k cos(2 pi w_k . x + phi_k))  (log-Gaussian random
//    field from Fourier modes),
//  * a Gaussian bump exp(-|x - c|^2 / width^2),
//  * a constant.
// For the orthonormal Legendre basis on an affine cell the projection
// coefficient is c_l = sum_q w_q phi_l(x_q) f(x_q) (reference mass = I); with
// `scale_by_volume` the result is the load vector int_K f phi_l = |K| c_l.
// The Fourier sum is evaluated separably per cell: exp(i(2 pi w.x + phi))
// factors into one complex exponential per axis at the q points of that
// axis, so each mode costs 3q sincos and 2 complex products per point.
#include <cuda_runtime.h>
#include <cmath>
#include <cstdint>
#include <string>

#include "gbfem_internal.cuh"
#include "tables.hpp"

namespace gbfem {

struct ProjArgs {
  int nc[3];
  double lower[3], h[3];
  long long ncells;
  int n, q;
  int kind;
  double param[8];      // bump: centre[3], width; constant: value
  const double* modes;  // [nmodes][5] = wx, wy, wz, phi, a (device)
  int nmodes;
  double scale;         // 1 or |K|
  int precision;
  void* out;
  double B[kMaxQ * kMaxN];
  double pts[kMaxQ], wts[kMaxQ];
};

// One CTA per cell; thread t handles quadrature point t (q^3 <= 343).
__global__ void __launch_bounds__(352) project_kernel(const ProjArgs a) {
  __shared__ double fq[kMaxQ * kMaxQ * kMaxQ];
  __shared__ double ex[3][kMaxQ][2];  // per-axis complex exponentials of one mode
  const long long cell = blockIdx.x;
  if (cell >= a.ncells) return;
  const int q = a.q, n = a.n, q3 = q * q * q;
  const long long cz = cell / ((long long)a.nc[0] * a.nc[1]);
  const long long rem = cell - cz * (long long)a.nc[0] * a.nc[1];
  const long long cy = rem / a.nc[0], cx = rem - cy * a.nc[0];
  const long long cc[3] = {cx, cy, cz};
  const int t = threadIdx.x;
  int ia = 0, ib = 0, ic = 0;
  double x[3] = {0, 0, 0};
  if (t < q3) {
    ia = t % q; ib = (t / q) % q; ic = t / (q * q);  // x fastest
    const int idx[3] = {ia, ib, ic};
    for (int d = 0; d < 3; ++d) x[d] = a.lower[d] + (double(cc[d]) + a.pts[idx[d]]) * a.h[d];
  }
  double val = 0.0;
  if (a.kind == GBFEM_FN_EXP_FOURIER) {
    double s = 0.0;
    for (int m = 0; m < a.nmodes; ++m) {
      const double* md = a.modes + 5 * m;
      __syncthreads();
      if (t < 3 * q) {
        const int d = t / q, k = t - d * q;
        const double xd = a.lower[d] + (double(cc[d]) + a.pts[k]) * a.h[d];
        double sn, cs;
        sincospi(2.0 * md[d] * xd, &sn, &cs);
        ex[d][k][0] = cs;
        ex[d][k][1] = sn;
      }
      __syncthreads();
      if (t < q3) {
        double cp, sp;
        sincos(md[3], &sp, &cp);
        // e^{i phi} * Ex * Ey * Ez, real part
        double re = cp * ex[0][ia][0] - sp * ex[0][ia][1];
        double im = cp * ex[0][ia][1] + sp * ex[0][ia][0];
        double r2 = re * ex[1][ib][0] - im * ex[1][ib][1];
        double i2 = re * ex[1][ib][1] + im * ex[1][ib][0];
        s += md[4] * (r2 * ex[2][ic][0] - i2 * ex[2][ic][1]);
      }
    }
    val = exp(s);
  } else if (a.kind == GBFEM_FN_GAUSSIAN) {
    double r2 = 0.0;
    for (int d = 0; d < 3; ++d) r2 += (x[d] - a.param[d]) * (x[d] - a.param[d]);
    val = exp(-r2 / (a.param[3] * a.param[3]));
  } else {
    val = a.param[0];
  }
  if (t < q3) fq[t] = val * a.wts[ia] * a.wts[ib] * a.wts[ic];
  __syncthreads();
  // c_l = sum_q w_q phi_l(x_q) f(x_q), l = i0 n^2 + i1 n + i2 (i0: x-degree)
  const int n3 = n * n * n;
  for (int l = t; l < n3; l += blockDim.x) {
    const int i0 = l / (n * n), i1 = (l / n) % n, i2 = l % n;
    double acc = 0.0;
    for (int c3 = 0; c3 < q; ++c3)
      for (int b3 = 0; b3 < q; ++b3) {
        const double byz = a.B[b3 * n + i1] * a.B[c3 * n + i2];
        for (int a3 = 0; a3 < q; ++a3) acc += a.B[a3 * n + i0] * byz * fq[(c3 * q + b3) * q + a3];
      }
    acc *= a.scale;
    if (a.precision == GBFEM_F64) static_cast<double*>(a.out)[cell * n3 + l] = acc;
    else static_cast<float*>(a.out)[cell * n3 + l] = float(acc);
  }
}

// SplitMix64 (Steele, Lea & Flood, OOPSLA 2014): the seeded stream of the
// random Fourier modes.
static uint64_t splitmix64(uint64_t& s) {
  uint64_t z = (s += 0x9E3779B97F4A7C15ULL);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
  return z ^ (z >> 31);
}
static double uniform01(uint64_t& s) { return (double(splitmix64(s) >> 11) + 0.5) * (1.0 / 9007199254740992.0); }

}  // namespace gbfem

using namespace gbfem;

extern "C" {

int gbfem_fourier_modes(uint64_t seed, int nmodes, double corr_length, double stddev, double* modes) {
  if (!modes || nmodes <= 0 || !(corr_length > 0)) return set_error(GBFEM_ERR_INVALID, "gbfem_fourier_modes: bad argument");
  uint64_t s = seed;
  const double pi = 3.14159265358979323846;
  const double sw = 1.0 / (2.0 * pi * corr_length);  // std of each wave-number component
  for (int m = 0; m < nmodes; ++m) {
    double g[3];
    for (int d = 0; d < 3; d += 1) {
      // Box-Muller
      const double u1 = uniform01(s), u2 = uniform01(s);
      g[d] = std::sqrt(-2.0 * std::log(u1)) * std::cos(2.0 * pi * u2);
    }
    for (int d = 0; d < 3; ++d) modes[5 * m + d] = sw * g[d];
    modes[5 * m + 3] = 2.0 * pi * uniform01(s);
    modes[5 * m + 4] = stddev * std::sqrt(2.0 / nmodes);
  }
  return GBFEM_OK;
}

int gbfem_dg_project(const gbfem_grid_desc* grid, int order, int quad_points, int kind, const double* params,
                     const double* modes_host, int nmodes, int scale_by_volume, int precision, void* out,
                     void* stream) {
  if (!grid || !out) return set_error(GBFEM_ERR_INVALID, "gbfem_dg_project: null argument");
  if (grid->dim != 3) return set_error(GBFEM_ERR_INVALID, "gbfem_dg_project: 3-D grids only");
  if (order < 0 || order > 4) return set_error(GBFEM_ERR_NOT_IMPLEMENTED, "gbfem_dg_project: order 0..4");
  const int q = quad_points > 0 ? quad_points : order + 2;
  if (q > kMaxQ || q < 1) return set_error(GBFEM_ERR_INVALID, "gbfem_dg_project: bad quad_points");
  if (kind == GBFEM_FN_EXP_FOURIER && (!modes_host || nmodes <= 0))
    return set_error(GBFEM_ERR_INVALID, "gbfem_dg_project: Fourier modes missing");
  if ((kind == GBFEM_FN_GAUSSIAN || kind == GBFEM_FN_CONSTANT) && !params)
    return set_error(GBFEM_ERR_INVALID, "gbfem_dg_project: params missing");
  ProjArgs a{};
  double vol = 1.0;
  for (int d = 0; d < 3; ++d) {
    if (grid->cells[d] <= 0) return set_error(GBFEM_ERR_INVALID, "gbfem_dg_project: bad grid");
    a.nc[d] = grid->cells[d];
    a.lower[d] = grid->lower[d];
    a.h[d] = (grid->upper[d] - grid->lower[d]) / grid->cells[d];
    vol *= a.h[d];
  }
  a.ncells = (long long)a.nc[0] * a.nc[1] * a.nc[2];
  a.n = order + 1;
  a.q = q;
  a.kind = kind;
  if (params) for (int i = 0; i < (kind == GBFEM_FN_GAUSSIAN ? 4 : 1); ++i) a.param[i] = params[i];
  a.nmodes = kind == GBFEM_FN_EXP_FOURIER ? nmodes : 0;
  a.scale = scale_by_volume ? vol : 1.0;
  a.precision = precision;
  a.out = out;
  Tables1D t = make_tables(a.n, q);
  for (int i = 0; i < q; ++i) {
    a.pts[i] = double(t.pts[i]);
    a.wts[i] = double(t.wts[i]);
    for (int l = 0; l < a.n; ++l) a.B[i * a.n + l] = double(t.B[i][l]);
  }
  double* dmodes = nullptr;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (a.nmodes) {
    GBFEM_CUDA_TRY(cudaMalloc(&dmodes, sizeof(double) * 5 * nmodes));
    GBFEM_CUDA_TRY(cudaMemcpyAsync(dmodes, modes_host, sizeof(double) * 5 * nmodes, cudaMemcpyHostToDevice, s));
  }
  a.modes = dmodes;
  project_kernel<<<unsigned(a.ncells), 352, 0, s>>>(a);
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess && dmodes) e = cudaStreamSynchronize(s);
  if (dmodes) cudaFree(dmodes);
  if (e != cudaSuccess) return set_cuda_error(e, "gbfem_dg_project");
  return GBFEM_OK;
}

}  // extern "C"
