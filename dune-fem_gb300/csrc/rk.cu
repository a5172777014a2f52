// Explicit SSP-RK3 time stepping of the method-of-lines DG operator.
//
// The space operator is L(u) = -M^{-1} A(u): A is the DG operator (its
// apply is the GalerkinOperator evaluation) and M^{-1} the inverse mass
// matrix, which for the orthonormal Legendre basis on an affine cell is
// 1/|K| (operator/1order/localmassmatrix.hh:303-316, 412-430, applied by
// MOLGalerkinOperator::applyInverseMass, schemes/molgalerkin.hh:100-124).
// The stages follow ExplicitRungeKuttaSolver::solve
// (solver/rungekutta/explicit.hh:160-215) with the TVD3 Butcher table
// (solver/rungekutta/butchertable.cc:43-52):
//   k_0 = L(u);  k_i = L(u + dt sum_{j<i} A_ij k_j);  u += dt sum_j b_j k_j.
// The stage combinations are single fused passes over the vectors, with the
// factor -1/|K| folded into the coefficients.
#include <cuda_runtime.h>
#include <cfloat>
#include <cmath>
#include <new>

#include "blas.cuh"
#include "gbfem_internal.cuh"
#include "operator_impl.hpp"

namespace gbfem {

// y = u + c0 w0 + c1 w1 + c2 w2 (nw terms)
template <typename T>
__global__ void k_stage(long long n, const T* u, int nw, const T* __restrict__ w0, double c0,
                        const T* __restrict__ w1, double c1, const T* __restrict__ w2, double c2, T* y) {  // y may alias u
  const T a0 = T(c0), a1 = T(c1), a2 = T(c2);
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    T v = u[i];
    v += a0 * w0[i];
    if (nw > 1) v += a1 * w1[i];
    if (nw > 2) v += a2 * w2[i];
    y[i] = v;
  }
}

// v[i] = uniform(-1, 1) from a SplitMix64 hash of (seed, i)
template <typename T>
__global__ void k_random_fill(long long n, unsigned long long seed, T* v) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    unsigned long long z = seed + 0x9E3779B97F4A7C15ULL * (unsigned long long)(i + 1);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    z ^= z >> 31;
    v[i] = T(double(z >> 11) * (2.0 / 9007199254740992.0) - 1.0);
  }
}

}  // namespace gbfem

struct gbfem_rk_solver_s {
  gbfem_operator op = nullptr;
  void* k[3] = {nullptr, nullptr, nullptr};
  void* y = nullptr;
  double minv = 1.0;  // 1/|K|
};

using namespace gbfem;

extern "C" {

int gbfem_rk3_create(gbfem_operator op, gbfem_rk_solver* out) {
  if (!op || !out) return set_error(GBFEM_ERR_INVALID, "gbfem_rk3_create: null argument");
  if (op->kind != OpKind::DG) return set_error(GBFEM_ERR_NOT_IMPLEMENTED, "gbfem_rk3_create: DG operators only");
  *out = nullptr;
  auto* rk = new (std::nothrow) gbfem_rk_solver_s();
  if (!rk) return set_error(GBFEM_ERR_INVALID, "out of host memory");
  rk->op = op;
  double vol = 1.0;
  for (int d = 0; d < 3; ++d) vol *= (op->dg.grid.upper[d] - op->dg.grid.lower[d]) / op->dg.grid.cells[d];
  rk->minv = 1.0 / vol;
  const size_t bytes = size_t(op->ndofs) * (op->precision == GBFEM_F64 ? 8 : 4);
  for (int i = 0; i < 4; ++i) {
    void* p = nullptr;
    cudaError_t e = cudaMalloc(&p, bytes);
    if (e != cudaSuccess) {
      gbfem_rk3_destroy(rk);
      return set_cuda_error(e, "gbfem_rk3_create");
    }
    if (i < 3) rk->k[i] = p;
    else rk->y = p;
  }
  *out = rk;
  return GBFEM_OK;
}

int gbfem_rk3_destroy(gbfem_rk_solver rk) {
  if (!rk) return GBFEM_OK;
  for (void* p : rk->k) if (p) cudaFree(p);
  if (rk->y) cudaFree(rk->y);
  delete rk;
  return GBFEM_OK;
}

int gbfem_rk3_step(gbfem_rk_solver rk, void* u, double dt, void* stream) {
  if (!rk || !u) return set_error(GBFEM_ERR_INVALID, "gbfem_rk3_step: null argument");
  static const double A[3][3] = {{0.0, 0.0, 0.0}, {1.0, 0.0, 0.0}, {0.25, 0.25, 0.0}};
  static const double b[3] = {1.0 / 6.0, 1.0 / 6.0, 2.0 / 3.0};
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const long long n = rk->op->ndofs;
  const double f = -dt * rk->minv;  // dt * L = -dt/|K| * A
  // k_j hold A(stage_j) (unscaled); the coefficients carry -dt/|K|.
  GBFEM_TRY(gbfem_operator_apply(rk->op, u, rk->k[0], s));
  for (int i = 1; i < 3; ++i) {
    if (rk->op->precision == GBFEM_F64)
      k_stage<double><<<stream_grid(n), 256, 0, s>>>(n, (const double*)u, i, (const double*)rk->k[0], A[i][0] * f,
                                                     (const double*)rk->k[1], A[i][1] * f, nullptr, 0.0,
                                                     (double*)rk->y);
    else
      k_stage<float><<<stream_grid(n), 256, 0, s>>>(n, (const float*)u, i, (const float*)rk->k[0], A[i][0] * f,
                                                    (const float*)rk->k[1], A[i][1] * f, nullptr, 0.0,
                                                    (float*)rk->y);
    GBFEM_CUDA_TRY(cudaGetLastError());
    GBFEM_TRY(gbfem_operator_apply(rk->op, rk->y, rk->k[i], s));
  }
  if (rk->op->precision == GBFEM_F64)
    k_stage<double><<<stream_grid(n), 256, 0, s>>>(n, (const double*)u, 3, (const double*)rk->k[0], b[0] * f,
                                                   (const double*)rk->k[1], b[1] * f, (const double*)rk->k[2],
                                                   b[2] * f, (double*)u);
  else
    k_stage<float><<<stream_grid(n), 256, 0, s>>>(n, (const float*)u, 3, (const float*)rk->k[0], b[0] * f,
                                                  (const float*)rk->k[1], b[1] * f, (const float*)rk->k[2],
                                                  b[2] * f, (float*)u);
  GBFEM_CUDA_TRY(cudaGetLastError());
  return GBFEM_OK;
}

int gbfem_dg_time_step_estimate(gbfem_operator op, int power_iterations, uint64_t seed, double* dt_estimate,
                                double* dt_upper_bound) {
  if (!op || !dt_estimate || !dt_upper_bound || power_iterations < 0)
    return set_error(GBFEM_ERR_INVALID, "gbfem_dg_time_step_estimate: invalid argument");
  if (op->kind != OpKind::DG) return set_error(GBFEM_ERR_NOT_IMPLEMENTED, "gbfem_dg_time_step_estimate: DG only");
  const gbfem_dg_desc& d = op->dg;
  double hmin = 1e300, vol = 1.0, bnorm = 0.0;
  for (int k = 0; k < 3; ++k) {
    const double h = (d.grid.upper[k] - d.grid.lower[k]) / d.grid.cells[k];
    hmin = h < hmin ? h : hmin;
    vol *= h;
    bnorm += d.velocity[k] * d.velocity[k];
  }
  bnorm = std::sqrt(bnorm);
  *dt_estimate = bnorm > 0.0 ? hmin / (bnorm * (2 * d.order + 1)) : DBL_MAX;
  *dt_upper_bound = DBL_MAX;
  if (power_iterations == 0) return GBFEM_OK;
  // power iteration for rho(M^{-1} A), M^{-1} = 1/|K|; 2/rho keeps dt*lambda
  // inside SSP-RK3's real stability interval [-2.51, 0]
  const long long n = op->ndofs;
  const int prec = op->precision;
  const size_t bytes = size_t(n) * (prec == GBFEM_F64 ? 8 : 4);
  void *v = nullptr, *av = nullptr;
  cudaError_t e = cudaMalloc(&v, bytes);
  if (e == cudaSuccess) e = cudaMalloc(&av, bytes);
  struct Free { void** a; void** b; ~Free() { if (*a) cudaFree(*a); if (*b) cudaFree(*b); } } fr{&v, &av};
  if (e != cudaSuccess) return set_cuda_error(e, "gbfem_dg_time_step_estimate");
  if (prec == GBFEM_F64) k_random_fill<double><<<stream_grid(n), 256>>>(n, seed, static_cast<double*>(v));
  else k_random_fill<float><<<stream_grid(n), 256>>>(n, seed, static_cast<float*>(v));
  GBFEM_CUDA_TRY(cudaGetLastError());
  double vv = 0.0, rho = 0.0;
  GBFEM_TRY(gbfem_dot(prec, n, v, v, &vv, nullptr));
  for (int it = 0; it < power_iterations; ++it) {
    GBFEM_TRY(gbfem_operator_apply(op, v, av, nullptr));
    double aa = 0.0;
    GBFEM_TRY(gbfem_dot(prec, n, av, av, &aa, nullptr));
    if (!(aa > 0.0) || !std::isfinite(aa)) break;
    rho = std::sqrt(aa / vv) / vol;
    GBFEM_TRY(gbfem_scal(prec, n, 1.0 / std::sqrt(aa), av, nullptr));
    void* t = v;
    v = av;
    av = t;
    vv = 1.0;
  }
  if (rho > 0.0) *dt_upper_bound = 2.0 / rho;
  return GBFEM_OK;
}

}  // extern "C"
