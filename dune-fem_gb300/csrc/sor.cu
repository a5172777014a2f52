// Jacobi / Gauss-Seidel / SOR / SSOR preconditioners of an assembled DG
// operator: FemPreconditioning (solver/fempreconditioning.hh:59-161) over
// SparseRowMatrix::forwardIterative / backwardIterative
// (operator/matrix/spmatrix.hh:376-480), which sweep the rows in natural
// order:
//   x_i = w (b_i - sum_{j != i} a_ij x_j) / a_ii
// with x read from the vector being written (Gauss-Seidel, SOR, SSOR) or from
// the previous iterate (Jacobi).  The near-zero diagonal rule is the
// reference's (|a_ii| < 16 eps -> 1).
//
// GPU form of the natural-order sweep.  A row of cell c couples to c itself
// and its six face neighbours.  With the cell index x + Nx (y + Ny z), every
// neighbour with a smaller index (also across a periodic boundary) has level
// x+y+z exactly one less, or lies on a larger level when it was wrapped from
// the far side, where natural order sees its old value too.  So the sweep runs
// level by level (one launch per level, Nx+Ny+Nz-2 per sweep), all cells of a
// level in parallel, one warp per cell walking its rows in order: each row
// sees the new values of the cell's earlier rows and of the earlier levels,
// and the old values of everything after it, which is the sequential sweep's
// data dependence.  Sums are warp reductions in a fixed order (rounding
// differs from the reference's left-to-right sum, not the values used).
#include <cuda_runtime.h>
#include <algorithm>
#include <cmath>
#include <new>
#include <vector>

#include "blas.cuh"
#include "gbfem_internal.cuh"
#include "operator_impl.hpp"
#include "solver_impl.hpp"

namespace gbfem {

template <typename T>
__global__ void __launch_bounds__(128) k_sor_level(const T* __restrict__ blocks, const long long* __restrict__ col,
                                                  const T* __restrict__ dinv, const T* __restrict__ b,
                                                  const T* xold, T* x, const int* __restrict__ cells, long long count,
                                                  int nloc, T w, int forward) {
  const long long wi = (long long)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  if (wi >= count) return;
  const long long c = cells[wi];
  for (int rr = 0; rr < nloc; ++rr) {
    const int r = forward ? rr : nloc - 1 - rr;
    double acc = 0.0;
    for (int k = 0; k < 7; ++k) {
      const long long cc = col[c * 7 + k];
      if (cc < 0) continue;
      const T* B = blocks + ((c * 7 + k) * (long long)nloc + r) * nloc;
      for (int j = lane; j < nloc; j += 32) {
        if (k == 0 && j == r) continue;
        acc += double(B[j]) * double(xold[cc * nloc + j]);
      }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
    const long long row = c * nloc + r;
    if (lane == 0) x[row] = T(double(w) * ((double(b[row]) - acc) * double(dinv[row])));
    __syncwarp();
  }
}

template <typename T>
__global__ void k_sor_dinv(long long n, T* d) {
  const T eps = T(16) * (sizeof(T) == 8 ? T(2.220446049250313e-16) : T(1.1920929e-07));
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const T v = d[i];
    d[i] = (v < eps && v > -eps) ? T(1) : T(1) / v;
  }
}

int sor_apply(const gbfem_preconditioner_s* pc, const void* r, void* z, cudaStream_t s) {
  const auto* op = pc->sor_op;
  const long long n = pc->n;
  const int nloc = op->nloc;
  const size_t es = pc->precision == GBFEM_F64 ? 8 : 4;
  GBFEM_CUDA_TRY(cudaMemsetAsync(z, 0, size_t(n) * es, s));
  const bool jacobi = pc->sor_method == GBFEM_SMOOTHER_JACOBI;
  if (jacobi) GBFEM_CUDA_TRY(cudaMemsetAsync(pc->sor_tmp, 0, size_t(n) * es, s));
  void* xold = jacobi ? pc->sor_tmp : z;
  auto sweep = [&](bool forward) -> int {
    const int nlev = int(pc->sor_level_offsets.size()) - 1;
    for (int li = 0; li < (jacobi ? 1 : nlev); ++li) {
      const int l = forward ? li : nlev - 1 - li;
      const long long b0 = jacobi ? 0 : pc->sor_level_offsets[l];
      const long long cnt = jacobi ? op->ncells : pc->sor_level_offsets[l + 1] - b0;
      if (cnt <= 0) continue;
      const unsigned grid = unsigned((cnt + 3) / 4);
      if (pc->precision == GBFEM_F64)
        k_sor_level<double><<<grid, 128, 0, s>>>((const double*)op->bsr_blocks, op->bsr_col, (const double*)pc->data,
                                                 (const double*)r, (const double*)xold, (double*)z,
                                                 pc->sor_cells + b0, cnt, nloc, pc->sor_relax, forward ? 1 : 0);
      else
        k_sor_level<float><<<grid, 128, 0, s>>>((const float*)op->bsr_blocks, op->bsr_col, (const float*)pc->data,
                                                (const float*)r, (const float*)xold, (float*)z, pc->sor_cells + b0,
                                                cnt, nloc, float(pc->sor_relax), forward ? 1 : 0);
    }
    GBFEM_CUDA_TRY(cudaGetLastError());
    return GBFEM_OK;
  };
  for (int i = 0; i < pc->sor_sweeps; ++i) {
    GBFEM_TRY(sweep(true));
    if (pc->sor_method == GBFEM_SMOOTHER_SSOR) GBFEM_TRY(sweep(false));
    if (jacobi && i < pc->sor_sweeps - 1)
      GBFEM_CUDA_TRY(cudaMemcpyAsync(pc->sor_tmp, z, size_t(n) * es, cudaMemcpyDeviceToDevice, s));
  }
  return GBFEM_OK;
}

}  // namespace gbfem

using namespace gbfem;

extern "C" int gbfem_preconditioner_sor_create(gbfem_operator op, int method, int iterations, double relaxation,
                                               gbfem_preconditioner* out) {
  if (!op || !out) return set_error(GBFEM_ERR_INVALID, "gbfem_preconditioner_sor_create: null argument");
  *out = nullptr;
  if (op->kind != OpKind::BSR)
    return set_error(GBFEM_ERR_INVALID, "gbfem_preconditioner_sor_create: needs an assembled operator (gbfem_operator_assemble)");
  if (method != GBFEM_SMOOTHER_JACOBI && method != GBFEM_SMOOTHER_GAUSS_SEIDEL && method != GBFEM_SMOOTHER_SOR &&
      method != GBFEM_SMOOTHER_SSOR)
    return set_error(GBFEM_ERR_INVALID, "gbfem_preconditioner_sor_create: unknown method");
  if (iterations < 1) return set_error(GBFEM_ERR_INVALID, "gbfem_preconditioner_sor_create: iterations < 1");
  auto* pc = new (std::nothrow) gbfem_preconditioner_s();
  if (!pc) return set_error(GBFEM_ERR_INVALID, "out of host memory");
  pc->kind = PcKind::Sor;
  pc->precision = op->precision;
  pc->n = op->ndofs;
  pc->nloc = op->nloc;
  pc->sor_op = op;
  pc->sor_method = method;
  pc->sor_sweeps = iterations;
  // Gauss-Seidel relaxes with 1 (fempreconditioning.hh:89)
  pc->sor_relax = method == GBFEM_SMOOTHER_GAUSS_SEIDEL ? 1.0 : relaxation;
  const size_t es = op->precision == GBFEM_F64 ? 8 : 4;
  // cells grouped by level x+y+z
  const int nx = op->dg.grid.cells[0], ny = op->dg.grid.cells[1], nz = op->dg.grid.cells[2];
  const int nlev = nx + ny + nz - 2;
  std::vector<long long> counts(nlev + 1, 0);
  for (int z = 0; z < nz; ++z)
    for (int y = 0; y < ny; ++y)
      for (int x = 0; x < nx; ++x) ++counts[x + y + z + 1];
  for (int l = 0; l < nlev; ++l) counts[l + 1] += counts[l];
  pc->sor_level_offsets = counts;
  std::vector<int> cells(op->ncells);
  std::vector<long long> fill(counts.begin(), counts.end() - 1);
  for (int z = 0; z < nz; ++z)
    for (int y = 0; y < ny; ++y)
      for (int x = 0; x < nx; ++x) cells[fill[x + y + z]++] = x + nx * (y + ny * z);
  cudaError_t e = cudaMalloc(&pc->data, size_t(op->ndofs) * es);
  if (e == cudaSuccess) e = cudaMalloc(&pc->sor_cells, size_t(op->ncells) * sizeof(int));
  if (e == cudaSuccess && method == GBFEM_SMOOTHER_JACOBI) e = cudaMalloc(&pc->sor_tmp, size_t(op->ndofs) * es);
  if (e == cudaSuccess)
    e = cudaMemcpy(pc->sor_cells, cells.data(), size_t(op->ncells) * sizeof(int), cudaMemcpyHostToDevice);
  if (e != cudaSuccess) {
    gbfem_preconditioner_destroy(pc);
    return set_cuda_error(e, "gbfem_preconditioner_sor_create");
  }
  int rc = bsr_apply(op, nullptr, pc->data, nullptr, 1);  // the diagonal (extractDiagonal)
  if (rc == GBFEM_OK) {
    if (op->precision == GBFEM_F64) k_sor_dinv<double><<<stream_grid(pc->n), 256>>>(pc->n, (double*)pc->data);
    else k_sor_dinv<float><<<stream_grid(pc->n), 256>>>(pc->n, (float*)pc->data);
    e = cudaDeviceSynchronize();
    if (e != cudaSuccess) rc = set_cuda_error(e, "gbfem_preconditioner_sor_create");
  }
  if (rc) {
    gbfem_preconditioner_destroy(pc);
    return rc;
  }
  *out = pc;
  return GBFEM_OK;
}
