// Assembled DG operator: the Jacobian in block-sparse-row form, for the
// matrix-based path (DifferentiableGalerkinOperator::assemble,
// schemes/galerkin.hh:1195-1314, 1548-1643, into a SparseRowMatrix,
// operator/matrix/spmatrix.hh:148-180).
//
// Each cell row holds 7 dense nloc x nloc blocks: slot 0 couples the cell to
// itself, slot 1 + f to its neighbour through face f (-x,+x,-y,+y,-z,+z); a
// missing neighbour (boundary) is a zero block with column -1.  The blocks
// come from the matrix-free kernel applied to unit vectors (slot 0: own dofs
// e_j; slots 1..6: the neighbour's dofs e_j, own dofs 0), so the assembled
// matrix reproduces the matrix-free apply (tests: A x == op(x)).
// The assembled operator is an ordinary gbfem_operator: apply is the
// block SpMV, so the solvers take it unchanged.
#include <cuda_runtime.h>
#include <new>

#include "blas.cuh"
#include "gbfem_internal.cuh"
#include "operator_impl.hpp"

namespace gbfem {

// y_c = sum_k B[c][k] x[col[c][k]]: one CTA per cell, one warp per row group
template <typename T>
__global__ void bsr_apply_kernel(const T* __restrict__ blocks, const long long* __restrict__ col,
                                 const T* __restrict__ x, T* __restrict__ y, int nb, long long ncells) {
  extern __shared__ __align__(16) unsigned char smraw[];
  T* xs = reinterpret_cast<T*>(smraw);  // [7][nb]
  const long long c = blockIdx.x;
  if (c >= ncells) return;
  for (int e = threadIdx.x; e < 7 * nb; e += blockDim.x) {
    const int k = e / nb, j = e - k * nb;
    const long long cc = col[c * 7 + k];
    xs[e] = cc >= 0 ? x[cc * nb + j] : T(0);
  }
  __syncthreads();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
  for (int row = warp; row < nb; row += nw) {
    double s = 0.0;
    for (int k = 0; k < 7; ++k) {
      const T* B = blocks + ((c * 7 + k) * (long long)nb + row) * nb;
      for (int j = lane; j < nb; j += 32) s += double(B[j]) * double(xs[k * nb + j]);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
    if (lane == 0) y[c * nb + row] = T(s);
  }
}

template <typename T>
__global__ void bsr_diag_kernel(const T* __restrict__ blocks, T* __restrict__ diag, int nb, long long ncells) {
  const long long n = ncells * nb;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x) {
    const long long c = e / nb;
    const int i = int(e - c * nb);
    diag[e] = blocks[((c * 7) * (long long)nb + i) * nb + i];
  }
}

__global__ void bsr_columns_kernel(long long* __restrict__ col, int nx, int ny, int nz, int px, int py, int pz,
                                   long long ncells) {
  for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < ncells;
       c += (long long)gridDim.x * blockDim.x) {
    const long long x = c % nx, y = (c / nx) % ny, z = c / ((long long)nx * ny);
    const long long xyz[3] = {x, y, z};
    const int nn[3] = {nx, ny, nz}, per[3] = {px, py, pz};
    col[c * 7] = c;
    for (int f = 0; f < 6; ++f) {
      const int d = f >> 1;
      long long q[3] = {xyz[0], xyz[1], xyz[2]};
      q[d] += (f & 1) ? 1 : -1;
      long long v = -1;
      if (q[d] >= 0 && q[d] < nn[d]) v = q[0] + (long long)nx * (q[1] + (long long)ny * q[2]);
      else if (per[d]) {
        q[d] = (q[d] + nn[d]) % nn[d];
        v = q[0] + (long long)nx * (q[1] + (long long)ny * q[2]);
      }
      col[c * 7 + 1 + f] = v;
    }
  }
}

int bsr_apply(const gbfem_operator_s* op, const void* x, void* y, cudaStream_t s, int diag_only) {
  const int nb = op->nloc;
  const long long nc = op->ncells;
  if (diag_only) {
    if (op->precision == GBFEM_F64)
      bsr_diag_kernel<double><<<stream_grid(op->ndofs), 256, 0, s>>>((const double*)op->bsr_blocks, (double*)y, nb, nc);
    else
      bsr_diag_kernel<float><<<stream_grid(op->ndofs), 256, 0, s>>>((const float*)op->bsr_blocks, (float*)y, nb, nc);
  } else {
    const size_t sm = size_t(7) * nb * (op->precision == GBFEM_F64 ? 8 : 4);
    if (op->precision == GBFEM_F64)
      bsr_apply_kernel<double><<<unsigned(nc), 128, sm, s>>>((const double*)op->bsr_blocks, op->bsr_col,
                                                             (const double*)x, (double*)y, nb, nc);
    else
      bsr_apply_kernel<float><<<unsigned(nc), 128, sm, s>>>((const float*)op->bsr_blocks, op->bsr_col,
                                                            (const float*)x, (float*)y, nb, nc);
  }
  GBFEM_CUDA_TRY(cudaGetLastError());
  return GBFEM_OK;
}

}  // namespace gbfem

using namespace gbfem;

extern "C" int gbfem_operator_assemble(gbfem_operator op, gbfem_operator* out) {
  if (!op || !out) return set_error(GBFEM_ERR_INVALID, "gbfem_operator_assemble: null argument");
  *out = nullptr;
  if (op->kind != OpKind::DG) return set_error(GBFEM_ERR_NOT_IMPLEMENTED, "gbfem_operator_assemble: DG operators only");
  if (op->nonlinear)
    return set_error(GBFEM_ERR_INVALID, "gbfem_operator_assemble: nonlinear operator (assemble its Jacobian)");
  auto* a = new (std::nothrow) gbfem_operator_s();
  if (!a) return set_error(GBFEM_ERR_INVALID, "out of host memory");
  *a = *op;
  a->kind = OpKind::BSR;
  a->host_u = a->host_w = nullptr;
  a->pipe = nullptr;
  a->jac_points = nullptr;
  a->nonlinear = 0;
  a->kq_cache = a->kf_cache = nullptr;
  a->owns_kcache = false;
  a->jit_lib = a->jit_kernel = nullptr;
  a->owns_kfield = false;
  a->form = a->form_jacobian = 0;  // the matrix of a form's Jacobian is a plain matrix
  a->form_u0 = nullptr;
  a->owns_form_u0 = false;
  a->bsr_blocks = nullptr;
  a->bsr_col = nullptr;
  a->trace_buf = nullptr;
  const int nb = op->nloc;
  const size_t es = op->precision == GBFEM_F64 ? 8 : 4;
  const size_t bsz = size_t(nb) * nb * es;
  cudaError_t e = cudaMalloc(&a->bsr_blocks, size_t(op->ncells) * 7 * bsz);
  if (e == cudaSuccess) e = cudaMalloc(&a->bsr_col, size_t(op->ncells) * 7 * sizeof(long long));
  if (e != cudaSuccess) {
    gbfem_operator_destroy(a);
    return set_cuda_error(e, "gbfem_operator_assemble: allocation");
  }
  const gbfem_grid_desc& g = op->dg.grid;
  bsr_columns_kernel<<<stream_grid(op->ncells), 256>>>(a->bsr_col, g.cells[0], g.cells[1], g.cells[2], g.periodic[0],
                                                        g.periodic[1], g.periodic[2], op->ncells);
  // batches of cells: slot 0 through a temporary (unit mode 1), slots 1..6 in place (unit mode 3)
  long long batch = (1LL << 30) / (long long)bsz;
  if (batch < 1) batch = 1;
  if (batch > op->ncells) batch = op->ncells;
  void* tmp = nullptr;
  e = cudaMalloc(&tmp, size_t(batch) * bsz);
  int rc = e == cudaSuccess ? GBFEM_OK : set_cuda_error(e, "gbfem_operator_assemble: temporary");
  for (long long c0 = 0; c0 < op->ncells && rc == GBFEM_OK; c0 += batch) {
    const long long cnt = c0 + batch <= op->ncells ? batch : op->ncells - c0;
    rc = dg_apply(op, nullptr, nullptr, nullptr, 1, tmp, c0, cnt);
    if (rc) break;
    e = cudaMemcpy2DAsync(static_cast<char*>(a->bsr_blocks) + size_t(c0) * 7 * bsz, 7 * bsz, tmp, bsz, bsz,
                          size_t(cnt), cudaMemcpyDeviceToDevice, nullptr);
    if (e != cudaSuccess) { rc = set_cuda_error(e, "gbfem_operator_assemble: copy"); break; }
    rc = dg_apply(op, nullptr, nullptr, nullptr, 3, static_cast<char*>(a->bsr_blocks) + size_t(c0) * 7 * bsz, c0,
                  cnt);
  }
  if (tmp) cudaFree(tmp);
  if (rc == GBFEM_OK) {
    e = cudaDeviceSynchronize();
    if (e != cudaSuccess) rc = set_cuda_error(e, "gbfem_operator_assemble");
  }
  if (rc) {
    gbfem_operator_destroy(a);
    return rc;
  }
  *out = a;
  return GBFEM_OK;
}
