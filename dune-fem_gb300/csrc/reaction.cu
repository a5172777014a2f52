// Nonlinear DG operator S(u) = A u + R(u) and its Jacobian operator
// A + R'(u0): instantiation of the reaction kernels and the entry points.
//
// ≙ GalerkinOperator with a nonlinear UFL integrand (r(u) v dx added to the
// SIPG/upwind form), DifferentiableGalerkinOperator::jacobian(u, jOp)
// (schemes/galerkin.hh:1548-1643) and the linearised integrals
// (schemes/galerkin.hh:362-410).  The Jacobian is matrix-free: the linear
// part re-uses the DG kernels and the linearised reaction is stored as its
// weighted values at the Gauss points of every cell.
#include <cuda_runtime.h>
#include <cmath>
#include <new>
#include <string>

#include "gbfem_internal.cuh"
#include "operator_impl.hpp"
#include "reaction_kernel.cuh"

namespace gbfem {

static const DgTablesT<double>& tables_of(const gbfem_operator_s* op, const double*) { return op->tab64; }
static const DgTablesT<float>& tables_of(const gbfem_operator_s* op, const float*) { return op->tab32; }

template <typename T>
static void fill_react_tabs(const gbfem_operator_s* op, ReactTabsT<T>* t) {
  const DgTablesT<T>& src = tables_of(op, static_cast<const T*>(nullptr));
  for (int e = 0; e < kDgMaxQ * kDgMaxN; ++e) t->B[e] = src.B[e];
  for (int a = 0; a < kDgMaxQ; ++a) t->w[a] = src.w[a];
  for (int a = 0; a < kDgMaxQ; ++a) t->xq[a] = src.x[a];
  double vol = 1.0;
  for (int k = 0; k < 3; ++k) {
    const double h = (op->dg.grid.upper[k] - op->dg.grid.lower[k]) / op->dg.grid.cells[k];
    vol *= h;
    t->lower[k] = T(op->dg.grid.lower[k]);
    t->h[k] = T(h);
    t->nc[k] = op->dg.grid.cells[k];
  }
  t->detK = T(vol);
  t->c1 = T(op->react[0]);
  t->c3 = T(op->react[1]);
  t->ce = T(op->react[2]);
}

template <typename T, int N, int Q>
static int reaction_launch_nq(const gbfem_operator_s* op, int mode, const void* u, void* w, void* pts,
                              long long cell_begin, long long count, int blocks_mode, cudaStream_t s) {
  ReactTabsT<T> tb;
  fill_react_tabs(op, &tb);
  if (blocks_mode) {
    if (count > 2147483647LL) return set_error(GBFEM_ERR_INVALID, "reaction blocks: grid too large");
    dg_reaction_blocks_kernel<T, N, Q><<<unsigned(count), 256, 0, s>>>(
        static_cast<const T*>(pts), static_cast<T*>(w), cell_begin, count, blocks_mode == 2, tb);
  } else {
    constexpr int CPB = 4;
    const long long grid = (count + CPB - 1) / CPB;
    if (grid > 2147483647LL) return set_error(GBFEM_ERR_INVALID, "reaction: grid too large");
    dg_reaction_kernel<T, N, Q, CPB><<<unsigned(grid), 128, 0, s>>>(
        mode, static_cast<const T*>(u), static_cast<T*>(w), static_cast<T*>(pts), cell_begin, count, tb);
  }
  GBFEM_CUDA_TRY(cudaGetLastError());
  return GBFEM_OK;
}

template <typename T>
static int reaction_launch_t(const gbfem_operator_s* op, int mode, const void* u, void* w, void* pts,
                             long long cell_begin, long long count, int blocks_mode, cudaStream_t s) {
#define GBFEM_R_CASE(NN, QQ) \
  if (op->n == NN && op->q == QQ) return reaction_launch_nq<T, NN, QQ>(op, mode, u, w, pts, cell_begin, count, blocks_mode, s);
  GBFEM_R_CASE(2, 2)
  GBFEM_R_CASE(2, 3)
  GBFEM_R_CASE(3, 3)
  GBFEM_R_CASE(3, 4)
  GBFEM_R_CASE(4, 4)
  GBFEM_R_CASE(4, 5)
  GBFEM_R_CASE(5, 5)
  GBFEM_R_CASE(5, 6)
#undef GBFEM_R_CASE
  return set_error(GBFEM_ERR_NOT_IMPLEMENTED, "reaction: unsupported (p, q)");
}

// mode 0/1/2 of dg_reaction_kernel on cells [cell_begin, cell_begin+count);
// blocks_mode 1: add the linearised blocks into w (block-diagonal layout
// relative to cell_begin), 2: add their diagonal into w.
// the user's run-time compiled reaction (modes 0 and 1: they evaluate r, r')
template <typename T>
static int reaction_launch_jit(const gbfem_operator_s* op, int mode, const void* u, void* w, void* pts,
                               long long cell_begin, long long count, cudaStream_t s) {
  ReactTabsT<T> tb;
  fill_react_tabs(op, &tb);
  constexpr int CPB = 4;
  const long long grid = (count + CPB - 1) / CPB;
  if (grid > 2147483647LL) return set_error(GBFEM_ERR_INVALID, "reaction: grid too large");
  void* args[] = {&mode, const_cast<void**>(&u), &w, &pts, &cell_begin, &count, &tb};
  GBFEM_CUDA_TRY(cudaLaunchKernel(reinterpret_cast<const void*>(op->jit_kernel), dim3(unsigned(grid)), dim3(128),
                                  args, 0, s));
  return GBFEM_OK;
}

int reaction_launch(const gbfem_operator_s* op, int mode, const void* u, void* w, void* pts, long long cell_begin,
                    long long count, int blocks_mode, cudaStream_t s) {
  if (count <= 0) return GBFEM_OK;
  if (op->jit_kernel && !blocks_mode && mode != 2)
    return op->precision == GBFEM_F64 ? reaction_launch_jit<double>(op, mode, u, w, pts, cell_begin, count, s)
                                      : reaction_launch_jit<float>(op, mode, u, w, pts, cell_begin, count, s);
  return op->precision == GBFEM_F64 ? reaction_launch_t<double>(op, mode, u, w, pts, cell_begin, count, blocks_mode, s)
                                    : reaction_launch_t<float>(op, mode, u, w, pts, cell_begin, count, blocks_mode, s);
}

}  // namespace gbfem

using namespace gbfem;

extern "C" {

int gbfem_dg_nonlinear_operator_create(const gbfem_dg_desc* desc, const gbfem_reaction* reaction,
                                       gbfem_operator* out) {
  if (!desc || !reaction || !out) return set_error(GBFEM_ERR_INVALID, "gbfem_dg_nonlinear_operator_create: null argument");
  GBFEM_TRY(gbfem_dg_operator_create(desc, out));
  gbfem_operator op = *out;
  op->nonlinear = 1;
  op->react[0] = reaction->linear;
  op->react[1] = reaction->cubic;
  op->react[2] = reaction->exponential;
  return GBFEM_OK;
}

int gbfem_dg_nonlinear_operator_create_jit(const gbfem_dg_desc* desc, const char* cubin_path, gbfem_operator* out) {
  if (!desc || !cubin_path || !out)
    return set_error(GBFEM_ERR_INVALID, "gbfem_dg_nonlinear_operator_create_jit: null argument");
  GBFEM_TRY(gbfem_dg_operator_create(desc, out));
  gbfem_operator op = *out;
  // the cubin holds one kernel per (precision, n, q), named for it
  const std::string name = std::string("gbfem_user_reaction_") + (op->precision == GBFEM_F64 ? "f64" : "f32") +
                           "_n" + std::to_string(op->n) + "_q" + std::to_string(op->q);
  cudaLibrary_t lib = nullptr;
  cudaError_t e = cudaLibraryLoadFromFile(&lib, cubin_path, nullptr, nullptr, 0, nullptr, nullptr, 0);
  if (e != cudaSuccess) {
    (void)cudaGetLastError();  // the failed runtime call must not surface at the next launch check
    gbfem_operator_destroy(op);
    *out = nullptr;
    return set_cuda_error(e, (std::string("gbfem_dg_nonlinear_operator_create_jit: loading ") + cubin_path).c_str());
  }
  cudaKernel_t k = nullptr;
  e = cudaLibraryGetKernel(&k, lib, name.c_str());
  if (e != cudaSuccess) {
    (void)cudaGetLastError();
    cudaLibraryUnload(lib);
    gbfem_operator_destroy(op);
    *out = nullptr;
    return set_cuda_error(e, ("gbfem_dg_nonlinear_operator_create_jit: no kernel " + name +
                              " in the cubin (compiled for another precision / order / quadrature?)").c_str());
  }
  op->jit_lib = lib;
  op->jit_kernel = reinterpret_cast<void*>(k);
  op->nonlinear = 1;
  return GBFEM_OK;
}

int gbfem_operator_nonlinear(gbfem_operator op, int* nonlinear) {
  if (!op || !nonlinear) return set_error(GBFEM_ERR_INVALID, "gbfem_operator_nonlinear: null argument");
  *nonlinear = op->nonlinear;
  return GBFEM_OK;
}

int gbfem_operator_jacobian_create(gbfem_operator op, gbfem_operator* jac) {
  if (!op || !jac) return set_error(GBFEM_ERR_INVALID, "gbfem_operator_jacobian_create: null argument");
  *jac = nullptr;
  if (op->kind != OpKind::DG) return set_error(GBFEM_ERR_NOT_IMPLEMENTED, "gbfem_operator_jacobian_create: DG only");
  auto* j = new (std::nothrow) gbfem_operator_s();
  if (!j) return set_error(GBFEM_ERR_INVALID, "out of host memory");
  *j = *op;
  j->host_u = j->host_w = nullptr;
  j->bsr_blocks = nullptr;
  j->bsr_col = nullptr;
  j->trace_buf = nullptr;
  j->pipe = nullptr;
  j->jac_points = nullptr;
  j->nonlinear = 0;
  j->owns_kcache = false;  // shares the operator's kappa point caches
  j->jit_lib = j->jit_kernel = nullptr;  // the Jacobian applies the stored linearisation only
  j->owns_kfield = false;
  j->owns_form_u0 = false;
  if (op->form && op->nonlinear) {
    // a form's Jacobian: the dual-number kernel at a stored point (the form's
    // kernels stay owned by the form)
    const size_t bytes = size_t(op->ndofs) * (op->precision == GBFEM_F64 ? 8 : 4);
    const cudaError_t e = cudaMalloc(&j->form_u0, bytes);
    if (e != cudaSuccess) {
      delete j;
      return set_cuda_error(e, "gbfem_operator_jacobian_create");
    }
    cudaMemset(j->form_u0, 0, bytes);
    j->owns_form_u0 = true;
    j->form_jacobian = 1;
  } else if (op->nonlinear) {
    const size_t bytes = size_t(op->ncells) * op->q * op->q * op->q * (op->precision == GBFEM_F64 ? 8 : 4);
    const cudaError_t e = cudaMalloc(&j->jac_points, bytes);
    if (e != cudaSuccess) {
      delete j;
      return set_cuda_error(e, "gbfem_operator_jacobian_create");
    }
    cudaMemset(j->jac_points, 0, bytes);
  }
  *jac = j;
  return GBFEM_OK;
}

int gbfem_operator_jacobian(gbfem_operator op, const void* u, gbfem_operator jac, void* stream) {
  if (!op || !u || !jac) return set_error(GBFEM_ERR_INVALID, "gbfem_operator_jacobian: null argument");
  if (jac->ncells != op->ncells || jac->q != op->q || jac->n != op->n || jac->precision != op->precision ||
      jac->nloc != op->nloc)
    return set_error(GBFEM_ERR_INVALID, "gbfem_operator_jacobian: jacobian was created for another operator");
  if (!op->nonlinear) return GBFEM_OK;  // the Jacobian of a linear operator is the operator
  if (op->form) {
    if (!jac->form_jacobian || !jac->form_u0)
      return set_error(GBFEM_ERR_INVALID, "gbfem_operator_jacobian: jacobian was created for another operator");
    const size_t bytes = size_t(op->ndofs) * (op->precision == GBFEM_F64 ? 8 : 4);
    GBFEM_CUDA_TRY(cudaMemcpyAsync(jac->form_u0, u, bytes, cudaMemcpyDeviceToDevice, static_cast<cudaStream_t>(stream)));
    return GBFEM_OK;
  }
  if (!jac->jac_points) return set_error(GBFEM_ERR_INVALID, "gbfem_operator_jacobian: jacobian has no linearisation storage");
  jac->react[0] = op->react[0];
  jac->react[1] = op->react[1];
  jac->react[2] = op->react[2];
  return reaction_launch(op, 1, u, nullptr, jac->jac_points, 0, op->ncells, 0, static_cast<cudaStream_t>(stream));
}

}  // extern "C"
