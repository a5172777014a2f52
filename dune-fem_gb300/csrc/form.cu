// General DG forms compiled at run time (form_kernel.cuh): the operator made
// from a cubin the Python package generates, its apply, and the dual-number
// linearisation behind its Jacobian (apply, diagonal blocks, diagonal,
// neighbour couplings).  ≙ a GalerkinOperator / DifferentiableGalerkinOperator
// over UFL-generated integrands (schemes/galerkin.hh:1383-1504, 1548-1643;
// python/dune/models/integrands/ufl.py:197-348).
#include <cuda_runtime.h>
#include <cstring>
#include <string>

#include "form_kernel.cuh"
#include "gbfem_internal.cuh"
#include "operator_impl.hpp"

namespace gbfem {

namespace {

constexpr int kFormThreads = 128;
constexpr int kFormMaxComponents = 4;

template <typename R>
void fill_form_args(const gbfem_operator_s* op, form::FormArgs<R>* a) {
  std::memset(a, 0, sizeof(*a));
  const gbfem_dg_desc& d = op->dg;
  double h[3], vol = 1.0;
  for (int k = 0; k < 3; ++k) {
    a->nc[k] = d.grid.cells[k];
    a->periodic[k] = d.grid.periodic[k];
    h[k] = (d.grid.upper[k] - d.grid.lower[k]) / d.grid.cells[k];
    vol *= h[k];
  }
  a->ncells = op->ncells;
  a->detK = R(vol);
  for (int k = 0; k < 3; ++k) {
    a->lower[k] = R(d.grid.lower[k]);
    a->h[k] = R(h[k]);
    a->invh[k] = R(1.0 / h[k]);
    a->faceA[k] = R(vol / h[k]);
    a->sigma[k] = R(d.penalty / h[k]);  // h_F = |K| / |F| = h_d
  }
}

long long form_smem(const gbfem_operator_s* op) {
  const int rb = op->precision == GBFEM_F64 ? 8 : 4;
  const int cpb = form::form_cells_per_block(op->q, op->form_m);
  // the linearised kernel holds two reals per value
  return form::form_smem_bytes(op->n, op->q, op->form_m, cpb, 2 * rb, rb);
}

template <typename R>
int form_launch(const gbfem_operator_s* op, int mode, const void* u, const void* du, void* w, void* blocks,
                long long cell_begin, long long cell_count, cudaStream_t s) {
  form::FormArgs<R> a;
  fill_form_args(op, &a);
  a.u = static_cast<const R*>(u);
  a.du = static_cast<const R*>(du);
  a.w = static_cast<R*>(w);
  a.blocks = static_cast<R*>(blocks);
  a.mode = mode;
  a.cell_begin = cell_begin;
  a.cell_count = cell_count;
  const DgTablesT<R>& t = op->precision == GBFEM_F64 ? reinterpret_cast<const DgTablesT<R>&>(op->tab64)
                                                    : reinterpret_cast<const DgTablesT<R>&>(op->tab32);
  DgTablesT<R> tabs = t;
  const long long count = cell_count > 0 ? cell_count : op->ncells - cell_begin;
  if (count <= 0) return GBFEM_OK;
  const long long vper = mode == 4 ? 6LL * op->nloc : (mode >= 2 ? op->nloc : 1);
  const int cpb = form::form_cells_per_block(op->q, op->form_m);
  const long long grid = (count * vper + cpb - 1) / cpb;
  if (grid > 2147483647LL) return set_error(GBFEM_ERR_INVALID, "form operator: grid too large");
  const int rb = int(sizeof(R));
  const long long smem = form::form_smem_bytes(op->n, op->q, op->form_m, cpb, mode == 0 ? rb : 2 * rb, rb);
  void* kernel = mode == 0 ? op->form_val : op->form_lin;
  void* args[] = {&a, &tabs};
  GBFEM_CUDA_TRY(cudaLaunchKernel(reinterpret_cast<const void*>(kernel), dim3(unsigned(grid)), dim3(kFormThreads),
                                  args, size_t(smem), s));
  return GBFEM_OK;
}

}  // namespace

int form_apply(const gbfem_operator_s* op, const void* u, void* w, cudaStream_t s, int unit_mode, void* blocks,
               long long cell_begin, long long cell_count) {
  // unit modes of dg_apply: 1 diagonal blocks, 2 diagonal, 3 neighbour couplings
  int mode;
  const void* point = op->form_u0;
  const void* dir = nullptr;
  if (unit_mode == 0) {
    if (op->form_jacobian) {
      mode = 1;
      dir = u;
    } else {
      mode = 0;
      point = u;
    }
  } else if (unit_mode == 1) {
    mode = 2;
  } else if (unit_mode == 2) {
    mode = 3;
    cell_begin = 0;
    cell_count = 0;
  } else if (unit_mode == 3) {
    mode = 4;
  } else {
    return set_error(GBFEM_ERR_INVALID, "form operator: unknown unit mode");
  }
  if (op->precision == GBFEM_F64)
    return form_launch<double>(op, mode, point, dir, w, blocks, cell_begin, cell_count, s);
  return form_launch<float>(op, mode, point, dir, w, blocks, cell_begin, cell_count, s);
}

}  // namespace gbfem

using namespace gbfem;

extern "C" {

int gbfem_form_operator_create(const gbfem_dg_desc* desc, int components, const char* cubin_path,
                               gbfem_operator* out) {
  if (!desc || !cubin_path || !out) return set_error(GBFEM_ERR_INVALID, "gbfem_form_operator_create: null argument");
  *out = nullptr;
  if (components < 1 || components > kFormMaxComponents)
    return set_error(GBFEM_ERR_NOT_IMPLEMENTED, "gbfem_form_operator_create: 1..4 components");
  if (desc->kappa || desc->kappa_cell)
    return set_error(GBFEM_ERR_INVALID, "gbfem_form_operator_create: coefficients belong in the form");
  gbfem_dg_desc d = *desc;
  d.algorithm = GBFEM_ALGO_QUADRATURE;  // no closed-form buffers
  GBFEM_TRY(gbfem_dg_operator_create(&d, out));
  gbfem_operator op = *out;
  op->form = 1;
  op->form_m = components;
  op->nloc = components * op->n * op->n * op->n;
  op->ndofs = op->ncells * op->nloc;
  op->nonlinear = 1;
  const std::string base = std::string("gbfem_form_") + (op->precision == GBFEM_F64 ? "f64" : "f32") + "_n" +
                           std::to_string(op->n) + "_q" + std::to_string(op->q) + "_m" + std::to_string(components);
  auto fail = [&](int rc) {
    (void)cudaGetLastError();  // the failed runtime call must not surface at the next launch check
    gbfem_operator_destroy(op);
    *out = nullptr;
    return rc;
  };
  cudaLibrary_t lib = nullptr;
  cudaError_t e = cudaLibraryLoadFromFile(&lib, cubin_path, nullptr, nullptr, 0, nullptr, nullptr, 0);
  if (e != cudaSuccess)
    return fail(set_cuda_error(e, (std::string("gbfem_form_operator_create: loading ") + cubin_path).c_str()));
  op->jit_lib = lib;
  cudaKernel_t kv = nullptr, kl = nullptr;
  e = cudaLibraryGetKernel(&kv, lib, (base + "_val").c_str());
  if (e == cudaSuccess) e = cudaLibraryGetKernel(&kl, lib, (base + "_lin").c_str());
  if (e != cudaSuccess)
    return fail(set_cuda_error(e, ("gbfem_form_operator_create: no kernels " + base +
                                   "_val/_lin in the cubin (compiled for another precision, order, "
                                   "quadrature or component count?)").c_str()));
  op->form_val = reinterpret_cast<void*>(kv);
  op->form_lin = reinterpret_cast<void*>(kl);
  const long long smem = form_smem(op);
  if (smem > 227 * 1024) return fail(set_error(GBFEM_ERR_NOT_IMPLEMENTED, "gbfem_form_operator_create: too large"));
  if (smem > 48 * 1024) {
    int dev = 0;
    e = cudaGetDevice(&dev);
    if (e == cudaSuccess)
      e = cudaKernelSetAttributeForDevice(kv, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem), dev);
    if (e == cudaSuccess)
      e = cudaKernelSetAttributeForDevice(kl, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem), dev);
    if (e != cudaSuccess) return fail(set_cuda_error(e, "gbfem_form_operator_create: shared memory"));
  }
  return GBFEM_OK;
}

int gbfem_operator_components(gbfem_operator op, int* components) {
  if (!op || !components) return set_error(GBFEM_ERR_INVALID, "gbfem_operator_components: null argument");
  *components = op->form ? op->form_m : 1;
  return GBFEM_OK;
}

}  // extern "C"
