// Definition of the opaque preconditioner handle.
#pragma once
#include <cuda_runtime.h>

#include "../../include/gbfem.h"

namespace gbfem {

enum class PcKind { Diagonal = 1, BlockJacobi = 2, External = 3 };

int precond_apply(const struct ::gbfem_preconditioner_s* pc, const void* r, void* z, cudaStream_t s);

}  // namespace gbfem

struct gbfem_preconditioner_s {
  gbfem::PcKind kind = gbfem::PcKind::Diagonal;
  int precision = GBFEM_F64;
  long long n = 0;
  int nloc = 1;
  void* data = nullptr;  // diagonal inverse or block inverses
  bool owns_data = true;
  int storage = GBFEM_F64;   // block Jacobi: GBFEM_F64, GBFEM_F32 or GBFEM_F16 (scaled) blocks
  float* scales = nullptr;   // GBFEM_F16 storage: one scale per block
  // External (e.g. the learned preconditioner): z = P(r)
  int (*ext_apply)(void* ctx, const void* r, void* z, cudaStream_t s) = nullptr;
  void (*ext_destroy)(void* ctx) = nullptr;
  void* ext_ctx = nullptr;
  // Flexible solvers switch to this preconditioner when the iteration with
  // this one stagnates (the learned preconditioner's block-Jacobi fallback).
  struct gbfem_preconditioner_s* fallback = nullptr;
};
