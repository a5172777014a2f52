// Definition of the opaque preconditioner handle.
#pragma once
#include <cuda_runtime.h>

#include <vector>

#include "../../include/gbfem.h"

namespace gbfem {

enum class PcKind { Diagonal = 1, BlockJacobi = 2, External = 3, Sor = 4, ScaledBlock = 5 };

int precond_apply(const struct ::gbfem_preconditioner_s* pc, const void* r, void* z, cudaStream_t s);
// Jacobi / Gauss-Seidel / SOR / SSOR sweeps over an assembled operator (sor.cu)
int sor_apply(const struct ::gbfem_preconditioner_s* pc, const void* r, void* z, cudaStream_t s);
// scaled block Jacobi on the tensor cores (sb_tc.cu): set-up from the
// (type, start, count) tiles, and the apply
int sb_tc_setup(struct ::gbfem_preconditioner_s* pc, const std::vector<int>& tiles3, int nb, cudaStream_t s);
int sb_tc_apply(const struct ::gbfem_preconditioner_s* pc, const float* kcell, const float* r, float* z,
                cudaStream_t s);

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
  // Sor (and ScaledBlock: the cellwise-kappa operator): the operator (not owned), method (GBFEM_SMOOTHER_*),
  // sweeps, relaxation, cells grouped by level x+y+z with the level offsets,
  // and the previous iterate of Jacobi; data holds 1/diag
  const struct gbfem_operator_s* sor_op = nullptr;
  int sor_method = 0, sor_sweeps = 1;
  double sor_relax = 1.0;
  int* sor_cells = nullptr;
  void* sor_tmp = nullptr;
  std::vector<long long> sor_level_offsets;
  // ScaledBlock: sor_cells holds the cells sorted by boundary type; tiles of
  // (type, start, count) into it
  int* sb_tiles = nullptr;
  long long sb_ntiles = 0;
  // ScaledBlock on the tensor cores: tiles without padding, A_hi | A_lo
  // images per type, the kernel's status word (1 = a wait timed out)
  int sb_engine = GBFEM_SB_ENGINE_TENSOR;
  int* sb_tc_tiles = nullptr;
  int sb_tc_ntiles = 0;
  int sb_tc_wide = 0;  // 64-cell tiles with K = 64 (blocks of up to 64 dofs)
  void* sb_tc_img = nullptr;
  int* sb_tc_status = nullptr;
};
