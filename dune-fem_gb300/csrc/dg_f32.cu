// FP32 instantiations of the DG apply kernel (the inner-solve precision of
// the mixed-precision path).
#include <type_traits>

#include "dg_cell_kernel.cuh"
#include "dg_launch.cuh"

namespace gbfem {
int dg_launch_f32(const DgArgsT<float>& a, const DgTablesT<float>& t, int n, int q, bool kappa,
                  cudaStream_t s) {
  return dg_launch<float>(a, t, n, q, kappa, s);
}
int dg_const_launch_f32(const DgArgsT<float>& a, const DgConstTablesT<float>& t, int n, float* traces, int phase,
                        cudaStream_t s, float* ucopy) {
  return dg_const_launch<float>(a, t, n, traces, phase, s, ucopy);
}
// One-kernel closed form (dg_cell_kernel.cuh) for n <= 4 over the whole grid.
template <int N, bool ADV, bool KC>
static int dg_cell_launch_one(const DgArgsT<float>& a, const DgConstTablesT<float>& t, cudaStream_t s) {
  auto kern = dg_cell_kernel<N, ADV, KC>;
  constexpr size_t smem = CellSlots<N>::BYTES;
  GBFEM_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem)));
  const long long nbx = (a.nc[0] + kCellBX - 1) / kCellBX, nby = (a.nc[1] + kCellBY - 1) / kCellBY,
                  nbz = (a.nc[2] + kCellBZ - 1) / kCellBZ;
  const long long blocks = nbx * nby * nbz;
  if (blocks <= 0) return GBFEM_OK;
  if (blocks > 2147483647LL) return set_error(GBFEM_ERR_INVALID, "dg apply: grid too large");
  kern<<<unsigned(blocks), kCellThreads, smem, s>>>(a, t);
  GBFEM_CUDA_TRY(cudaGetLastError());
  return GBFEM_OK;
}

bool dg_cell_supported(int n) { return n >= 2 && n <= 4; }

int dg_cell_launch_f32(const DgArgsT<float>& a, const DgConstTablesT<float>& t, int n, cudaStream_t s) {
  const bool kc = a.kcell != nullptr, adv = a.advect != 0;
#define GBFEM_CELL_CASE(NN)                                              \
  if (n == NN) {                                                         \
    if (kc) return dg_cell_launch_one<NN, false, true>(a, t, s);         \
    if (adv) return dg_cell_launch_one<NN, true, false>(a, t, s);        \
    return dg_cell_launch_one<NN, false, false>(a, t, s);                \
  }
  GBFEM_CELL_CASE(2)
  GBFEM_CELL_CASE(3)
  GBFEM_CELL_CASE(4)
#undef GBFEM_CELL_CASE
  return set_error(GBFEM_ERR_NOT_IMPLEMENTED, "dg apply: one-kernel closed form needs p <= 3");
}

int dg_kappa_points_f32(const float* kappa, float* kq, float* kf, long long ncells, const DgTablesT<float>& t, int n,
                         int q, cudaStream_t s) {
  return dg_kappa_points<float>(kappa, kq, kf, ncells, t, n, q, s);
}
}  // namespace gbfem
