// Instantiation and launch of dg_apply_kernel for the supported (n, q)
// pairs: n = p+1 in 2..5, q in {p+1, p+2}.
#pragma once
#include "dg_const_kernel.cuh"
#include "dg_kernel.cuh"
#include "gbfem_internal.cuh"

namespace gbfem {

#ifndef GBFEM_QUAD_CPB_MAX_F32
#define GBFEM_QUAD_CPB_MAX_F32 8
#endif
#ifndef GBFEM_QUAD_CPB_MAX_F64
#define GBFEM_QUAD_CPB_MAX_F64 8
#endif

template <typename T, int N, int Q, bool KAPPA>
int dg_launch_one(const DgArgsT<T>& args, const DgTablesT<T>& tabs, cudaStream_t stream) {
  // Cells per CTA: as many as fit ~100 KB of shared memory, at most
  // GBFEM_QUAD_CPB_MAX_F32 / _F64 (default 8); FP32 uses 32 threads per cell,
  // FP64 256 threads per CTA.
  constexpr int PER_CELL = DgSmem<N, Q, KAPPA, 1>::PER_CELL;
  constexpr int CPB0 = (100 * 1024) / (PER_CELL * int(sizeof(T)));
  constexpr int CAP = sizeof(T) == 4 ? GBFEM_QUAD_CPB_MAX_F32 : GBFEM_QUAD_CPB_MAX_F64;
  constexpr int CPB1 = CPB0 >= 8 ? 8 : (CPB0 >= 4 ? 4 : (CPB0 >= 2 ? 2 : 1));
  constexpr int CPB = CPB1 < CAP ? CPB1 : CAP;
  constexpr int THREADS = sizeof(T) == 4 ? 32 * CPB : 256;
  const size_t smem = size_t(DgSmem<N, Q, KAPPA, CPB>::TOTAL) * sizeof(T);
  auto kern = dg_apply_kernel<T, N, Q, KAPPA, CPB>;
  GBFEM_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem)));
  constexpr int N3 = N * N * N;
  const long long ucount = args.cell_count > 0 ? args.cell_count : args.ncells;
  const long long nvirt = args.unit_mode ? ucount * (args.unit_mode == 3 ? 6 * N3 : N3) : ucount;
  const long long blocks = (nvirt + CPB - 1) / CPB;
  if (blocks <= 0) return GBFEM_OK;
  if (blocks > 2147483647LL) return set_error(GBFEM_ERR_INVALID, "dg apply: grid too large");
  kern<<<unsigned(blocks), THREADS, smem, stream>>>(args, tabs);
  GBFEM_CUDA_TRY(cudaGetLastError());
  return GBFEM_OK;
}

template <typename T>
int dg_launch(const DgArgsT<T>& args, const DgTablesT<T>& tabs, int n, int q, bool kappa, cudaStream_t stream) {
#define GBFEM_DG_CASE(NN, QQ)                                                    \
  if (n == NN && q == QQ)                                                        \
    return kappa ? dg_launch_one<T, NN, QQ, true>(args, tabs, stream)            \
                 : dg_launch_one<T, NN, QQ, false>(args, tabs, stream);
  GBFEM_DG_CASE(2, 2)
  GBFEM_DG_CASE(2, 3)
  GBFEM_DG_CASE(3, 3)
  GBFEM_DG_CASE(3, 4)
  GBFEM_DG_CASE(4, 4)
  GBFEM_DG_CASE(4, 5)
  GBFEM_DG_CASE(5, 5)
  GBFEM_DG_CASE(5, 6)
#undef GBFEM_DG_CASE
  return set_error(GBFEM_ERR_NOT_IMPLEMENTED, "dg apply: unsupported (p, q)");
}

// phase bit 1: traces of the cells [cell_begin, cell_begin + count); bit 2:
// the apply of those cells (reads the traces of their neighbours, which must
// be current).  count = cell_count, 0 = all cells.
template <typename T, int N>
int dg_const_launch_one(const DgArgsT<T>& args, const DgConstTablesT<T>& tabs, T* traces, int phase,
                        cudaStream_t stream, T* ucopy) {
  constexpr int CPB = N <= 2 ? 32 : (N <= 4 ? 16 : 8);
  const long long count = args.cell_count > 0 ? args.cell_count : args.ncells;
  const long long blocks = (count + CPB - 1) / CPB;
  if (blocks <= 0) return GBFEM_OK;
  if (blocks > 2147483647LL) return set_error(GBFEM_ERR_INVALID, "dg apply: grid too large");
  if (phase & 1) {
    const long long titems = count * 3 * N * N;
    long long tblocks = (titems + 255) / 256;
    if (tblocks > 152LL * 32) tblocks = 152LL * 32;
    if (args.kcell)
      dg_trace_kernel<T, N, true><<<unsigned(tblocks), 256, 0, stream>>>(args.u, traces, args.cell_begin, count,
                                                                         tabs, ucopy);
    else
      dg_trace_kernel<T, N, false><<<unsigned(tblocks), 256, 0, stream>>>(args.u, traces, args.cell_begin, count,
                                                                          tabs, ucopy);
  }
  if (phase & 2) {
    if (args.kcell)
      dg_const_kernel<T, N, CPB, false, true><<<unsigned(blocks), 256, 0, stream>>>(args, traces, tabs);
    else if (args.advect)
      dg_const_kernel<T, N, CPB, true><<<unsigned(blocks), 256, 0, stream>>>(args, traces, tabs);
    else
      dg_const_kernel<T, N, CPB, false><<<unsigned(blocks), 256, 0, stream>>>(args, traces, tabs);
  }
  GBFEM_CUDA_TRY(cudaGetLastError());
  return GBFEM_OK;
}

template <typename T>
int dg_const_launch(const DgArgsT<T>& args, const DgConstTablesT<T>& tabs, int n, T* traces, int phase,
                    cudaStream_t stream, T* ucopy = nullptr) {
  switch (n) {
    case 2: return dg_const_launch_one<T, 2>(args, tabs, traces, phase, stream, ucopy);
    case 3: return dg_const_launch_one<T, 3>(args, tabs, traces, phase, stream, ucopy);
    case 4: return dg_const_launch_one<T, 4>(args, tabs, traces, phase, stream, ucopy);
    case 5: return dg_const_launch_one<T, 5>(args, tabs, traces, phase, stream, ucopy);
  }
  return set_error(GBFEM_ERR_NOT_IMPLEMENTED, "dg apply: unsupported order");
}

template <typename T, int N, int Q>
int dg_kappa_points_one(const T* kappa, T* kq, T* kf, long long ncells, const DgTablesT<T>& tabs,
                        cudaStream_t stream) {
  const long long total = ncells * (Q * Q * Q + 6 * Q * Q);
  long long blocks = (total + 255) / 256;
  if (blocks > 152LL * 64) blocks = 152LL * 64;
  if (blocks < 1) return GBFEM_OK;
  dg_kappa_points_kernel<T, N, Q><<<unsigned(blocks), 256, 0, stream>>>(kappa, kq, kf, ncells, tabs);
  GBFEM_CUDA_TRY(cudaGetLastError());
  return GBFEM_OK;
}

template <typename T>
int dg_kappa_points(const T* kappa, T* kq, T* kf, long long ncells, const DgTablesT<T>& tabs, int n, int q,
                    cudaStream_t stream) {
#define GBFEM_KP_CASE(NN, QQ) \
  if (n == NN && q == QQ) return dg_kappa_points_one<T, NN, QQ>(kappa, kq, kf, ncells, tabs, stream);
  GBFEM_KP_CASE(2, 2)
  GBFEM_KP_CASE(2, 3)
  GBFEM_KP_CASE(3, 3)
  GBFEM_KP_CASE(3, 4)
  GBFEM_KP_CASE(4, 4)
  GBFEM_KP_CASE(4, 5)
  GBFEM_KP_CASE(5, 5)
  GBFEM_KP_CASE(5, 6)
#undef GBFEM_KP_CASE
  return set_error(GBFEM_ERR_NOT_IMPLEMENTED, "dg kappa points: unsupported (p, q)");
}

}  // namespace gbfem
