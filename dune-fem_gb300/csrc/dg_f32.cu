// FP32 instantiations of the DG apply kernel (the inner-solve precision of
// the mixed-precision path).
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
int dg_kappa_points_f32(const float* kappa, float* kq, float* kf, long long ncells, const DgTablesT<float>& t, int n,
                         int q, cudaStream_t s) {
  return dg_kappa_points<float>(kappa, kq, kf, ncells, t, n, q, s);
}
}  // namespace gbfem
