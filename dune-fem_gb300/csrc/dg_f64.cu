// FP64 instantiations of the DG apply kernel.
#include "dg_launch.cuh"

namespace gbfem {
int dg_launch_f64(const DgArgsT<double>& a, const DgTablesT<double>& t, int n, int q, bool kappa,
                  cudaStream_t s) {
  return dg_launch<double>(a, t, n, q, kappa, s);
}
int dg_const_launch_f64(const DgArgsT<double>& a, const DgConstTablesT<double>& t, int n, double* traces, int phase,
                        cudaStream_t s, double* ucopy) {
  return dg_const_launch<double>(a, t, n, traces, phase, s, ucopy);
}
int dg_kappa_points_f64(const double* kappa, double* kq, double* kf, long long ncells, const DgTablesT<double>& t, int n,
                         int q, cudaStream_t s) {
  return dg_kappa_points<double>(kappa, kq, kf, ncells, t, n, q, s);
}
}  // namespace gbfem
