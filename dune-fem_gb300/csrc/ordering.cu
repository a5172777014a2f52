// Local dof orderings of the tensor Legendre DG space.
//
// The library's layout is the reference's non-hierarchical one: local index
// i0 n^2 + i1 n + i2 with i0 the x-degree (space/shapefunctionset/
// legendre.hh:168-193, DefaultFactory::fill).  The hierarchical variant (the
// Python default dglegendre(hierarchical=True)) sorts the same shape
// functions by maximal degree, then lexicographically by (i0, i1, i2)
// (LegendreShapeFunctionSet::Compare, legendre.hh:236-249, sorted at
// :294-299).  The comparison is a strict total order, so the permutation is
// unique.  gbfem_dg_permute converts whole dof vectors on the device.
#include <cuda_runtime.h>
#include <algorithm>
#include <array>
#include <vector>

#include "blas.cuh"
#include "gbfem_internal.cuh"

namespace gbfem {

constexpr int kMaxLocal = 125;  // (p+1)^3 for p <= 4

struct Perm {
  int p[kMaxLocal];
};

static int hierarchical_permutation(int order, int dim, int* perm) {
  const int n = order + 1;
  int nloc = 1;
  for (int d = 0; d < dim; ++d) nloc *= n;
  std::vector<std::array<int, 3>> idx(nloc);
  for (int l = 0; l < nloc; ++l) {
    int r = l;
    std::array<int, 3> m{0, 0, 0};
    for (int d = dim - 1; d >= 0; --d) {
      m[d] = r % n;
      r /= n;
    }
    idx[l] = m;
  }
  std::vector<int> order_of(nloc);
  for (int l = 0; l < nloc; ++l) order_of[l] = l;
  auto maxdeg = [&](int l) { return std::max(idx[l][0], std::max(idx[l][1], idx[l][2])); };
  std::sort(order_of.begin(), order_of.end(), [&](int a, int b) {
    if (maxdeg(a) != maxdeg(b)) return maxdeg(a) < maxdeg(b);
    return std::lexicographical_compare(idx[a].begin(), idx[a].begin() + dim, idx[b].begin(), idx[b].begin() + dim);
  });
  for (int h = 0; h < nloc; ++h) perm[h] = order_of[h];
  return nloc;
}

// to_hier: out[c][h] = in[c][perm[h]];  else out[c][perm[h]] = in[c][h]
template <typename T>
__global__ void k_permute(long long ncells, int nloc, int to_hier, const T* __restrict__ in, T* __restrict__ out,
                          const __grid_constant__ Perm perm) {
  const long long total = ncells * nloc;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total;
       e += (long long)gridDim.x * blockDim.x) {
    const long long c = e / nloc;
    const int h = int(e - c * nloc);
    if (to_hier) out[e] = in[c * nloc + perm.p[h]];
    else out[c * nloc + perm.p[h]] = in[e];
  }
}

template <typename T>
__global__ void k_cell_means(long long ncells, int nloc, const T* __restrict__ in, T* __restrict__ out) {
  for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < ncells; c += (long long)gridDim.x * blockDim.x)
    out[c] = in[c * nloc];
}

}  // namespace gbfem

using namespace gbfem;

extern "C" {

int gbfem_legendre_hierarchical_permutation(int order, int dim, int* perm) {
  if (!perm || order < 0 || order > 4 || dim < 1 || dim > 3)
    return set_error(GBFEM_ERR_INVALID, "gbfem_legendre_hierarchical_permutation: invalid argument");
  hierarchical_permutation(order, dim, perm);
  return GBFEM_OK;
}

int gbfem_dg_permute(int precision, int64_t ncells, int order, int to_hierarchical, const void* in, void* out,
                     void* stream) {
  if (!in || !out || in == out || order < 0 || order > 4 || ncells < 0)
    return set_error(GBFEM_ERR_INVALID, "gbfem_dg_permute: invalid argument (in and out must differ)");
  Perm perm{};
  const int nloc = hierarchical_permutation(order, 3, perm.p);
  const long long n = ncells * nloc;
  if (n == 0) return GBFEM_OK;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (precision == GBFEM_F64)
    k_permute<double><<<stream_grid(n), 256, 0, s>>>(ncells, nloc, to_hierarchical, static_cast<const double*>(in),
                                                     static_cast<double*>(out), perm);
  else if (precision == GBFEM_F32)
    k_permute<float><<<stream_grid(n), 256, 0, s>>>(ncells, nloc, to_hierarchical, static_cast<const float*>(in),
                                                    static_cast<float*>(out), perm);
  else
    return set_error(GBFEM_ERR_INVALID, "gbfem_dg_permute: precision");
  GBFEM_CUDA_TRY(cudaGetLastError());
  return GBFEM_OK;
}

int gbfem_dg_cell_means(int precision, int64_t ncells, int order, const void* in, void* out, void* stream) {
  if (!in || !out || order < 0 || order > 4 || ncells < 0)
    return set_error(GBFEM_ERR_INVALID, "gbfem_dg_cell_means: invalid argument");
  const int nloc = (order + 1) * (order + 1) * (order + 1);
  if (ncells == 0) return GBFEM_OK;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (precision == GBFEM_F64)
    k_cell_means<double><<<stream_grid(ncells), 256, 0, s>>>(ncells, nloc, static_cast<const double*>(in),
                                                            static_cast<double*>(out));
  else
    k_cell_means<float><<<stream_grid(ncells), 256, 0, s>>>(ncells, nloc, static_cast<const float*>(in),
                                                           static_cast<float*>(out));
  GBFEM_CUDA_TRY(cudaGetLastError());
  return GBFEM_OK;
}

}  // extern "C"
