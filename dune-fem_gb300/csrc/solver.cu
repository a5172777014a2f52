// Krylov inverse operators and preconditioners on device-resident dof
// vectors.
//
// The loops follow dune-fem's LinearSolver templates statement by statement
// (solver/linear/cg.hh:18-117, gmres.hh:116-299, bicgstab.hh:63-222) so the
// iteration counts and iterates match the reference's.  Only vector
// operations and scalar products run on the device; the Krylov scalars
// (alpha, beta, Givens rotations) are FP64 host values, as in the
// reference.  Each dot product is the deterministic two-pass FP64 reduction
// of blas.cu, read back with one stream synchronisation.  FCG and FGMRES
// (flexible variants for a preconditioner that changes between iterations,
// e.g. the learned one) follow Notay (2000) and Saad (1993).
#include <cuda_fp16.h>
#include <cuda_runtime.h>
#include <algorithm>
#include <chrono>
#include <climits>
#include <cmath>
#include <cstdio>
#include <new>
#include <string>
#include <type_traits>
#include <vector>

#include "blas.cuh"
#include "gbfem_internal.cuh"
#include "operator_impl.hpp"
#include "solver_impl.hpp"

namespace gbfem {

// ---------------------------------------------------------------- kernels --
template <typename T>
__global__ void k_axpby(long long n, double a, const T* __restrict__ x, double b, T* __restrict__ y) {
  // y = a*x + b*y
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    y[i] = T(a) * x[i] + T(b) * y[i];
}
template <typename T>
__global__ void k_axpbypcz(long long n, double a, const T* __restrict__ x, double b, const T* __restrict__ y,
                           double c, T* __restrict__ z) {
  // z = a*x + b*y + c*z
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    z[i] = T(a) * x[i] + T(b) * y[i] + T(c) * z[i];
}
template <typename T>
__global__ void k_diag_apply(long long n, const T* __restrict__ dinv, const T* __restrict__ r, T* __restrict__ z) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    z[i] = r[i] * dinv[i];
}
template <typename T>
__global__ void k_diag_invert(long long n, T* __restrict__ d) {
  // DiagonalPreconditionerBase: near-zero entries become 1 (diagonalpreconditioner.hh:94-99)
  const T eps = T(16) * (sizeof(T) == 8 ? T(2.220446049250313e-16) : T(1.1920929e-07));
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const T v = d[i];
    d[i] = (v < eps && v > -eps) ? T(1) : T(1) / v;
  }
}

// In-place Gauss-Jordan inversion with partial pivoting of one nb x nb block
// per CTA, in FP64 shared memory; result stored in TO.
template <typename TI, typename TO>
__global__ void k_block_invert(const TI* __restrict__ blocks, TO* __restrict__ inv, int nb, long long nblocks,
                               int* __restrict__ singular, float* __restrict__ scales) {
  extern __shared__ __align__(16) unsigned char smraw[];
  double* a = reinterpret_cast<double*>(smraw);  // nb*nb
  int* perm = reinterpret_cast<int*>(a + nb * nb);  // nb
  __shared__ int s_piv;
  const long long b = blockIdx.x;
  if (b >= nblocks) return;
  const TI* src = blocks + b * nb * nb;
  for (int e = threadIdx.x; e < nb * nb; e += blockDim.x) a[e] = double(src[e]);
  __syncthreads();
  for (int k = 0; k < nb; ++k) {
    if (threadIdx.x < 32) {
      // warp-parallel partial pivoting: largest |a[i][k]|, ties to the smallest i
      int p = nb;
      double best = -1.0;
      for (int i = k + int(threadIdx.x); i < nb; i += 32) {
        const double v = fabs(a[i * nb + k]);
        if (v > best) { best = v; p = i; }
      }
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        const double ob = __shfl_down_sync(0xffffffffu, best, o);
        const int op = __shfl_down_sync(0xffffffffu, p, o);
        if (ob > best || (ob == best && op < p)) { best = ob; p = op; }
      }
      if (threadIdx.x == 0) {
        if (p >= nb) p = k;  // only NaN in the column: keep the row, flag below
        s_piv = p;
        perm[k] = p;
        if (!(best > 0.0)) atomicExch(singular, 1);
      }
    }
    __syncthreads();
    const int p = s_piv;
    if (p != k)
      for (int j = threadIdx.x; j < nb; j += blockDim.x) {
        const double t = a[k * nb + j];
        a[k * nb + j] = a[p * nb + j];
        a[p * nb + j] = t;
      }
    __syncthreads();
    const double piv = a[k * nb + k];
    const double ipiv = piv != 0.0 ? 1.0 / piv : 0.0;
    __syncthreads();
    // scale pivot row; a[k][k] becomes 1/piv
    for (int j = threadIdx.x; j < nb; j += blockDim.x) a[k * nb + j] = (j == k) ? ipiv : a[k * nb + j] * ipiv;
    __syncthreads();
    // eliminate column k from all other rows
    for (int e = threadIdx.x; e < nb * nb; e += blockDim.x) {
      const int i = e / nb, j = e - i * nb;
      if (i == k) continue;
      const double f = a[i * nb + k];
      if (j == k) continue;
      a[e] -= f * a[k * nb + j];
    }
    __syncthreads();
    for (int i = threadIdx.x; i < nb; i += blockDim.x)
      if (i != k) a[i * nb + k] = -a[i * nb + k] * ipiv;
    __syncthreads();
  }
  // undo the row interchanges as column interchanges, last first
  for (int k = nb - 1; k >= 0; --k) {
    const int p = perm[k];
    if (p != k)
      for (int i = threadIdx.x; i < nb; i += blockDim.x) {
        const double t = a[i * nb + k];
        a[i * nb + k] = a[i * nb + p];
        a[i * nb + p] = t;
      }
    __syncthreads();
  }
  // stored transposed (column j contiguous) for the coalesced apply
  TO* dst = inv + b * nb * nb;
  if constexpr (std::is_same<TO, __half>::value) {
    // FP16 storage: entries / max|entry| of the block, the max as an FP32 scale
    __shared__ double s_max[32];
    double m = 0.0;
    for (int e = threadIdx.x; e < nb * nb; e += blockDim.x) m = fmax(m, fabs(a[e]));
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_down_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0) s_max[threadIdx.x >> 5] = m;
    __syncthreads();
    if (threadIdx.x == 0) {
      double mm = 0.0;
      for (int w = 0; w < int(blockDim.x >> 5); ++w) mm = fmax(mm, s_max[w]);
      s_max[0] = mm > 0.0 ? mm : 1.0;
      scales[b] = float(s_max[0]);
    }
    __syncthreads();
    // rows of the transposed block padded to an even length ld (pad = 0), so
    // the apply reads two rows per __half2 load
    const int ld = nb + (nb & 1);
    TO* dsth = inv + b * (long long)nb * ld;
    const double inv_scale = 1.0 / s_max[0];
    for (int e = threadIdx.x; e < nb * ld; e += blockDim.x) {
      const int j = e / ld, i = e - j * ld;
      dsth[e] = i < nb ? __float2half_rn(float(a[i * nb + j] * inv_scale)) : __float2half_rn(0.0f);
    }
  } else {
    for (int e = threadIdx.x; e < nb * nb; e += blockDim.x) {
      const int i = e / nb, j = e - i * nb;
      dst[j * nb + i] = TO(a[e]);
    }
  }
}

// FP16 blocks with per-block scale, FP32 vectors: z_K = s_K (Binv_K / s_K) r_K.
// The transposed blocks have rows of even length ld = nb + (nb & 1); a thread
// computes rows 2t and 2t+1 from __half2 loads (ld / 2 threads per cell), so a
// warp load is 128 bytes as in the FP32 apply.
__global__ void k_block_apply_h(const __half* __restrict__ binvT, const float* __restrict__ scales,
                                const float* __restrict__ r, float* __restrict__ z, int nb, long long ncells, int cpb) {
  extern __shared__ __align__(16) unsigned char smraw[];
  float* rs = reinterpret_cast<float*>(smraw);  // [cpb][nb]
  const int ld = nb + (nb & 1), tpc = ld / 2;
  const long long c0 = (long long)blockIdx.x * cpb;
  const int ncell = int(ncells - c0 < cpb ? ncells - c0 : cpb);
  for (int e = threadIdx.x; e < ncell * nb; e += blockDim.x) rs[e] = r[c0 * nb + e];
  __syncthreads();
  const int lc = threadIdx.x / tpc, t = threadIdx.x - lc * tpc;
  if (lc >= ncell) return;
  const __half2* B = reinterpret_cast<const __half2*>(binvT + (c0 + lc) * (long long)nb * ld) + t;
  const float* rc = rs + lc * nb;
  float a0 = 0.0f, a1 = 0.0f;
  for (int j = 0; j < nb; ++j) {
    const float2 bb = __half22float2(B[(long long)j * (ld / 2)]);
    a0 = fmaf(bb.x, rc[j], a0);
    a1 = fmaf(bb.y, rc[j], a1);
  }
  const float sc = scales[c0 + lc];
  const int i = 2 * t;
  z[(c0 + lc) * nb + i] = a0 * sc;
  if (i + 1 < nb) z[(c0 + lc) * nb + i + 1] = a1 * sc;
}

// z_K = Binv_K r_K with Binv_K stored transposed (binvT[K][j][i]): one thread
// per row i, CPB cells per CTA, r_K broadcast from shared memory.  For fixed j
// the threads of a cell read consecutive addresses, so the block stream is
// coalesced; the sum over j has a fixed order.
template <typename T>
__global__ void k_block_apply(const T* __restrict__ binvT, const T* __restrict__ r, T* __restrict__ z, int nb,
                              long long ncells, int cpb) {
  extern __shared__ __align__(16) unsigned char smraw[];
  T* rs = reinterpret_cast<T*>(smraw);  // [cpb][nb]
  const long long c0 = (long long)blockIdx.x * cpb;
  const int ncell = int(ncells - c0 < cpb ? ncells - c0 : cpb);
  for (int e = threadIdx.x; e < ncell * nb; e += blockDim.x) rs[e] = r[c0 * nb + e];
  __syncthreads();
  const int lc = threadIdx.x / nb, i = threadIdx.x - lc * nb;
  if (lc >= ncell) return;
  const T* B = binvT + (c0 + lc) * (long long)nb * nb + i;
  const T* rc = rs + lc * nb;
  T acc = T(0);
  for (int j = 0; j < nb; ++j) acc = fma(B[(long long)j * nb], rc[j], acc);
  z[(c0 + lc) * nb + i] = acc;
}

// Scaled shared-block Jacobi of an operator with a constant kappa per cell
// (no mass, no advection): z_c = Hinv_t(c) r_c / kappa_c.  Hinv_t is the
// inverse diagonal block of the kappa = 1 operator for the cell's boundary
// type t (at most 27 per grid), stored transposed like the block-Jacobi
// blocks; one thread per row, cpb cells per CTA.
__device__ __forceinline__ int cell_type(long long c, const int* nc, const int* per) {
  const long long nxy = (long long)nc[0] * nc[1];
  const long long z = c / nxy, rem = c - z * nxy, y = rem / nc[0], x = rem - y * nc[0];
  const long long xyz[3] = {x, y, z};
  int t = 0, mul = 1;
  for (int d = 0; d < 3; ++d) {
    int td, md;
    if (per[d]) { td = 0; md = 2; }
    else if (nc[d] <= 2) { td = int(xyz[d]); md = nc[d]; }
    else { td = xyz[d] == 0 ? 0 : (xyz[d] == nc[d] - 1 ? 2 : 1); md = 3; }
    t += td * mul;
    mul *= md;
  }
  return t;
}

struct GridShape {
  int nc[3];
  int per[3];
};

__global__ void k_scaled_block_apply(const float* __restrict__ hinvT, const float* __restrict__ kcell,
                                     const float* __restrict__ r, float* __restrict__ z, int nb, long long ncells,
                                     int cpb, GridShape g) {
  extern __shared__ __align__(16) unsigned char smraw[];
  float* rs = reinterpret_cast<float*>(smraw);  // [cpb][nb]
  const long long c0 = (long long)blockIdx.x * cpb;
  const int ncell = int(ncells - c0 < cpb ? ncells - c0 : cpb);
  for (int e = threadIdx.x; e < ncell * nb; e += blockDim.x) rs[e] = r[c0 * nb + e];
  __syncthreads();
  const int lc = threadIdx.x / nb, i = threadIdx.x - lc * nb;
  if (lc >= ncell) return;
  const long long c = c0 + lc;
  const float* B = hinvT + (long long)cell_type(c, g.nc, g.per) * nb * nb + i;
  const float* rc = rs + lc * nb;
  float acc = 0.0f;
  for (int j = 0; j < nb; ++j) acc = fmaf(__ldg(B + (long long)j * nb), rc[j], acc);
  z[c * nb + i] = acc / kcell[c];
}

// The same on tiles of up to 32 cells of one boundary type (nb <= 128): the
// cells sorted by type at creation, each type's list cut into tiles (interior
// tiles are runs of consecutive cells) and padded with empty tiles to a
// multiple of kSbGroups, so that a quad of consecutive tiles has one type.
// One CTA per SM owns a contiguous range of quads and stages their type's
// inverse in shared memory (rows padded to 128) once, reloading it only where
// the type changes.  Its kSbGroups groups of 8 warps each take one tile of a
// quad: they gather the residuals of their next tile (transposed, [j][cell])
// with cp.async while the nb x 32 product of the current one runs with 4 x 4
// register tiles per thread, and stage the product back through shared
// memory so that each cell's nb results go out as one contiguous run.  A
// group synchronises on its own named barrier; the whole CTA only where the
// inverse changes.
constexpr int kSbTile = 32;
constexpr int kSbGroups = 4;
constexpr int kSbGroupThreads = 256;

__device__ __forceinline__ void sb_cp_async4(float* dst, const float* src) {
  const unsigned d = static_cast<unsigned>(__cvta_generic_to_shared(dst));
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(d), "l"(src) : "memory");
}
__device__ __forceinline__ void sb_cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void sb_cp_async_wait() {
  asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory");
}
// barrier 1 + g among the kSbGroupThreads threads of group g (0 is __syncthreads)
__device__ __forceinline__ void sb_group_sync(int g) {
  asm volatile("bar.sync %0, %1;\n" ::"r"(1 + g), "n"(kSbGroupThreads) : "memory");
}

__global__ void __launch_bounds__(kSbGroups * kSbGroupThreads, 1)
    k_scaled_block_apply_tiled(const float* __restrict__ hinvT, const float* __restrict__ kcell,
                               const int* __restrict__ cells, const int* __restrict__ tiles,
                               const float* __restrict__ r, float* __restrict__ z, int nb, int nquads) {
  extern __shared__ __align__(16) unsigned char smraw[];
  __shared__ float sInvK[kSbGroups][kSbTile];
  const int tid = threadIdx.x;
  const int g = tid / kSbGroupThreads, gt = tid - g * kSbGroupThreads;
  const int rstride = nb * kSbTile;  // a multiple of 32: every loop below keeps whole warps
  float* Hs = reinterpret_cast<float*>(smraw);      // [nb][128]  (transposed inverse: Hs[j][i])
  float* Rb = Hs + nb * 128 + g * 2 * rstride;      // this group's 2 x [nb][32]
  const int q0 = int((long long)blockIdx.x * nquads / gridDim.x);
  const int q1 = int((long long)(blockIdx.x + 1) * nquads / gridDim.x);
  if (q0 >= q1) return;  // the same for the whole CTA
  const int lane = tid & 31;
  // lane l holds the index of the tile's cell l; the others take it by shuffle
  auto lane_cell = [&](int t) {
    const int start = tiles[3 * t + 1], count = tiles[3 * t + 2];
    return lane < count ? cells[start + lane] : 0;
  };
  auto gather = [&](int t, float* R) {
    const int count = tiles[3 * t + 2];
    const int mine = lane_cell(t);
    for (int e = gt; e < rstride; e += kSbGroupThreads) {
      const int c = e / nb, j = e - c * nb;  // c < 32
      const int cell = __shfl_sync(0xffffffffu, mine, c);
      float* dst = R + j * kSbTile + c;
      if (c < count) sb_cp_async4(dst, r + (long long)cell * nb + j);
      else *dst = 0.0f;
    }
    sb_cp_async_commit();
  };
  gather(kSbGroups * q0 + g, Rb);
  int cur_type = -1;
  const int rg = gt & 31, cg = gt >> 5;  // rows 4 rg .. 4 rg + 3, tile cells 4 cg .. 4 cg + 3
  for (int q = q0; q < q1; ++q) {
    const int t = kSbGroups * q + g;
    float* R = Rb + ((q - q0) & 1) * rstride;
    const int type = tiles[3 * t], count = tiles[3 * t + 2];  // type: the same for the quad
    if (type != cur_type) {
      __syncthreads();  // every group is done with the previous inverse
      const float* Hg = hinvT + (long long)type * nb * nb;
      for (int e = tid; e < nb * 128; e += blockDim.x) {
        const int j = e >> 7, i = e & 127;
        Hs[e] = i < nb ? __ldg(Hg + (long long)j * nb + i) : 0.0f;
      }
      __syncthreads();
      cur_type = type;
    }
    const int mine = lane_cell(t);
    if (gt < kSbTile) sInvK[g][gt] = gt < count ? 1.0f / kcell[mine] : 0.0f;
    if (q + 1 < q1) {
      gather(t + kSbGroups, Rb + ((q + 1 - q0) & 1) * rstride);
      sb_cp_async_wait<1>();  // this tile's group is complete, the next one's may still run
    } else {
      sb_cp_async_wait<0>();
    }
    sb_group_sync(g);  // R and the inverse kappas of this tile are visible to the group
    float acc[4][4] = {};
    for (int j = 0; j < nb; ++j) {
      const float4 a = *reinterpret_cast<const float4*>(Hs + j * 128 + 4 * rg);
      const float4 b = *reinterpret_cast<const float4*>(R + j * kSbTile + 4 * cg);
      const float av[4] = {a.x, a.y, a.z, a.w}, bv[4] = {b.x, b.y, b.z, b.w};
#pragma unroll
      for (int ii = 0; ii < 4; ++ii)
#pragma unroll
        for (int cc = 0; cc < 4; ++cc) acc[ii][cc] = fmaf(av[ii], bv[cc], acc[ii][cc]);
    }
    sb_group_sync(g);  // every read of R done: it takes the results [cell][i]
#pragma unroll
    for (int cc = 0; cc < 4; ++cc)
#pragma unroll
      for (int ii = 0; ii < 4; ++ii) {
        const int i = 4 * rg + ii;
        if (i < nb) R[(4 * cg + cc) * nb + i] = acc[ii][cc] * sInvK[g][4 * cg + cc];
      }
    sb_group_sync(g);
    const int total = count * nb;
    for (int e0 = gt - lane; e0 < total; e0 += kSbGroupThreads) {  // warp-uniform bound
      const int e = e0 + lane, c = e / nb;
      const int cell = __shfl_sync(0xffffffffu, mine, c < kSbTile ? c : kSbTile - 1);
      if (e < total) z[(long long)cell * nb + (e - c * nb)] = R[e];
    }
    sb_group_sync(g);  // R and sInvK[g] are free for the gather after next and the next tile
  }
}

// SMs of the current device (152 on GB300), for persistent grids.
static int num_sms() {
  static int n = 0;
  if (n <= 0) {
    int dev = 0, v = 0;
    if (cudaGetDevice(&dev) == cudaSuccess && cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev) ==
                                                  cudaSuccess && v > 0)
      n = v;
    else
      n = 152;
  }
  return n;
}

// ------------------------------------------------------------ vector ops --
struct Ctx {
  int prec;
  long long n;
  cudaStream_t s;
  double* d_partial = nullptr;
  double* d_res = nullptr;
  double* h_res = nullptr;  // pinned
  int op_applies = 0, pc_applies = 0;
  int setup(int precision, long long nn, cudaStream_t st) {
    prec = precision;
    n = nn;
    s = st;
    GBFEM_CUDA_TRY(cudaMalloc(&d_partial, sizeof(double) * (size_t(kMaxDotPairs) * dot_num_partials(n) + 8)));
    GBFEM_CUDA_TRY(cudaMalloc(&d_res, sizeof(double) * kMaxDotPairs));
    GBFEM_CUDA_TRY(cudaMallocHost(&h_res, sizeof(double) * kMaxDotPairs));
    return GBFEM_OK;
  }
  // out[l] = xs[l] . ys[l] for l < k, one pass and one host synchronisation
  // per kMaxDotPairs pairs; each bitwise equal to dot(xs[l], ys[l])
  int multi_dot(int k, const void* const* xs, const void* const* ys, double* out) {
    for (int l0 = 0; l0 < k; l0 += kMaxDotPairs) {
      const int kk = k - l0 < kMaxDotPairs ? k - l0 : kMaxDotPairs;
      GBFEM_TRY(multi_dot_device(prec, n, kk, xs + l0, ys + l0, d_res, d_partial, s));
      GBFEM_CUDA_TRY(cudaMemcpyAsync(h_res, d_res, sizeof(double) * kk, cudaMemcpyDeviceToHost, s));
      GBFEM_CUDA_TRY(cudaStreamSynchronize(s));
      for (int l = 0; l < kk; ++l) out[l0 + l] = h_res[l];
    }
    return GBFEM_OK;
  }
  // y += sum_l a[l] xs[l], in order
  int multi_axpy(int k, const double* a, const void* const* xs, void* y) {
    for (int l0 = 0; l0 < k; l0 += kMaxDotPairs) {
      const int kk = k - l0 < kMaxDotPairs ? k - l0 : kMaxDotPairs;
      GBFEM_TRY(multi_axpy_device(prec, n, kk, a + l0, xs + l0, y, s));
    }
    return GBFEM_OK;
  }
  ~Ctx() {
    if (d_partial) cudaFree(d_partial);
    if (d_res) cudaFree(d_res);
    if (h_res) cudaFreeHost(h_res);
  }
  size_t bytes() const { return size_t(n) * (prec == GBFEM_F64 ? 8 : 4); }
  int dot(const void* x, const void* y, double* out) {
    GBFEM_TRY(dot_device(prec, n, x, y, d_res, d_partial, s));
    GBFEM_CUDA_TRY(cudaMemcpyAsync(h_res, d_res, sizeof(double), cudaMemcpyDeviceToHost, s));
    GBFEM_CUDA_TRY(cudaStreamSynchronize(s));
    *out = h_res[0];
    return GBFEM_OK;
  }
  // y = a*x + b*y
  int axpby(double a, const void* x, double b, void* y) {
    if (prec == GBFEM_F64)
      k_axpby<double><<<stream_grid(n), 256, 0, s>>>(n, a, (const double*)x, b, (double*)y);
    else
      k_axpby<float><<<stream_grid(n), 256, 0, s>>>(n, a, (const float*)x, b, (float*)y);
    GBFEM_CUDA_TRY(cudaGetLastError());
    return GBFEM_OK;
  }
  // z = a*x + b*y + c*z
  int axpbypcz(double a, const void* x, double b, const void* y, double c, void* z) {
    if (prec == GBFEM_F64)
      k_axpbypcz<double><<<stream_grid(n), 256, 0, s>>>(n, a, (const double*)x, b, (const double*)y, c, (double*)z);
    else
      k_axpbypcz<float><<<stream_grid(n), 256, 0, s>>>(n, a, (const float*)x, b, (const float*)y, c, (float*)z);
    GBFEM_CUDA_TRY(cudaGetLastError());
    return GBFEM_OK;
  }
  // x *= a (in place)
  int scal(double a, void* x) { return gbfem_scal(prec, n, a, x, s); }
  int copy(const void* x, void* y) {
    GBFEM_CUDA_TRY(cudaMemcpyAsync(y, x, bytes(), cudaMemcpyDeviceToDevice, s));
    return GBFEM_OK;
  }
  int clear(void* x) {
    GBFEM_CUDA_TRY(cudaMemsetAsync(x, 0, bytes(), s));
    return GBFEM_OK;
  }
};

struct Vecs {
  std::vector<void*> v;
  ~Vecs() {
    for (void* p : v) cudaFree(p);
  }
  int alloc(int k, size_t bytes) {
    for (int i = 0; i < k; ++i) {
      void* p = nullptr;
      GBFEM_CUDA_TRY(cudaMalloc(&p, bytes));
      v.push_back(p);
    }
    return GBFEM_OK;
  }
  void* operator[](int i) const { return v[i]; }
};

static bool finite(double x) { return std::isfinite(x); }

int precond_apply(const gbfem_preconditioner_s* pc, const void* r, void* z, cudaStream_t s) {
  const long long n = pc->n;
  switch (pc->kind) {
    case PcKind::Diagonal:
      if (pc->precision == GBFEM_F64)
        k_diag_apply<double><<<stream_grid(n), 256, 0, s>>>(n, (const double*)pc->data, (const double*)r, (double*)z);
      else
        k_diag_apply<float><<<stream_grid(n), 256, 0, s>>>(n, (const float*)pc->data, (const float*)r, (float*)z);
      break;
    case PcKind::BlockJacobi: {
      const int nb = pc->nloc;
      const long long nc = n / nb;
      const int cpb = nb >= 128 ? 1 : 128 / nb;
      const int threads = ((cpb * nb + 31) / 32) * 32;
      const size_t sm = size_t(cpb) * nb * (pc->precision == GBFEM_F64 ? 8 : 4);
      const unsigned blocks = unsigned((nc + cpb - 1) / cpb);
      if (pc->storage == GBFEM_F16) {
        const int tpc = (nb + (nb & 1)) / 2;  // threads per cell: two rows each
        const int cpbh = tpc >= 128 ? 1 : 128 / tpc;
        const int th = ((cpbh * tpc + 31) / 32) * 32;
        const unsigned bh = unsigned((nc + cpbh - 1) / cpbh);
        k_block_apply_h<<<bh, th, size_t(cpbh) * nb * 4, s>>>((const __half*)pc->data, pc->scales, (const float*)r,
                                                            (float*)z, nb, nc, cpbh);
      }
      else if (pc->precision == GBFEM_F64)
        k_block_apply<double><<<blocks, threads, sm, s>>>((const double*)pc->data, (const double*)r, (double*)z, nb,
                                                          nc, cpb);
      else
        k_block_apply<float><<<blocks, threads, sm, s>>>((const float*)pc->data, (const float*)r, (float*)z, nb,
                                                         nc, cpb);
      break;
    }
    case PcKind::External:
      return pc->ext_apply(pc->ext_ctx, r, z, s);
    case PcKind::Sor:
      return sor_apply(pc, r, z, s);
    case PcKind::ScaledBlock: {
      const int nb = pc->nloc;
      const long long nc = n / nb;
      const int cpb = nb >= 128 ? 1 : 128 / nb;
      const int threads = ((cpb * nb + 31) / 32) * 32;
      GridShape g;
      for (int d = 0; d < 3; ++d) {
        g.nc[d] = pc->sor_op->dg.grid.cells[d];
        g.per[d] = pc->sor_op->dg.grid.periodic[d];
      }
      if (pc->sb_engine == GBFEM_SB_ENGINE_TENSOR && pc->sb_tc_tiles) {
        return sb_tc_apply(pc, (const float*)pc->sor_op->dg.kappa_cell, (const float*)r, (float*)z, s);
      } else if (pc->sb_tiles) {
        // one CTA per SM over a contiguous range of quads: the inverse and
        // two residual tiles per group, 192 KB at nb = 125
        const size_t sm = size_t(nb) * (128 + 2 * kSbGroups * kSbTile) * 4;
        GBFEM_CUDA_TRY(cudaFuncSetAttribute(k_scaled_block_apply_tiled, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                            int(sm)));
        const long long nquads = pc->sb_ntiles / kSbGroups;
        const long long grid = nquads < num_sms() ? nquads : num_sms();
        k_scaled_block_apply_tiled<<<unsigned(grid), kSbGroups * kSbGroupThreads, sm, s>>>(
            (const float*)pc->data, (const float*)pc->sor_op->dg.kappa_cell, pc->sor_cells, pc->sb_tiles,
            (const float*)r, (float*)z, nb, int(nquads));
      } else {
        k_scaled_block_apply<<<unsigned((nc + cpb - 1) / cpb), threads, size_t(cpb) * nb * 4, s>>>(
            (const float*)pc->data, (const float*)pc->sor_op->dg.kappa_cell, (const float*)r, (float*)z, nb, nc, cpb,
            g);
      }
      break;
    }
  }
  GBFEM_CUDA_TRY(cudaGetLastError());
  return GBFEM_OK;
}

static int op_apply(gbfem_operator op, const void* u, void* w, Ctx& c) {
  ++c.op_applies;
  return gbfem_operator_apply(op, u, w, c.s);
}
static int pc_apply(gbfem_preconditioner pc, const void* r, void* z, Ctx& c) {
  ++c.pc_applies;
  return precond_apply(pc, r, z, c.s);
}

// ------------------------------------------------------------------- CG ----
// LinearSolver::cg (solver/linear/cg.hh:18-117), same statements in order.
static int cg(gbfem_operator op, gbfem_preconditioner pc, const gbfem_solver_params& prm, const void* b, void* x,
              Ctx& c, gbfem_solver_info* info) {
  Vecs tmp;
  GBFEM_TRY(tmp.alloc(pc ? 5 : 3, c.bytes()));
  void* h = tmp[0];
  void* r = tmp[1];
  void* p = tmp[2];
  void* s = pc ? tmp[3] : p;
  void* q = pc ? tmp[4] : p;
  GBFEM_TRY(op_apply(op, x, h, c));
  GBFEM_TRY(c.copy(h, r));
  GBFEM_TRY(c.axpby(-1.0, b, 1.0, r));   // r = h - b
  GBFEM_TRY(c.copy(b, p));
  GBFEM_TRY(c.axpby(-1.0, h, 1.0, p));   // p = b - h
  if (pc) {
    GBFEM_TRY(pc_apply(pc, p, q, c));
    GBFEM_TRY(c.copy(q, s));
  }
  double prev = 0.0, residual = 0.0;
  GBFEM_TRY(c.dot(p, q, &residual));
  double bb = 1.0;
  // GBFEM_TOL_RELATIVE_RESIDUAL (not in the reference): stop on the
  // unpreconditioned residual ||b - A x|| <= eps ||b||, with p the recursively
  // updated residual (one more dot product per iteration with a
  // preconditioner); the iterates are those of the reference's loop.
  const bool true_res = prm.error_measure == GBFEM_TOL_RELATIVE_RESIDUAL;
  if (prm.error_measure == GBFEM_TOL_RELATIVE || true_res) GBFEM_TRY(c.dot(b, b, &bb));
  const double tolerance = prm.tolerance * prm.tolerance *
                           (prm.error_measure == GBFEM_TOL_RELATIVE || true_res ? bb
                            : prm.error_measure == GBFEM_TOL_RESIDUAL_REDUCTION ? residual : 1.0);
  double rr = residual;
  if (true_res && pc) GBFEM_TRY(c.dot(p, p, &rr));
  int it = 0;
  if (!finite(residual) || !finite(tolerance)) info->status = GBFEM_ERR_NONFINITE;
  for (it = 0; info->status == GBFEM_OK && (true_res ? rr : residual) > tolerance && it < prm.max_iterations;
       ++it) {
    if (it > 0) {
      const double beta = residual / prev;
      if (pc) GBFEM_TRY(c.axpby(1.0, s, beta, q));   // q = beta q + s
      else GBFEM_TRY(c.axpby(-1.0, r, beta, p));     // p = beta p - r
    }
    GBFEM_TRY(op_apply(op, q, h, c));
    double qdoth = 0.0;
    GBFEM_TRY(c.dot(q, h, &qdoth));
    const double alpha = residual / qdoth;
    if (!finite(alpha)) { info->status = GBFEM_ERR_NONFINITE; break; }
    GBFEM_TRY(c.axpby(alpha, q, 1.0, x));
    if (pc) {
      GBFEM_TRY(c.axpby(-alpha, h, 1.0, p));
      GBFEM_TRY(pc_apply(pc, p, s, c));
      prev = residual;
      GBFEM_TRY(c.dot(p, s, &residual));
    } else {
      GBFEM_TRY(c.axpby(alpha, h, 1.0, r));
      prev = residual;
      GBFEM_TRY(c.dot(r, r, &residual));
    }
    rr = residual;
    if (true_res && pc) GBFEM_TRY(c.dot(p, p, &rr));
    if (prm.verbose) std::printf("gbfem CG it: %d : residual %.6e\n", it, std::sqrt(std::fabs(residual)));
  }
  if (!finite(residual) || !finite(rr)) info->status = GBFEM_ERR_NONFINITE;  // a NaN ends the loop as if converged
  info->residual = std::sqrt(std::fabs(true_res ? rr : residual));
  info->iterations = it < prm.max_iterations ? it : -it;
  info->converged = (it < prm.max_iterations && info->status == GBFEM_OK) ? 1 : 0;
  return GBFEM_OK;
}

// ------------------------------------------------ CG, device-resident loop ---
// The same statements as cg() above, with the Krylov scalars in device memory
// (written by single-thread kernels) and the vector updates predicated on an
// "active" flag, so chunks of `chunk` iterations can be captured once into a
// CUDA graph and relaunched; the host reads the convergence flag once per
// chunk instead of synchronising on every scalar product.  Divisions and
// updates are the host loop's, so the iterates are identical.
enum { DS_RES = 0, DS_PREV, DS_QH, DS_NEW, DS_ALPHA, DS_BETA, DS_TOL, DS_ACTIVE, DS_DIR, DS_CONV, DS_IT, DS_MAX,
       DS_STATUS, DS_N };

// begin of an iteration + direction update (q = s + beta q with a
// preconditioner, p = beta p - r without): every thread derives the flags and
// beta itself from the fields no kernel of this launch writes; thread 0
// publishes them for the later kernels.
template <typename T>
__global__ void k_cg_begin_dir(long long n, double a, const T* __restrict__ x, T* __restrict__ y, double* ds) {
  const bool conv = ds[DS_CONV] != 0.0;
  const bool dir = !conv && ds[DS_IT] > 0.0;
  const double beta = dir ? ds[DS_RES] / ds[DS_PREV] : 0.0;
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    ds[DS_ACTIVE] = conv ? 0.0 : 1.0;
    ds[DS_DIR] = dir ? 1.0 : 0.0;
    ds[DS_BETA] = beta;
  }
  if (!dir) return;
  const T b = T(beta);
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    y[i] = T(a) * x[i] + b * y[i];
}
// pass 2 of <q, h>, then alpha = rho / <q, h>
__global__ void __launch_bounds__(kRedThreads) k_cg_final_alpha(const double* __restrict__ partial, int np,
                                                                double* ds) {
  const double qh = dot_final_sum(partial, np);
  if (threadIdx.x != 0) return;
  ds[DS_QH] = qh;
  if (ds[DS_ACTIVE] == 0.0) return;
  const double alpha = ds[DS_RES] / qh;
  if (!isfinite(alpha)) {
    ds[DS_STATUS] = 1.0;
    ds[DS_CONV] = 1.0;
    ds[DS_ACTIVE] = 0.0;
    return;
  }
  ds[DS_ALPHA] = alpha;
}
// x += alpha q; v += sv alpha h (v = p, sv = -1 with the diagonal
// preconditioner; v = r, sv = +1 without), if active; then, in the partition
// of pass 1 of a dot product: PC 0 the partial of <r, r>, PC 1 s = dinv p and
// the partial of <p, s>.
template <typename T, int PC>
__global__ void __launch_bounds__(kRedThreads) k_cg_update_dot(long long n, long long chunk, const T* __restrict__ q,
                                                               const T* __restrict__ h, T* __restrict__ x,
                                                               T* __restrict__ v, double sv,
                                                               const T* __restrict__ dinv, T* __restrict__ sz,
                                                               double* __restrict__ partial, const double* ds) {
  const bool active = ds[DS_ACTIVE] != 0.0;
  const T alpha = T(ds[DS_ALPHA]);
  const T sa = T(sv * ds[DS_ALPHA]);
  const long long b0 = (long long)blockIdx.x * chunk;
  long long b1 = b0 + chunk;
  if (b1 > n) b1 = n;
  DotAcc<T> acc;  // the order and arithmetic of dot_partial_kernel
  for (long long i = b0 + threadIdx.x; i < b1; i += kRedThreads) {
    T vi = v[i];
    if (active) {
      x[i] = alpha * q[i] + T(1) * x[i];
      vi = sa * h[i] + T(1) * vi;
      v[i] = vi;
    }
    if (PC == 1) {
      const T si = vi * dinv[i];
      sz[i] = si;
      acc.add(vi, si);
    } else {
      acc.add(vi, vi);
    }
  }
  const double sum = block_sum(acc.value());
  if (threadIdx.x == 0) partial[blockIdx.x] = sum;
}
// x += alpha q; p -= alpha h, if active (a general preconditioner follows):
// grid-stride, since no dot-product partition has to be kept
template <typename T>
__global__ void k_cg_update(long long n, const T* __restrict__ q, const T* __restrict__ h, T* __restrict__ x,
                            T* __restrict__ v, double sv, const double* ds) {
  if (ds[DS_ACTIVE] == 0.0) return;
  const T alpha = T(ds[DS_ALPHA]);
  const T sa = T(sv * ds[DS_ALPHA]);
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    x[i] = alpha * q[i] + T(1) * x[i];
    v[i] = sa * h[i] + T(1) * v[i];
  }
}
// pass 2 of the new rho, then the end of the iteration
__global__ void __launch_bounds__(kRedThreads) k_cg_final_end(const double* __restrict__ partial, int np,
                                                              double* ds) {
  const double rho = dot_final_sum(partial, np);
  if (threadIdx.x != 0) return;
  ds[DS_NEW] = rho;
  if (ds[DS_ACTIVE] == 0.0) return;
  ds[DS_PREV] = ds[DS_RES];
  ds[DS_RES] = ds[DS_NEW];
  ds[DS_IT] += 1.0;
  if (!(ds[DS_RES] > ds[DS_TOL]) || ds[DS_IT] >= ds[DS_MAX]) ds[DS_CONV] = 1.0;
  if (!isfinite(ds[DS_RES])) {
    ds[DS_STATUS] = 1.0;
    ds[DS_CONV] = 1.0;
  }
}

static int cg_device(gbfem_operator op, gbfem_preconditioner pc, const gbfem_solver_params& prm, const void* b,
                     void* x, Ctx& c, gbfem_solver_info* info) {
  Vecs tmp;
  GBFEM_TRY(tmp.alloc(pc ? 5 : 3, c.bytes()));
  void* h = tmp[0];
  void* r = tmp[1];
  void* p = tmp[2];
  void* s = pc ? tmp[3] : p;
  void* q = pc ? tmp[4] : p;
  double* ds = nullptr;
  GBFEM_CUDA_TRY(cudaMalloc(&ds, sizeof(double) * DS_N));
  struct Free { double* p; ~Free() { cudaFree(p); } } free_ds{ds};
  // set-up, as cg(): h = A x, r = h - b, p = b - h, q = s = P p
  GBFEM_TRY(op_apply(op, x, h, c));
  GBFEM_TRY(c.copy(h, r));
  GBFEM_TRY(c.axpby(-1.0, b, 1.0, r));
  GBFEM_TRY(c.copy(b, p));
  GBFEM_TRY(c.axpby(-1.0, h, 1.0, p));
  if (pc) {
    GBFEM_TRY(pc_apply(pc, p, q, c));
    GBFEM_TRY(c.copy(q, s));
  }
  double residual = 0.0, bb = 1.0;
  GBFEM_TRY(c.dot(p, q, &residual));
  if (prm.error_measure == GBFEM_TOL_RELATIVE) GBFEM_TRY(c.dot(b, b, &bb));
  const double tolerance = prm.tolerance * prm.tolerance *
                           (prm.error_measure == GBFEM_TOL_RELATIVE ? bb
                            : prm.error_measure == GBFEM_TOL_RESIDUAL_REDUCTION ? residual : 1.0);
  double h0[DS_N] = {};
  h0[DS_RES] = residual;
  h0[DS_TOL] = tolerance;
  h0[DS_MAX] = double(prm.max_iterations);
  h0[DS_CONV] = (residual > tolerance && 0 < prm.max_iterations) ? 0.0 : 1.0;
  if (!finite(residual) || !finite(tolerance)) { h0[DS_CONV] = 1.0; h0[DS_STATUS] = 1.0; }
  GBFEM_CUDA_TRY(cudaMemcpyAsync(ds, h0, sizeof(h0), cudaMemcpyHostToDevice, c.s));
  // one iteration, as a function of the stream
  const long long n = c.n;
  const int g = stream_grid(n);
  const int np = dot_num_partials(n);
  const long long dchunk = (n + np - 1) / np;
  const bool diag_pc = pc && pc->kind == PcKind::Diagonal;
  // one iteration, as a function of the stream: 6 launches (plus the operator
  // and a general preconditioner with its dot product)
  auto iteration = [&](cudaStream_t st) -> int {
    if (c.prec == GBFEM_F64) {
      if (pc) k_cg_begin_dir<double><<<g, 256, 0, st>>>(n, 1.0, (const double*)s, (double*)q, ds);
      else k_cg_begin_dir<double><<<g, 256, 0, st>>>(n, -1.0, (const double*)r, (double*)p, ds);
    } else {
      if (pc) k_cg_begin_dir<float><<<g, 256, 0, st>>>(n, 1.0, (const float*)s, (float*)q, ds);
      else k_cg_begin_dir<float><<<g, 256, 0, st>>>(n, -1.0, (const float*)r, (float*)p, ds);
    }
    GBFEM_TRY(gbfem_operator_apply(op, q, h, st));
    int npp = 0;
    GBFEM_TRY(dot_partial_device(c.prec, n, q, h, c.d_partial, &npp, st));
    k_cg_final_alpha<<<1, kRedThreads, 0, st>>>(c.d_partial, np, ds);
    void* v = pc ? p : r;
    const double sv = pc ? -1.0 : 1.0;
    const int mode = !pc ? 0 : (diag_pc ? 1 : 2);
#define GBFEM_CG_UPDATE(TT, M)                                                                              \
  k_cg_update_dot<TT, M><<<np, kRedThreads, 0, st>>>(n, dchunk, (const TT*)q, (const TT*)h, (TT*)x, (TT*)v, sv, \
                                                     diag_pc ? (const TT*)pc->data : nullptr, (TT*)s, c.d_partial, ds)
    if (c.prec == GBFEM_F64) {
      if (mode == 0) GBFEM_CG_UPDATE(double, 0);
      else if (mode == 1) GBFEM_CG_UPDATE(double, 1);
      else k_cg_update<double><<<g, 256, 0, st>>>(n, (const double*)q, (const double*)h, (double*)x, (double*)v, sv, ds);
    } else {
      if (mode == 0) GBFEM_CG_UPDATE(float, 0);
      else if (mode == 1) GBFEM_CG_UPDATE(float, 1);
      else k_cg_update<float><<<g, 256, 0, st>>>(n, (const float*)q, (const float*)h, (float*)x, (float*)v, sv, ds);
    }
#undef GBFEM_CG_UPDATE
    if (mode == 2) {
      GBFEM_TRY(precond_apply(pc, p, s, st));
      GBFEM_TRY(dot_partial_device(c.prec, n, p, s, c.d_partial, &npp, st));
    }
    k_cg_final_end<<<1, kRedThreads, 0, st>>>(c.d_partial, np, ds);
    GBFEM_CUDA_TRY(cudaGetLastError());
    return GBFEM_OK;
  };
  // capture `chunk` iterations into a graph on a private stream
  const int chunk = prm.graph_chunk > 0 ? prm.graph_chunk : 16;
  cudaStream_t st = nullptr;
  GBFEM_CUDA_TRY(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
  struct FreeStream { cudaStream_t s; ~FreeStream() { cudaStreamDestroy(s); } } free_st{st};
  GBFEM_CUDA_TRY(cudaStreamSynchronize(c.s));
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  GBFEM_CUDA_TRY(cudaStreamBeginCapture(st, cudaStreamCaptureModeRelaxed));
  int rc = GBFEM_OK;
  for (int k = 0; k < chunk && rc == GBFEM_OK; ++k) rc = iteration(st);
  cudaError_t e = cudaStreamEndCapture(st, &graph);
  if (rc) { if (graph) cudaGraphDestroy(graph); return rc; }
  if (e != cudaSuccess) return set_cuda_error(e, "cg graph capture");
  e = cudaGraphInstantiate(&exec, graph, 0);
  cudaGraphDestroy(graph);
  if (e != cudaSuccess) return set_cuda_error(e, "cg graph instantiate");
  struct FreeExec { cudaGraphExec_t g; ~FreeExec() { cudaGraphExecDestroy(g); } } free_exec{exec};
  double hs[DS_N];
  int launches = 0;
  while (true) {
    GBFEM_CUDA_TRY(cudaMemcpyAsync(hs, ds, sizeof(hs), cudaMemcpyDeviceToHost, st));
    GBFEM_CUDA_TRY(cudaStreamSynchronize(st));
    if (hs[DS_CONV] != 0.0) break;
    GBFEM_CUDA_TRY(cudaGraphLaunch(exec, st));
    ++launches;
    if (prm.verbose) std::printf("gbfem CG (graph) it: %d : residual %.6e\n", int(hs[DS_IT]), std::sqrt(hs[DS_RES]));
  }
  const int it = int(hs[DS_IT]);
  if (hs[DS_STATUS] != 0.0) info->status = GBFEM_ERR_NONFINITE;
  info->residual = std::sqrt(std::fabs(hs[DS_RES]));
  info->iterations = it < prm.max_iterations ? it : -it;
  info->converged = (it < prm.max_iterations && info->status == GBFEM_OK) ? 1 : 0;
  // applies launched: the set-up's plus every captured iteration (the ones
  // after convergence recompute unchanged vectors and are not counted in `it`)
  c.op_applies += chunk * launches + 1;
  c.pc_applies += pc ? chunk * launches + 1 : 0;
  return GBFEM_OK;
}

// ----------------------------------------------------------------- GMRES ---
static void rotate(double* x, double* y, double cc, double ss) {
  const double a = *x, b = *y;
  *x = cc * a + ss * b;
  *y = cc * b - ss * a;
}

// LinearSolver::gmres (solver/linear/gmres.hh:116-299), right-preconditioned
// restarted GMRES(m) with Givens rotations.  flexible = true keeps every
// preconditioned direction z_j = M_j^{-1} v_j and updates u += Z y (FGMRES,
// Saad 1993), so the preconditioner may change between iterations.
static int gmres(gbfem_operator op, gbfem_preconditioner pc, const gbfem_solver_params& prm, const void* b,
                 void* u, Ctx& c, gbfem_solver_info* info, bool flexible) {
  const int m = prm.restart > 0 ? prm.restart : 20;
  Vecs v, zf;
  GBFEM_TRY(v.alloc(m + 2, c.bytes()));
  if (flexible && pc) GBFEM_TRY(zf.alloc(m, c.bytes()));
  std::vector<double> H((m + 1) * m, 0.0), g(m + 1, 0.0), sn(m, 0.0), cs(m, 0.0), y(m, 0.0), gd(m + 1, 0.0);
  auto Hm = [&](int i, int j) -> double& { return H[i * m + j]; };
  double tol = prm.tolerance;
  if (prm.error_measure == GBFEM_TOL_RELATIVE) {
    double bb;
    GBFEM_TRY(c.dot(b, b, &bb));
    tol *= std::sqrt(bb);
  }
  int iterations = 0;
  double res = 0.0;
  while (true) {
    GBFEM_TRY(op_apply(op, u, v[0], c));
    GBFEM_TRY(c.axpby(-1.0, b, 1.0, v[0]));  // v0 = A u - b
    double d0;
    GBFEM_TRY(c.dot(v[0], v[0], &d0));
    res = std::sqrt(d0);
    if (prm.error_measure == GBFEM_TOL_RESIDUAL_REDUCTION && iterations == 0) tol *= res;
    if (!finite(res)) { info->status = GBFEM_ERR_NONFINITE; break; }
    if (prm.verbose) std::printf("gbfem GMRES outer iteration : %.6e\n", res);
    if (res <= tol * (1 + 1e-15)) break;
    g[0] = -res;
    for (int i = 1; i <= m; ++i) g[i] = 0.0;
    GBFEM_TRY(c.scal(1.0 / res, v[0]));
    int jlast = 0;
    for (int j = 0; j < m; ++j) {
      void* vj = v[j];
      void* vjp = v[j + 1];
      if (pc) {
        void* z = flexible ? zf[j] : v[m + 1];
        GBFEM_TRY(pc_apply(pc, vj, z, c));
        GBFEM_TRY(op_apply(op, z, vjp, c));
      } else {
        GBFEM_TRY(op_apply(op, vj, vjp, c));
      }
      // classical Gram-Schmidt: the j+1 products with the same vector in one
      // pass and one host read (the reference sums them in one comm.sum,
      // gmres.hh:91), then one fused update
      std::vector<const void*> xs(j + 1, vjp), vs(j + 1);
      for (int l = 0; l <= j; ++l) vs[l] = v[l];
      GBFEM_TRY(c.multi_dot(j + 1, xs.data(), vs.data(), gd.data()));
      for (int i = 0; i <= j; ++i) Hm(i, j) = gd[i];
      std::vector<double> neg(j + 1);
      for (int l = 0; l <= j; ++l) neg[l] = -gd[l];
      GBFEM_TRY(c.multi_axpy(j + 1, neg.data(), vs.data(), vjp));
      double nn;
      GBFEM_TRY(c.dot(vjp, vjp, &nn));
      Hm(j + 1, j) = std::sqrt(nn);
      GBFEM_TRY(c.scal(1.0 / Hm(j + 1, j), vjp));
      for (int i = 0; i < j; ++i) rotate(&Hm(i + 1, j), &Hm(i, j), cs[i], sn[i]);
      const double hjj = Hm(j, j), hjpj = Hm(j + 1, j);
      const double nrm = std::sqrt(hjj * hjj + hjpj * hjpj);
      cs[j] = hjj / nrm;
      sn[j] = -hjpj / nrm;
      rotate(&Hm(j + 1, j), &Hm(j, j), cs[j], sn[j]);
      rotate(&g[j + 1], &g[j], cs[j], sn[j]);
      ++iterations;
      jlast = j;
      if (prm.verbose) std::printf("gbfem GMRES it: %d : %.6e\n", iterations, std::fabs(g[j + 1]));
      if (!finite(g[j + 1])) { info->status = GBFEM_ERR_NONFINITE; break; }
      if (std::fabs(g[j + 1]) < tol || iterations >= prm.max_iterations) break;
    }
    if (info->status != GBFEM_OK) break;
    int last = iterations % m;
    if (last == 0) last = m;
    if (flexible) last = jlast + 1;
    for (int i = last - 1; i >= 0; --i) {
      double dt = 0.0;
      for (int k = 0; k < last - (i + 1); ++k) dt += Hm(i, i + 1 + k) * y[i + 1 + k];
      y[i] = (g[i] - dt) / Hm(i, i);
    }
    if (pc && !flexible) {
      void* ut = v[m];
      void* z = v[m + 1];
      GBFEM_TRY(c.clear(ut));
      for (int i = 0; i < last; ++i) GBFEM_TRY(c.axpby(y[i], v[i], 1.0, ut));
      GBFEM_TRY(pc_apply(pc, ut, z, c));
      GBFEM_TRY(c.axpby(1.0, z, 1.0, u));
    } else if (pc && flexible) {
      for (int i = 0; i < last; ++i) GBFEM_TRY(c.axpby(y[i], zf[i], 1.0, u));
    } else {
      for (int i = 0; i < last; ++i) GBFEM_TRY(c.axpby(y[i], v[i], 1.0, u));
    }
    res = std::fabs(g[last]);
    if (std::fabs(g[last]) < tol) break;
    // The reference loops on here even past maxIterations (gmres.hh:150-286);
    // stop instead.
    if (iterations >= prm.max_iterations) break;
  }
  info->residual = res;
  info->iterations = iterations < prm.max_iterations ? iterations : -iterations;
  info->converged = (iterations < prm.max_iterations && info->status == GBFEM_OK) ? 1 : 0;
  return GBFEM_OK;
}

// -------------------------------------------------------------- BiCGstab ---
// LinearSolver::bicgstab (solver/linear/bicgstab.hh:63-222), right
// preconditioning with x the preconditioned variable, as the reference.
static int bicgstab(gbfem_operator op, gbfem_preconditioner pc, const gbfem_solver_params& prm, const void* b,
                    void* x, Ctx& c, gbfem_solver_info* info) {
  Vecs t;
  GBFEM_TRY(t.alloc(pc ? 6 : 5, c.bytes()));
  void *r = t[0], *rs = t[1], *p = t[2], *s = t[3], *tmp = t[4];
  void* z = pc ? t[5] : r;
  double tol = prm.tolerance, gdot[5];
  if (prm.error_measure == GBFEM_TOL_RELATIVE) {
    GBFEM_TRY(c.dot(b, b, &gdot[0]));
    tol *= std::sqrt(gdot[0]);
  }
  if (pc) {
    GBFEM_TRY(pc_apply(pc, x, z, c));
    GBFEM_TRY(op_apply(op, z, r, c));
  } else {
    GBFEM_TRY(op_apply(op, x, r, c));
  }
  GBFEM_TRY(c.axpby(1.0, b, -1.0, r));  // r = b - r
  GBFEM_TRY(c.copy(r, p));
  GBFEM_TRY(c.copy(r, rs));
  GBFEM_TRY(c.dot(r, rs, &gdot[0]));
  double nu = gdot[0];
  if (prm.error_measure == GBFEM_TOL_RESIDUAL_REDUCTION) tol *= std::sqrt(nu);
  int iterations = 0;
  double res = 0.0;
  while (true) {
    if (pc) {
      GBFEM_TRY(pc_apply(pc, p, z, c));
      GBFEM_TRY(op_apply(op, z, tmp, c));
    } else {
      GBFEM_TRY(op_apply(op, p, tmp, c));
    }
    GBFEM_TRY(c.dot(tmp, rs, &gdot[0]));
    const double alpha = nu / gdot[0];
    GBFEM_TRY(c.copy(r, s));
    GBFEM_TRY(c.axpby(-alpha, tmp, 1.0, s));
    if (pc) {
      GBFEM_TRY(pc_apply(pc, s, z, c));
      GBFEM_TRY(op_apply(op, z, r, c));
    } else {
      GBFEM_TRY(op_apply(op, s, r, c));
    }
    {
      // the five products of this step in one pass and one host read
      const void* xs[5] = {r, r, s, s, r};
      const void* ys[5] = {s, r, s, rs, rs};
      GBFEM_TRY(c.multi_dot(5, xs, ys, gdot));
    }
    const double omega = gdot[0] / gdot[1];
    res = std::sqrt(gdot[2] - omega * (2.0 * gdot[0] - omega * gdot[1]));
    const double beta = (gdot[3] - omega * gdot[4]) * alpha / (omega * nu);
    nu = gdot[3] - omega * gdot[4];
    GBFEM_TRY(c.axpbypcz(alpha, p, omega, s, 1.0, x));
    ++iterations;
    if (!finite(res) || !finite(beta)) { info->status = GBFEM_ERR_NONFINITE; break; }
    if (res < tol || iterations >= prm.max_iterations) break;
    GBFEM_TRY(c.axpby(1.0, s, -omega, r));                       // r = s - omega r
    GBFEM_TRY(c.axpbypcz(1.0, r, -omega * beta, tmp, beta, p));  // p = r + beta (p - omega tmp)
    if (prm.verbose) std::printf("gbfem BiCGstab it: %d : %.6e\n", iterations, res);
  }
  if (pc) {
    GBFEM_TRY(pc_apply(pc, x, z, c));
    GBFEM_TRY(c.copy(z, x));
  }
  info->residual = res;
  info->iterations = iterations >= prm.max_iterations ? -iterations : iterations;
  info->converged = (iterations < prm.max_iterations && info->status == GBFEM_OK) ? 1 : 0;
  return GBFEM_OK;
}

// ------------------------------------------------------------------- FCG ---
// Flexible CG with truncated A-orthogonalisation against the last mmax
// directions (Notay, SIAM J. Sci. Comput. 22(4), 2000):
//   z_k = M_k^{-1} r_k,  d_k = z_k - sum_i (z_k . w_i)/(d_i . w_i) d_i,  w_i = A d_i,
//   alpha = (d_k . r_k)/(d_k . w_k),  x += alpha d_k,  r -= alpha w_k.
// Residual r = b - A x; stopping as in cg.hh (||r||^2 against eps^2 ||b||^2).
// Fallback: when the preconditioner has one (the learned preconditioner's
// block Jacobi) and the residual norm has not dropped by 10 % within
// kStagnation iterations, or the step is not finite, the iteration switches
// to the fallback and restarts its direction history.  The FP64 residual
// decides convergence either way.
static int fcg(gbfem_operator op, gbfem_preconditioner pc, const gbfem_solver_params& prm, const void* b, void* x,
               Ctx& c, gbfem_solver_info* info) {
  const int mmax = prm.restart > 0 ? prm.restart : 1;
  // residual norms of CG-type methods plateau for tens of iterations on
  // these problems while the A-norm error keeps falling, so the window is long
  constexpr int kStagnation = 200;
  Vecs t, dirs, ws;
  GBFEM_TRY(t.alloc(2, c.bytes()));
  GBFEM_TRY(dirs.alloc(mmax + 1, c.bytes()));
  GBFEM_TRY(ws.alloc(mmax + 1, c.bytes()));
  void *r = t[0], *z = t[1];
  std::vector<double> dw(mmax + 1, 1.0);
  GBFEM_TRY(op_apply(op, x, r, c));
  GBFEM_TRY(c.axpby(1.0, b, -1.0, r));  // r = b - A x
  double rr, bb = 1.0;
  GBFEM_TRY(c.dot(r, r, &rr));
  if (prm.error_measure == GBFEM_TOL_RELATIVE) GBFEM_TRY(c.dot(b, b, &bb));
  const double tolerance = prm.tolerance * prm.tolerance *
                           (prm.error_measure == GBFEM_TOL_RELATIVE ? bb
                            : prm.error_measure == GBFEM_TOL_RESIDUAL_REDUCTION ? rr : 1.0);
  gbfem_preconditioner cur = pc;
  int it = 0, hist = 0, mark_it = 0;
  double mark_rr = rr;
  if (!finite(rr) || !finite(tolerance)) info->status = GBFEM_ERR_NONFINITE;
  for (it = 0; info->status == GBFEM_OK && rr > tolerance && it < prm.max_iterations; ++it) {
    const int slot = hist % (mmax + 1);
    void* d = dirs[slot];
    void* w = ws[slot];
    if (cur) GBFEM_TRY(pc_apply(cur, r, z, c));
    else GBFEM_TRY(c.copy(r, z));
    GBFEM_TRY(c.copy(z, d));
    const int kept = hist < mmax ? hist : mmax;
    for (int k = 1; k <= kept; ++k) {
      const int sl = (hist - k) % (mmax + 1);
      double zw;
      GBFEM_TRY(c.dot(z, ws[sl], &zw));
      GBFEM_TRY(c.axpby(-zw / dw[sl], dirs[sl], 1.0, d));
    }
    GBFEM_TRY(op_apply(op, d, w, c));
    double dwk, dr;
    GBFEM_TRY(c.dot(d, w, &dwk));
    GBFEM_TRY(c.dot(d, r, &dr));
    const double alpha = dr / dwk;
    if (!finite(alpha) || !(dwk > 0.0)) {
      if (cur && cur->fallback && cur != cur->fallback) {  // a bad direction from the variable preconditioner
        cur = cur->fallback;
        ++info->fallbacks;
        hist = 0;
        mark_it = it;
        mark_rr = rr;
        continue;
      }
      info->status = GBFEM_ERR_NONFINITE;
      break;
    }
    dw[slot] = dwk;
    ++hist;
    GBFEM_TRY(c.axpby(alpha, d, 1.0, x));
    GBFEM_TRY(c.axpby(-alpha, w, 1.0, r));
    GBFEM_TRY(c.dot(r, r, &rr));
    if (rr < 0.81 * mark_rr) {
      mark_rr = rr;
      mark_it = it;
    } else if (it - mark_it >= kStagnation && cur && cur->fallback && cur != cur->fallback) {
      cur = cur->fallback;
      ++info->fallbacks;
      hist = 0;
      mark_it = it;
      mark_rr = rr;
    }
    if (prm.verbose) std::printf("gbfem FCG it: %d : residual %.6e\n", it, std::sqrt(rr));
  }
  info->residual = std::sqrt(rr);
  info->iterations = it < prm.max_iterations ? it : -it;
  info->converged = (it < prm.max_iterations && info->status == GBFEM_OK) ? 1 : 0;
  return GBFEM_OK;
}

int solve_impl(gbfem_operator op, gbfem_preconditioner pc, const gbfem_solver_params& prm, const void* f, void* u,
               gbfem_solver_info* info, cudaStream_t s) {
  Ctx c;
  GBFEM_TRY(c.setup(op->precision, op->ndofs, s));
  *info = gbfem_solver_info{};
  const auto t0 = std::chrono::steady_clock::now();
  int rc;
  if (prm.error_measure < GBFEM_TOL_ABSOLUTE || prm.error_measure > GBFEM_TOL_RELATIVE_RESIDUAL)
    return set_error(GBFEM_ERR_INVALID, "gbfem_solve: unknown error measure");
  // the other methods already stop on the unpreconditioned residual
  gbfem_solver_params pr = prm;
  if (prm.method != GBFEM_SOLVER_CG && pr.error_measure == GBFEM_TOL_RELATIVE_RESIDUAL)
    pr.error_measure = GBFEM_TOL_RELATIVE;
  switch (prm.method) {
    case GBFEM_SOLVER_CG:
      // device-resident loop unless the preconditioner is external (its apply
      // may synchronise the host, which a graph capture cannot hold) or the
      // stop is on the unpreconditioned residual (host loop)
      rc = (pr.graph_chunk > 0 && !(pc && pc->kind == PcKind::External) &&
            pr.error_measure != GBFEM_TOL_RELATIVE_RESIDUAL)
               ? cg_device(op, pc, pr, f, u, c, info)
               : cg(op, pc, pr, f, u, c, info);
      break;
    case GBFEM_SOLVER_GMRES: rc = gmres(op, pc, pr, f, u, c, info, false); break;
    case GBFEM_SOLVER_FGMRES: rc = gmres(op, pc, pr, f, u, c, info, true); break;
    case GBFEM_SOLVER_BICGSTAB: rc = bicgstab(op, pc, pr, f, u, c, info); break;
    case GBFEM_SOLVER_FCG: rc = fcg(op, pc, pr, f, u, c, info); break;
    default: return set_error(GBFEM_ERR_INVALID, "gbfem_solve: unknown method " + std::to_string(prm.method));
  }
  GBFEM_CUDA_TRY(cudaStreamSynchronize(s));
  info->time_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
  info->operator_applies = c.op_applies;
  info->preconditioner_applies = c.pc_applies;
  return rc;
}

}  // namespace gbfem

using namespace gbfem;

extern "C" {

int gbfem_solver_params_default(gbfem_solver_params* prm) {
  if (!prm) return set_error(GBFEM_ERR_INVALID, "null params");
  prm->method = GBFEM_SOLVER_CG;
  prm->tolerance = 1e-8;
  prm->error_measure = GBFEM_TOL_ABSOLUTE;
  prm->max_iterations = INT_MAX;
  prm->restart = 20;
  prm->verbose = 0;
  prm->graph_chunk = 0;
  return GBFEM_OK;
}

int gbfem_preconditioner_diagonal_create(gbfem_operator op, gbfem_preconditioner* out) {
  if (!op || !out) return set_error(GBFEM_ERR_INVALID, "gbfem_preconditioner_diagonal_create: null argument");
  *out = nullptr;
  auto* pc = new (std::nothrow) gbfem_preconditioner_s();
  if (!pc) return set_error(GBFEM_ERR_INVALID, "out of host memory");
  pc->kind = PcKind::Diagonal;
  pc->precision = op->precision;
  pc->n = op->ndofs;
  pc->nloc = 1;
  const size_t bytes = size_t(pc->n) * (pc->precision == GBFEM_F64 ? 8 : 4);
  cudaError_t e = cudaMalloc(&pc->data, bytes);
  if (e != cudaSuccess) { delete pc; return set_cuda_error(e, "diagonal preconditioner"); }
  int rc = gbfem_operator_diagonal(op, pc->data, nullptr);
  if (rc) { gbfem_preconditioner_destroy(pc); return rc; }
  if (pc->precision == GBFEM_F64) k_diag_invert<double><<<stream_grid(pc->n), 256>>>(pc->n, (double*)pc->data);
  else k_diag_invert<float><<<stream_grid(pc->n), 256>>>(pc->n, (float*)pc->data);
  e = cudaDeviceSynchronize();
  if (e != cudaSuccess) { gbfem_preconditioner_destroy(pc); return set_cuda_error(e, "diagonal invert"); }
  *out = pc;
  return GBFEM_OK;
}

int gbfem_preconditioner_block_jacobi_create(gbfem_operator op, int precision, gbfem_preconditioner* out) {
  if (!op || !out) return set_error(GBFEM_ERR_INVALID, "gbfem_preconditioner_block_jacobi_create: null argument");
  *out = nullptr;
  if (op->kind != OpKind::DG && op->kind != OpKind::BSR)
    return set_error(GBFEM_ERR_NOT_IMPLEMENTED, "block Jacobi needs a DG operator");
  if (precision != GBFEM_F64 && precision != GBFEM_F32 && precision != GBFEM_F16)
    return set_error(GBFEM_ERR_INVALID, "bad precision");
  auto* pc = new (std::nothrow) gbfem_preconditioner_s();
  if (!pc) return set_error(GBFEM_ERR_INVALID, "out of host memory");
  pc->kind = PcKind::BlockJacobi;
  pc->storage = precision;
  pc->precision = precision == GBFEM_F16 ? GBFEM_F32 : precision;  // vectors
  pc->n = op->ndofs;
  pc->nloc = op->nloc;
  const int nb = op->nloc;
  const size_t isz = precision == GBFEM_F64 ? 8 : (precision == GBFEM_F32 ? 4 : 2);
  const size_t osz = op->precision == GBFEM_F64 ? 8 : 4;
  const int ldh = nb + (nb & 1);  // FP16: rows padded to an even length
  const size_t block_elems = precision == GBFEM_F16 ? size_t(nb) * ldh : size_t(nb) * nb;
  cudaError_t e = cudaMalloc(&pc->data, size_t(op->ncells) * block_elems * isz);
  if (e == cudaSuccess && precision == GBFEM_F16) e = cudaMalloc(&pc->scales, size_t(op->ncells) * sizeof(float));
  if (e != cudaSuccess) { gbfem_preconditioner_destroy(pc); return set_cuda_error(e, "block Jacobi storage"); }
  // blocks in batches of cells (bounded temporary: <= ~1 GB)
  long long batch = (1LL << 30) / ((long long)nb * nb * (long long)osz);
  if (batch < 1) batch = 1;
  if (batch > op->ncells) batch = op->ncells;
  void* tmp = nullptr;
  int* d_sing = nullptr;
  e = cudaMalloc(&tmp, size_t(batch) * nb * nb * osz);
  if (e == cudaSuccess) e = cudaMalloc(&d_sing, sizeof(int));
  if (e == cudaSuccess) e = cudaMemset(d_sing, 0, sizeof(int));
  if (e != cudaSuccess) {
    if (tmp) cudaFree(tmp);
    gbfem_preconditioner_destroy(pc);
    return set_cuda_error(e, "block Jacobi temporary");
  }
  int rc = GBFEM_OK;
  const size_t sm = size_t(nb) * nb * 8 + size_t(nb) * 4;
  for (long long c0 = 0; c0 < op->ncells && rc == GBFEM_OK; c0 += batch) {
    const long long cnt = (c0 + batch <= op->ncells) ? batch : op->ncells - c0;
    if (op->kind == OpKind::BSR) {
      const size_t bsz = size_t(nb) * nb * osz;
      e = cudaMemcpy2D(tmp, bsz, static_cast<char*>(op->bsr_blocks) + size_t(c0) * 7 * bsz, 7 * bsz, bsz,
                       size_t(cnt), cudaMemcpyDeviceToDevice);
      if (e != cudaSuccess) { rc = set_cuda_error(e, "block Jacobi from assembled operator"); break; }
    } else {
      rc = dg_apply(op, nullptr, nullptr, nullptr, 1, tmp, c0, cnt);
    }
    if (rc) break;
    float* sc = pc->scales ? pc->scales + c0 : nullptr;
    if (precision == GBFEM_F16 && op->precision == GBFEM_F64) {
      cudaFuncSetAttribute(k_block_invert<double, __half>, cudaFuncAttributeMaxDynamicSharedMemorySize, int(sm));
      k_block_invert<double, __half><<<unsigned(cnt), 256, sm>>>((const double*)tmp,
                                                                ((__half*)pc->data) + c0 * (long long)block_elems, nb,
                                                                cnt, d_sing, sc);
    } else if (precision == GBFEM_F16) {
      cudaFuncSetAttribute(k_block_invert<float, __half>, cudaFuncAttributeMaxDynamicSharedMemorySize, int(sm));
      k_block_invert<float, __half><<<unsigned(cnt), 256, sm>>>((const float*)tmp,
                                                               ((__half*)pc->data) + c0 * (long long)block_elems, nb,
                                                               cnt, d_sing, sc);
    } else if (op->precision == GBFEM_F64 && precision == GBFEM_F64) {
      cudaFuncSetAttribute(k_block_invert<double, double>, cudaFuncAttributeMaxDynamicSharedMemorySize, int(sm));
      k_block_invert<double, double><<<unsigned(cnt), 256, sm>>>((const double*)tmp,
                                                                ((double*)pc->data) + c0 * nb * nb, nb, cnt, d_sing, sc);
    } else if (op->precision == GBFEM_F64) {
      cudaFuncSetAttribute(k_block_invert<double, float>, cudaFuncAttributeMaxDynamicSharedMemorySize, int(sm));
      k_block_invert<double, float><<<unsigned(cnt), 256, sm>>>((const double*)tmp,
                                                               ((float*)pc->data) + c0 * nb * nb, nb, cnt, d_sing, sc);
    } else if (precision == GBFEM_F64) {
      cudaFuncSetAttribute(k_block_invert<float, double>, cudaFuncAttributeMaxDynamicSharedMemorySize, int(sm));
      k_block_invert<float, double><<<unsigned(cnt), 256, sm>>>((const float*)tmp,
                                                               ((double*)pc->data) + c0 * nb * nb, nb, cnt, d_sing, sc);
    } else {
      cudaFuncSetAttribute(k_block_invert<float, float>, cudaFuncAttributeMaxDynamicSharedMemorySize, int(sm));
      k_block_invert<float, float><<<unsigned(cnt), 256, sm>>>((const float*)tmp,
                                                              ((float*)pc->data) + c0 * nb * nb, nb, cnt, d_sing, sc);
    }
    e = cudaGetLastError();
    if (e != cudaSuccess) rc = set_cuda_error(e, "block invert launch");
  }
  int sing = 0;
  if (rc == GBFEM_OK) {
    e = cudaMemcpy(&sing, d_sing, sizeof(int), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) rc = set_cuda_error(e, "block invert");
  }
  cudaFree(tmp);
  cudaFree(d_sing);
  if (rc == GBFEM_OK && sing) rc = set_error(GBFEM_ERR_INVALID, "block Jacobi: a diagonal block is singular");
  if (rc) { gbfem_preconditioner_destroy(pc); return rc; }
  *out = pc;
  return GBFEM_OK;
}

int gbfem_preconditioner_scaled_block_jacobi_create(gbfem_operator op, gbfem_preconditioner* out) {
  return gbfem_preconditioner_scaled_block_jacobi_create_engine(op, GBFEM_SB_ENGINE_TENSOR, out);
}

int gbfem_preconditioner_status(gbfem_preconditioner pc, int* status) {
  if (!pc || !status) return set_error(GBFEM_ERR_INVALID, "gbfem_preconditioner_status: null argument");
  *status = 0;
  if (pc->sb_tc_status) {
    GBFEM_CUDA_TRY(cudaDeviceSynchronize());
    GBFEM_CUDA_TRY(cudaMemcpy(status, pc->sb_tc_status, sizeof(int), cudaMemcpyDeviceToHost));
  }
  return GBFEM_OK;
}

int gbfem_preconditioner_scaled_block_jacobi_create_engine(gbfem_operator op, int engine, gbfem_preconditioner* out) {
  if (!op || !out) return set_error(GBFEM_ERR_INVALID, "gbfem_preconditioner_scaled_block_jacobi_create: null argument");
  *out = nullptr;
  if (engine != GBFEM_SB_ENGINE_TENSOR && engine != GBFEM_SB_ENGINE_FMA)
    return set_error(GBFEM_ERR_INVALID, "scaled block Jacobi: unknown engine");
  const gbfem_dg_desc& d = op->dg;
  if (op->kind != OpKind::DG || !d.kappa_cell || op->precision != GBFEM_F32 || d.mass != 0.0 || op->nonlinear)
    return set_error(GBFEM_ERR_INVALID,
                     "scaled block Jacobi: needs an FP32 DG operator with kappa_cell, no mass, not nonlinear");
  // the kappa = 1 operator on a grid with one cell per boundary type, same cell size
  gbfem_dg_desc t = d;
  t.kappa = nullptr;
  t.kappa_cell = nullptr;
  t.precision = GBFEM_F64;
  t.algorithm = GBFEM_ALGO_QUADRATURE;
  for (int k = 0; k < 3; ++k) {
    const double h = (d.grid.upper[k] - d.grid.lower[k]) / d.grid.cells[k];
    const int m = d.grid.periodic[k] ? 2 : (d.grid.cells[k] <= 2 ? d.grid.cells[k] : 3);
    t.grid.cells[k] = m;
    t.grid.lower[k] = 0.0;
    t.grid.upper[k] = m * h;
  }
  gbfem_operator top = nullptr;
  GBFEM_TRY(gbfem_dg_operator_create(&t, &top));
  struct OpFree { gbfem_operator o; ~OpFree() { gbfem_operator_destroy(o); } } top_free{top};
  gbfem_preconditioner tbj = nullptr;
  GBFEM_TRY(gbfem_preconditioner_block_jacobi_create(top, GBFEM_F32, &tbj));  // inverted, transposed, FP32
  auto* pc = new (std::nothrow) gbfem_preconditioner_s();
  if (!pc) {
    gbfem_preconditioner_destroy(tbj);
    return set_error(GBFEM_ERR_INVALID, "out of host memory");
  }
  pc->kind = PcKind::ScaledBlock;
  pc->sb_engine = engine;
  pc->precision = GBFEM_F32;
  pc->n = op->ndofs;
  pc->nloc = op->nloc;
  pc->sor_op = op;
  pc->data = tbj->data;  // take over the inverted type blocks
  tbj->data = nullptr;
  gbfem_preconditioner_destroy(tbj);
  if (op->nloc > 32 && op->nloc <= 128) {
    // cells sorted by boundary type (stable: interior runs stay consecutive), tiles of <= 32
    const int* nc = d.grid.cells;
    std::vector<std::vector<int>> by_type(27);
    for (long long c = 0; c < op->ncells; ++c) {
      const long long nxy = (long long)nc[0] * nc[1];
      const long long zz = c / nxy, rem = c - zz * nxy, yy = rem / nc[0], xx = rem - yy * nc[0];
      const long long xyz[3] = {xx, yy, zz};
      int t = 0, mul = 1;
      for (int k = 0; k < 3; ++k) {
        int td, md;
        if (d.grid.periodic[k]) { td = 0; md = 2; }
        else if (nc[k] <= 2) { td = int(xyz[k]); md = nc[k]; }
        else { td = xyz[k] == 0 ? 0 : (xyz[k] == nc[k] - 1 ? 2 : 1); md = 3; }
        t += td * mul;
        mul *= md;
      }
      by_type[t].push_back(int(c));
    }
    std::vector<int> list, tiles;
    list.reserve(size_t(op->ncells));
    for (int t = 0; t < 27; ++t) {
      int ntype = 0;
      for (size_t k = 0; k < by_type[t].size(); k += kSbTile, ++ntype) {
        const int cnt = int(std::min<size_t>(kSbTile, by_type[t].size() - k));
        tiles.push_back(t);
        tiles.push_back(int(list.size()));
        tiles.push_back(cnt);
        list.insert(list.end(), by_type[t].begin() + k, by_type[t].begin() + k + cnt);
      }
      // empty tiles up to a whole quad of this type
      for (; ntype % kSbGroups != 0; ++ntype) {
        tiles.push_back(t);
        tiles.push_back(0);
        tiles.push_back(0);
      }
    }
    cudaError_t e = cudaMalloc(&pc->sor_cells, list.size() * sizeof(int));
    if (e == cudaSuccess) e = cudaMalloc(&pc->sb_tiles, tiles.size() * sizeof(int));
    if (e == cudaSuccess) e = cudaMemcpy(pc->sor_cells, list.data(), list.size() * sizeof(int), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(pc->sb_tiles, tiles.data(), tiles.size() * sizeof(int), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
      gbfem_preconditioner_destroy(pc);
      return set_cuda_error(e, "scaled block Jacobi: tiles");
    }
    pc->sb_ntiles = (long long)(tiles.size() / 3);
    if (engine == GBFEM_SB_ENGINE_TENSOR) {
      const int rc = sb_tc_setup(pc, tiles, op->nloc, 0);
      if (rc) {
        gbfem_preconditioner_destroy(pc);
        return rc;
      }
    }
  }
  *out = pc;
  return GBFEM_OK;
}

int gbfem_preconditioner_apply(gbfem_preconditioner pc, const void* r, void* z, void* stream) {
  if (!pc || !r || !z) return set_error(GBFEM_ERR_INVALID, "gbfem_preconditioner_apply: null argument");
  return precond_apply(pc, r, z, static_cast<cudaStream_t>(stream));
}

int gbfem_preconditioner_precision(gbfem_preconditioner pc, int* precision) {
  if (!pc || !precision) return set_error(GBFEM_ERR_INVALID, "null argument");
  *precision = pc->precision;
  return GBFEM_OK;
}

int gbfem_preconditioner_destroy(gbfem_preconditioner pc) {
  if (!pc) return GBFEM_OK;
  if (pc->data && pc->owns_data) cudaFree(pc->data);
  if (pc->scales) cudaFree(pc->scales);
  if (pc->sor_cells) cudaFree(pc->sor_cells);
  if (pc->sb_tiles) cudaFree(pc->sb_tiles);
  if (pc->sb_tc_tiles) cudaFree(pc->sb_tc_tiles);
  if (pc->sb_tc_img) cudaFree(pc->sb_tc_img);
  if (pc->sb_tc_status) cudaFree(pc->sb_tc_status);
  if (pc->sor_tmp) cudaFree(pc->sor_tmp);
  if (pc->ext_destroy) pc->ext_destroy(pc->ext_ctx);
  delete pc;
  return GBFEM_OK;
}

int gbfem_solve(gbfem_operator op, gbfem_preconditioner pc, const gbfem_solver_params* prm, const void* f, void* u,
                gbfem_solver_info* info) {
  if (!op || !prm || !f || !u || !info) return set_error(GBFEM_ERR_INVALID, "gbfem_solve: null argument");
  if (pc && pc->precision != op->precision)
    return set_error(GBFEM_ERR_INVALID, "gbfem_solve: preconditioner and operator precisions differ");
  if (pc && pc->n != op->ndofs) return set_error(GBFEM_ERR_INVALID, "gbfem_solve: preconditioner size mismatch");
  return solve_impl(op, pc, *prm, f, u, info, nullptr);
}

}  // extern "C"

namespace gbfem {

// The FP32 inner solve as an FP64 preconditioner: z = ||r|| A32^{-1}(r / ||r||),
// A32^{-1} the inner Krylov solve to its relative tolerance.  It is a
// nonlinear (inexact) preconditioner, so the outer method must be flexible.
struct InnerSolvePc {
  gbfem_operator op32;
  gbfem_preconditioner pc32;
  gbfem_solver_params ip;
  long long n;
  void* r32;
  void* d32;
  long long inner_total = 0;
  int op_applies = 0, pc_applies = 0;
};

static int inner_solve_apply(void* ctx, const void* r, void* z, cudaStream_t s) {
  auto* x = static_cast<InnerSolvePc*>(ctx);
  double rr = 0.0;
  GBFEM_TRY(gbfem_dot(GBFEM_F64, x->n, r, r, &rr, s));
  const double rn = std::sqrt(rr);
  if (!(rn > 0.0) || !std::isfinite(rn)) {
    GBFEM_CUDA_TRY(cudaMemsetAsync(z, 0, size_t(x->n) * 8, s));
    return rn == 0.0 ? GBFEM_OK : set_error(GBFEM_ERR_NONFINITE, "mixed: non-finite residual");
  }
  GBFEM_TRY(gbfem_convert(x->n, GBFEM_F64, r, GBFEM_F32, x->r32, s));
  GBFEM_TRY(gbfem_scal(GBFEM_F32, x->n, 1.0 / rn, x->r32, s));
  GBFEM_CUDA_TRY(cudaMemsetAsync(x->d32, 0, size_t(x->n) * 4, s));
  gbfem_solver_info ii{};
  GBFEM_TRY(solve_impl(x->op32, x->pc32, x->ip, x->r32, x->d32, &ii, s));
  x->inner_total += ii.iterations >= 0 ? ii.iterations : -ii.iterations;
  x->op_applies += ii.operator_applies;
  x->pc_applies += ii.preconditioner_applies;
  GBFEM_TRY(gbfem_convert(x->n, GBFEM_F32, x->d32, GBFEM_F64, z, s));
  GBFEM_TRY(gbfem_scal(GBFEM_F64, x->n, rn, z, s));
  return GBFEM_OK;
}

}  // namespace gbfem

extern "C" {

// FP64 outer iteration around an FP32 inner solve.
//   refinement: r = f - A64 u;  while ||r|| > tol ||f||:  solve A32 d = r/||r|| (FP32),  u += ||r|| d
//   flexible:   FGMRES / FCG on A64 u = f with the inner solve as the preconditioner
int gbfem_solve_mixed(gbfem_operator op64, gbfem_operator op32, gbfem_preconditioner pc32, const gbfem_ir_params* prm,
                      const void* f, void* u, gbfem_solver_info* info) {
  if (!op64 || !op32 || !prm || !f || !u || !info) return set_error(GBFEM_ERR_INVALID, "gbfem_solve_mixed: null argument");
  if (op64->precision != GBFEM_F64 || op32->precision != GBFEM_F32)
    return set_error(GBFEM_ERR_INVALID, "gbfem_solve_mixed: needs an FP64 and an FP32 operator");
  if (op64->ndofs != op32->ndofs) return set_error(GBFEM_ERR_INVALID, "gbfem_solve_mixed: operator sizes differ");
  if (pc32 && pc32->precision != GBFEM_F32) return set_error(GBFEM_ERR_INVALID, "gbfem_solve_mixed: pc must be FP32");
  if (prm->outer_method != 0 && prm->outer_method != GBFEM_SOLVER_FGMRES && prm->outer_method != GBFEM_SOLVER_FCG)
    return set_error(GBFEM_ERR_INVALID, "gbfem_solve_mixed: outer_method must be 0, FGMRES or FCG");
  *info = gbfem_solver_info{};
  const auto t0 = std::chrono::steady_clock::now();
  const long long n = op64->ndofs;
  Ctx c64, c32;
  GBFEM_TRY(c64.setup(GBFEM_F64, n, nullptr));
  GBFEM_TRY(c32.setup(GBFEM_F32, n, nullptr));
  Vecs v64, v32;
  GBFEM_TRY(v64.alloc(2, size_t(n) * 8));
  GBFEM_TRY(v32.alloc(2, size_t(n) * 4));
  void *r = v64[0], *d64 = v64[1], *r32 = v32[0], *d32 = v32[1];
  double ff;
  GBFEM_TRY(c64.dot(f, f, &ff));
  const double fnorm = std::sqrt(ff);
  int inner_total = 0, outer = 0;
  double rel = 0.0, rel_hist[2] = {0.0, 0.0};
  gbfem_solver_params ip = prm->inner;
  ip.error_measure = GBFEM_TOL_RELATIVE;
  if (prm->outer_method != 0) {
    InnerSolvePc ctx{op32, pc32, ip, n, r32, d32};
    gbfem_preconditioner_s px;
    px.kind = PcKind::External;
    px.precision = GBFEM_F64;
    px.n = n;
    px.nloc = op64->nloc;
    px.owns_data = false;
    px.ext_apply = inner_solve_apply;
    px.ext_ctx = &ctx;
    gbfem_solver_params op{};
    GBFEM_TRY(gbfem_solver_params_default(&op));
    op.method = prm->outer_method;
    op.tolerance = prm->tolerance;
    op.error_measure = GBFEM_TOL_RELATIVE;
    op.max_iterations = prm->max_outer;
    op.restart = prm->outer_restart > 0 ? prm->outer_restart : 20;
    op.verbose = prm->inner.verbose;
    // One restart cycle at a time from the current u (restarted FGMRES(m) /
    // truncated FCG(m)), checking the true FP64 residual after each cycle:
    // the flexible method stops on its own residual estimate, which can sit
    // below the true residual, and a cycle without 10 % progress means the
    // rounding floor has been reached.
    gbfem_solver_info oi{};
    int outer_total = 0, applies = 0;
    double prev_rel = 0.0;
    for (int attempt = 0;; ++attempt) {
      const int remaining = prm->max_outer - outer_total;
      if (remaining <= 0) break;
      op.max_iterations = remaining < op.restart ? remaining : op.restart;
      oi = gbfem_solver_info{};
      const int rc = solve_impl(op64, &px, op, f, u, &oi, nullptr);
      if (rc) {
        px.ext_ctx = nullptr;
        return rc;
      }
      const int its = oi.iterations >= 0 ? oi.iterations : -oi.iterations;
      outer_total += its;
      applies += oi.operator_applies;
      GBFEM_TRY(op_apply(op64, u, r, c64));
      GBFEM_TRY(c64.axpby(1.0, f, -1.0, r));
      double rr;
      GBFEM_TRY(c64.dot(r, r, &rr));
      rel = fnorm > 0 ? std::sqrt(rr) / fnorm : std::sqrt(rr);
      if (prm->inner.verbose) std::printf("gbfem mixed flexible outer: %d iterations, true relative residual %.6e\n",
                                          outer_total, rel);
      if (!(rel > prm->tolerance) || its == 0 || oi.status != GBFEM_OK) break;
      if (attempt > 0 && rel > 0.9 * prev_rel) {
        info->stagnated = 1;
        break;
      }
      prev_rel = rel;
    }
    px.ext_ctx = nullptr;
    oi.iterations = outer_total;
    oi.operator_applies = applies;
    info->status = oi.status;
    if (!std::isfinite(rel)) info->status = GBFEM_ERR_NONFINITE;
    info->time_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    info->residual = rel;
    info->converged = (rel <= prm->tolerance && info->status == GBFEM_OK) ? 1 : 0;
    const long long it = ctx.inner_total < INT_MAX ? ctx.inner_total : INT_MAX;
    info->iterations = info->converged ? int(it) : -int(it);
    info->outer_iterations = outer_total;
    info->operator_applies = oi.operator_applies + 1 + ctx.op_applies;
    info->preconditioner_applies = ctx.pc_applies;
    return GBFEM_OK;
  }
  for (outer = 0; outer <= prm->max_outer; ++outer) {
    GBFEM_TRY(op_apply(op64, u, r, c64));
    GBFEM_TRY(c64.axpby(1.0, f, -1.0, r));  // r = f - A u
    double rr;
    GBFEM_TRY(c64.dot(r, r, &rr));
    const double rn = std::sqrt(rr);
    rel = fnorm > 0 ? rn / fnorm : rn;
    if (prm->inner.verbose) std::printf("gbfem IR outer %d : relative residual %.6e\n", outer, rel);
    if (!std::isfinite(rel)) { info->status = GBFEM_ERR_NONFINITE; break; }
    if (rel <= prm->tolerance || outer == prm->max_outer) break;
    // no 10 % progress over two refinement steps: the rounding floor of the
    // FP64 residual is above the tolerance
    if (outer >= 2 && rel > 0.9 * rel_hist[(outer - 2) % 2]) {
      info->stagnated = 1;
      break;
    }
    rel_hist[outer % 2] = rel;
    GBFEM_TRY(gbfem_convert(n, GBFEM_F64, r, GBFEM_F32, r32, nullptr));
    GBFEM_TRY(c32.scal(1.0 / rn, r32));
    GBFEM_TRY(c32.clear(d32));
    gbfem_solver_info ii{};
    GBFEM_TRY(solve_impl(op32, pc32, ip, r32, d32, &ii, nullptr));
    inner_total += ii.iterations >= 0 ? ii.iterations : -ii.iterations;
    c64.op_applies += ii.operator_applies;
    c64.pc_applies += ii.preconditioner_applies;
    GBFEM_TRY(gbfem_convert(n, GBFEM_F32, d32, GBFEM_F64, d64, nullptr));
    GBFEM_TRY(c64.axpby(rn, d64, 1.0, u));
  }
  GBFEM_CUDA_TRY(cudaDeviceSynchronize());
  info->time_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
  info->residual = rel;
  info->converged = (rel <= prm->tolerance && info->status == GBFEM_OK) ? 1 : 0;
  info->iterations = info->converged ? inner_total : -inner_total;
  info->outer_iterations = outer;
  info->operator_applies = c64.op_applies;
  info->preconditioner_applies = c64.pc_applies;
  return GBFEM_OK;
}

}  // extern "C"
