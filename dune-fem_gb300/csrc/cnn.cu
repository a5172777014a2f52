// Learned preconditioner: a 4-level convolutional network (U-Net shape, 32
// channels, 3x3x3 convolutions, BF16 weights and activations, FP32
// accumulation) over the cell grid, trained on the GPU by its own forward and
// backward kernels (cnn_kernels.cuh) with Adam.
//
// Input per cell: the residual's n^3 DG coefficients scaled by 1/rms(r),
// plus log of the cell mean of kappa; output per cell: n^3 coefficients.
// As a preconditioner it is additive with block Jacobi,
//     z = BJ(r) + S rms(r) NN(r / rms(r)),
// so the network only has to supply the smooth error block Jacobi misses.
// Flexible CG judges it with the FP64 residual and falls back to block Jacobi
// when it stagnates (solver.cu).  No counterpart in the reference.
//
// Layers (N = cells per direction, grid levels N, N/2, N/4, N/8):
//   x0 -[1x1, CIN0->32, relu]-> a0 -[3^3]-> s1 -pool-> p1 -[3^3]-> s2 -pool-> p2
//   -[3^3]-> s3 -pool-> p3 -[3^3]-> b4 -up+s3-> u3 -[3^3]-> d3 -up+s2-> u2 -[3^3]->
//   d2 -up+s1-> u1 -[3^3]-> d1 -[1x1, 32->COUT0]-> y
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <cudaTypedefs.h>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "blas.cuh"
#include "cnn_kernels.cuh"
#include "cnn_tc.cuh"
#include "convert.cuh"
#include "gbfem_internal.cuh"
#include "operator_impl.hpp"
#include "solver_impl.hpp"

namespace gbfem {
namespace cnn {

constexpr int C = 32;       // channels
constexpr int NLAYER = 9;   // 0: in-proj, 1..7: 3^3 convs, 8: out-proj

struct Layer {
  int taps = 1, cin = 0, cout = 0;
  long long nw = 0;
  float* w = nullptr;       // FP32 master [taps][cout][cin]
  float* g = nullptr;       // gradient
  float* m = nullptr;       // Adam moments
  float* v = nullptr;
  bf16* wb = nullptr;       // BF16 copy [taps][cout][cin]
  bf16* wbt = nullptr;      // BF16 flipped/transposed [taps][cin][cout] (backward-data)
};

// SplitMix64 + Box-Muller for the He initialisation
static uint64_t sm64(uint64_t& s) {
  uint64_t z = (s += 0x9E3779B97F4A7C15ULL);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
  return z ^ (z >> 31);
}
static double u01(uint64_t& s) { return (double(sm64(s) >> 11) + 0.5) * (1.0 / 9007199254740992.0); }

// wb = bf16(w); wbt[taps-1-t][ci][co] = bf16(w[t][co][ci])
__global__ void refresh_bf16_kernel(const float* __restrict__ w, bf16* __restrict__ wb, bf16* __restrict__ wbt,
                                    int taps, int cout, int cin) {
  const long long n = (long long)taps * cout * cin;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x) {
    const int ci = int(e % cin);
    const int co = int((e / cin) % cout);
    const int t = int(e / ((long long)cin * cout));
    const bf16 b = __float2bfloat16_rn(w[e]);
    wb[e] = b;
    wbt[((long long)(taps - 1 - t) * cin + ci) * cout + co] = b;
  }
}

__global__ void adam_kernel(float* __restrict__ w, const float* __restrict__ g, float* __restrict__ m,
                            float* __restrict__ v, long long n, float lr, float b1, float b2, float eps, float c1,
                            float c2) {
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x) {
    const float gg = g[e];
    const float mm = b1 * m[e] + (1.f - b1) * gg;
    const float vv = b2 * v[e] + (1.f - b2) * gg * gg;
    m[e] = mm;
    v[e] = vv;
    w[e] -= lr * (mm * c1) / (sqrtf(vv * c2) + eps);
  }
}

// x0[p][c]: c < nloc: r[p*nloc+c] / rms(r); c == nloc: log kappa_mean[p]; else 0.
// Channel pairs; each thread handles kEwUnroll of them per iteration and
// issues all their loads first.  The dof values are rounded to FP32 in
// integer arithmetic (convert.cuh), the product is FP32.
constexpr int kEwUnroll = 4;
template <typename T>
__global__ void assemble_input_kernel(const T* __restrict__ r, const float* __restrict__ logk,
                                      const double* __restrict__ rr, long long n, int nloc, int cin,
                                      long long P, int coarse, bf16* __restrict__ x0) {
  const double ms = rr[0] / double(n);
  const float inv = ms > 0.0 ? float(1.0 / sqrt(ms)) : 0.f;
  const unsigned half = unsigned(cin) / 2u, total = unsigned(P) * half, nl = unsigned(nloc);
  __nv_bfloat162* x2 = reinterpret_cast<__nv_bfloat162*>(x0);
  const unsigned stride = gridDim.x * blockDim.x;
  for (unsigned e0 = blockIdx.x * blockDim.x * kEwUnroll + threadIdx.x; e0 < total; e0 += stride * kEwUnroll) {
    T a[kEwUnroll][2];
    float lk[kEwUnroll];
    unsigned cs[kEwUnroll];
#pragma unroll
    for (int u = 0; u < kEwUnroll; ++u) {
      const unsigned e = e0 + u * blockDim.x;
      const unsigned p = e / half, c = 2u * (e - p * half);
      cs[u] = c;
      a[u][0] = a[u][1] = T(0);
      lk[u] = 0.f;
      if (e < total) {
        if (c < nl) a[u][0] = r[p * nl + c];
        if (c + 1 < nl) a[u][1] = r[p * nl + c + 1];
        if (c <= nl && nl <= c + 1) lk[u] = logk[p];
      }
    }
#pragma unroll
    for (int u = 0; u < kEwUnroll; ++u) {
      const unsigned e = e0 + u * blockDim.x;
      if (e >= total) continue;
      float v[2];
#pragma unroll
      for (unsigned j = 0; j < 2; ++j) {
        const unsigned cc = cs[u] + j;
        v[j] = 0.f;
        if (cc < nl) v[j] = (coarse && cc > 0) ? 0.f : to_f32(a[u][j]) * inv;
        else if (cc == nl) v[j] = lk[u];
      }
      x2[e] = __floats2bfloat162_rn(v[0], v[1]);
    }
  }
}

// Partial sums of r_i^2 in FP32 (values rounded to FP32 in integer
// arithmetic): one per block, fixed order; the normalisation rms(r) needs no
// more precision, and an FP64 product per dof would bind on the FP64 pipe.
template <typename T>
__global__ void sumsq_partial_kernel(const T* __restrict__ r, unsigned n, double* __restrict__ part) {
  __shared__ float red[256];
  float acc[kEwUnroll] = {0.f, 0.f, 0.f, 0.f};
  const unsigned stride = gridDim.x * blockDim.x;
  for (unsigned e0 = blockIdx.x * blockDim.x * kEwUnroll + threadIdx.x; e0 < n; e0 += stride * kEwUnroll) {
    T a[kEwUnroll];
#pragma unroll
    for (int u = 0; u < kEwUnroll; ++u) {
      const unsigned e = e0 + u * blockDim.x;
      a[u] = e < n ? r[e] : T(0);
    }
#pragma unroll
    for (int u = 0; u < kEwUnroll; ++u) {
      const float v = to_f32(a[u]);
      acc[u] = fmaf(v, v, acc[u]);
    }
  }
  red[threadIdx.x] = (acc[0] + acc[1]) + (acc[2] + acc[3]);
  __syncthreads();
  for (int o = 128; o > 0; o >>= 1) {
    if (int(threadIdx.x) < o) red[threadIdx.x] += red[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) part[blockIdx.x] = double(red[0]);
}

// out[0] = sum of the partials in block order
__global__ void sum_partials_kernel(const double* __restrict__ part, int np, double* __restrict__ out) {
  __shared__ double red[256];
  double s = 0.0;
  for (int i = threadIdx.x; i < np; i += 256) s += part[i];
  red[threadIdx.x] = s;
  __syncthreads();
  for (int o = 128; o > 0; o >>= 1) {
    if (int(threadIdx.x) < o) red[threadIdx.x] += red[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) out[0] = red[0];
}

// out[0] = sum_p r[p*nloc]^2: the coarse mode's normalisation (the cell
// means of r only), one CTA of 256 threads, fixed summation order
template <typename T>
__global__ void coarse_sumsq_kernel(const T* __restrict__ r, int nloc, long long P, double* __restrict__ out) {
  __shared__ double part[256];
  double s = 0.0;
  for (long long p = threadIdx.x; p < P; p += 256) {
    const double v = double(r[p * nloc]);
    s = fma(v, v, s);
  }
  part[threadIdx.x] = s;
  __syncthreads();
  for (int o = 128; o > 0; o >>= 1) {
    if (threadIdx.x < o) part[threadIdx.x] += part[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) out[0] = part[0];
}

// z[p*nloc+l] (+)= S * rms(r) * y[p][l]: the scale and the product in FP32,
// widened to T in integer arithmetic (an FP64 add only when accumulating);
// kEwUnroll values per thread and iteration, loads first
template <typename T>
__global__ void emit_output_kernel(const float* __restrict__ y, const double* __restrict__ rr, long long n, int nloc,
                                   int cout, long long P, float S, int accumulate, int coarse, T* __restrict__ z) {
  const float sc = float(double(S) * sqrt(rr[0] / double(n)));
  const unsigned nl = unsigned(nloc), total = unsigned(P) * nl, co = unsigned(cout);
  const unsigned stride = gridDim.x * blockDim.x;
  for (unsigned e0 = blockIdx.x * blockDim.x * kEwUnroll + threadIdx.x; e0 < total; e0 += stride * kEwUnroll) {
    float yv[kEwUnroll];
    T zv[kEwUnroll];
#pragma unroll
    for (int u = 0; u < kEwUnroll; ++u) {
      const unsigned e = e0 + u * blockDim.x;
      yv[u] = 0.f;
      zv[u] = T(0);
      if (e < total) {
        const unsigned p = e / nl, l = e - p * nl;
        if (!(coarse && l > 0)) yv[u] = y[p * co + l];
        if (accumulate) zv[u] = z[e];
      }
    }
#pragma unroll
    for (int u = 0; u < kEwUnroll; ++u) {
      const unsigned e = e0 + u * blockDim.x;
      if (e < total) z[e] = accumulate ? T(zv[u] + from_f32<T>(sc * yv[u])) : from_f32<T>(sc * yv[u]);
    }
  }
}

// diff[p][l] = y[p][l] - t[p*nloc+l] / (S rms) (0 on padded channels, and in
// coarse mode on every channel but the cell mean); dy = 2 diff / (P*nloc)
// (coarse: 2 diff / P); FP32 arithmetic
template <typename T>
__global__ void loss_grad_kernel(const float* __restrict__ y, const T* __restrict__ t, const double* __restrict__ rr,
                                 long long n, int nloc, int cout, long long P, float S, int coarse,
                                 float* __restrict__ diff, bf16* __restrict__ dy) {
  const double rms = sqrt(rr[0] / double(n));
  const float inv = rms > 0.0 ? float(1.0 / (double(S) * rms)) : 0.f;
  const unsigned co = unsigned(cout), nl = unsigned(nloc), total = unsigned(P) * co;
  const unsigned lim = coarse ? 1u : nl;
  const float scale = 2.f / float(coarse ? P : P * nloc);
  for (unsigned e = blockIdx.x * blockDim.x + threadIdx.x; e < total; e += gridDim.x * blockDim.x) {
    const unsigned p = e / co, c = e - p * co;
    float d = 0.f;
    if (c < lim) d = y[e] - to_f32(t[p * nl + c]) * inv;
    diff[e] = d;
    dy[e] = __float2bfloat16_rn(scale * d);
  }
}

// dy[p][c] = S rms(r) g[p*nloc + c] (chain rule through z = S rms(r) y); 0 on padded channels
template <typename T>
__global__ void grad_from_dofs_kernel(const T* __restrict__ g, const double* __restrict__ rr, long long n, int nloc,
                                      int cout, long long P, float S, int coarse, bf16* __restrict__ dy) {
  const float sc = float(double(S) * sqrt(rr[0] / double(n)));
  const unsigned co = unsigned(cout), nl = unsigned(nloc), total = unsigned(P) * co;
  for (unsigned e = blockIdx.x * blockDim.x + threadIdx.x; e < total; e += gridDim.x * blockDim.x) {
    const unsigned p = e / co, c = e - p * co;
    const float v = (c < nl && !(coarse && c > 0)) ? sc * to_f32(g[p * nl + c]) : 0.f;
    dy[e] = __float2bfloat16_rn(v);
  }
}

// logk[p] = log(kappa coefficient 0 of cell p) (the cell mean for the orthonormal basis)
template <typename T>
__global__ void logkappa_kernel(const T* __restrict__ kappa, int nloc, long long P, float* __restrict__ logk) {
  for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < P; p += (long long)gridDim.x * blockDim.x) {
    const double k = kappa ? double(kappa[p * nloc]) : 1.0;
    logk[p] = float(log(k > 1e-300 ? k : 1e-300));
  }
}

}  // namespace cnn
}  // namespace gbfem

using namespace gbfem;
using namespace gbfem::cnn;

struct gbfem_cnn_s {
  int N[4] = {0, 0, 0, 0};   // cells per direction at each level
  long long P[4] = {0, 0, 0, 0};
  int nloc = 0, cin0 = 0, cout0 = 0;
  long long ndofs = 0;
  float S = 1.0f;            // output scale
  int adam_t = 0;
  int coarse = 0;            // coarse mode: input the cell means of r, output the cell means only
  Layer L[NLAYER];
  // activations (BF16, channels-last)
  bf16 *x0 = nullptr, *a0 = nullptr, *s1 = nullptr, *p1 = nullptr, *s2 = nullptr, *p2 = nullptr, *s3 = nullptr,
       *p3 = nullptr, *b4 = nullptr, *u3 = nullptr, *d3 = nullptr, *u2 = nullptr, *d2 = nullptr, *u1 = nullptr,
       *d1 = nullptr;
  float* y = nullptr;
  // activation gradients: two buffers per level
  bf16* dy = nullptr;
  bf16* G[4][2] = {{nullptr, nullptr}, {nullptr, nullptr}, {nullptr, nullptr}, {nullptr, nullptr}};
  float* diff = nullptr;
  float* wpart = nullptr;    // weight-gradient partials
  long long wpart_elems = 0;
  float* logk = nullptr;
  double* d_rr = nullptr;    // r.r
  double* d_loss = nullptr;
  double* d_partial = nullptr;
  double* h_loss = nullptr;
  int* status = nullptr;     // set by a tensor-core convolution whose wait ran out
  struct ConvMap {
    CUtensorMap map;         // 4-D [z][y][x][32 channels] BF16, box of 128 positions, 64-byte swizzle
    const bf16* ptr;
    int N;
  };
  std::vector<ConvMap> conv_maps;  // the inputs of the 3x3x3 convolutions
  int conv_engine = GBFEM_CNN_CONV_TENSOR_CORE;
  std::vector<void*> allocs;
};

static int cnn_alloc(gbfem_cnn_s* c, void** p, size_t bytes) {
  cudaError_t e = cudaMalloc(p, bytes);
  if (e != cudaSuccess) return set_cuda_error(e, "gbfem_cnn: allocation");
  c->allocs.push_back(*p);
  return GBFEM_OK;
}

template <int CIN, int COUT, int TAPS, bool RELU, typename TOUT>
static int launch_conv(const bf16* in, const bf16* w, TOUT* out, int N, cudaStream_t s) {
  const size_t sm = size_t(TAPS) * COUT * CIN * sizeof(bf16);
  auto k = conv_fwd_kernel<CIN, COUT, TAPS, RELU, TOUT>;
  GBFEM_CUDA_TRY(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, int(sm)));
  const long long P = (long long)N * N * N;
  const unsigned blocks = unsigned((P + 63) / 64);
  k<<<blocks, 128, sm, s>>>(in, w, out, N);
  GBFEM_CUDA_TRY(cudaGetLastError());
  return GBFEM_OK;
}

// cuTensorMapEncodeTiled through the runtime's driver entry point (no link
// dependency on the driver library); null if unavailable
static PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  static bool tried = false;
  if (!tried) {
    tried = true;
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
  }
  return fn;
}

static bool tma_conv_level(int N) { return N >= 8 && N <= 256 && (N & (N - 1)) == 0; }

// tensor map of an activation buffer of an N^3 grid for conv_tma_kernel
static int conv_map(gbfem_cnn_s* c, const bf16* ptr, int N) {
  if (!tma_conv_level(N)) return GBFEM_OK;
  PFN_cuTensorMapEncodeTiled_v12000 enc = tensor_map_encoder();
  if (!enc) return GBFEM_OK;  // the mma.sync engine serves
  gbfem_cnn_s::ConvMap m{};
  m.ptr = ptr;
  m.N = N;
  const cuuint64_t dims[4] = {cuuint64_t(C), cuuint64_t(N), cuuint64_t(N), cuuint64_t(N)};
  const cuuint64_t strides[3] = {cuuint64_t(C) * 2, cuuint64_t(C) * 2 * N, cuuint64_t(C) * 2 * N * N};
  const cuuint32_t bx = N < kCtM ? N : kCtM;
  const cuuint32_t by = (kCtM / bx) < cuuint32_t(N) ? (kCtM / bx) : cuuint32_t(N);
  const cuuint32_t box[4] = {cuuint32_t(C), bx, by, cuuint32_t(kCtM) / (bx * by)};
  const cuuint32_t estr[4] = {1, 1, 1, 1};
  const CUresult r = enc(&m.map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 4, const_cast<bf16*>(ptr), dims, strides, box, estr,
                         CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_64B, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                         CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) return set_error(GBFEM_ERR_CUDA, "gbfem_cnn: tensor map of a convolution input");
  c->conv_maps.push_back(m);
  return GBFEM_OK;
}

// The 3x3x3 32 -> 32 convolution (forward: RELU; backward-data: the
// flipped weights, no RELU) on the engine the network is set to: TMA +
// tcgen05 where the level allows it (N a power of two >= 8), else mma.sync.
template <bool RELU>
static int launch_conv27(gbfem_cnn_s* c, const bf16* in, const bf16* w, bf16* out, int N, cudaStream_t s) {
  const CUtensorMap* map = nullptr;
  if (c->conv_engine == GBFEM_CNN_CONV_TENSOR_CORE)
    for (const auto& m : c->conv_maps)
      if (m.ptr == in && m.N == N) map = &m.map;
  if (!map) return launch_conv<C, C, 27, RELU, bf16>(in, w, out, N, s);
  static_assert(C == kCtN, "the tensor-core convolution is 32 -> 32 channels");
  static int sms = 0;
  if (sms == 0) {
    int dev = 0, v = 0;
    if (cudaGetDevice(&dev) == cudaSuccess && cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev) ==
                                                  cudaSuccess && v > 0)
      sms = v;
    else
      sms = 152;
  }
  const long long P = (long long)N * N * N;
  const long long ntiles = P / kCtM;
  const long long grid = ntiles < sms ? ntiles : sms;
  GBFEM_CUDA_TRY(cudaFuncSetAttribute(conv_tma_kernel<RELU>, cudaFuncAttributeMaxDynamicSharedMemorySize, int(kCtSmem)));
  conv_tma_kernel<RELU><<<unsigned(grid), kCtThreads, kCtSmem, s>>>(*map, w, out, N, c->status);
  GBFEM_CUDA_TRY(cudaGetLastError());
  return GBFEM_OK;
}

// positions per weight-gradient chunk for a grid of P positions
static int wgrad_chunk(long long P) {
  int pch = 1024;
  while (pch > 64 && (P + pch - 1) / pch < 152) pch /= 2;
  return pch;
}

template <int CIN, int COUT, int TAPS>
static int launch_wgrad(gbfem_cnn_s* c, const bf16* in, const bf16* dout, float* dw, int N, cudaStream_t s) {
  const long long P = (long long)N * N * N;
  const int pch = wgrad_chunk(P);
  const long long nch = (P + pch - 1) / pch;
  if (nch * TAPS * COUT * CIN > c->wpart_elems)
    return set_error(GBFEM_ERR_INVALID, "gbfem_cnn: weight-gradient scratch too small");
  conv_wgrad_kernel<CIN, COUT, TAPS><<<dim3(unsigned(nch), TAPS), 128, 0, s>>>(in, dout, c->wpart, N, pch);
  GBFEM_CUDA_TRY(cudaGetLastError());
  const int nelem = TAPS * COUT * CIN;
  wgrad_reduce_kernel<<<(nelem + 255) / 256, 256, 0, s>>>(c->wpart, dw, int(nch), nelem);
  GBFEM_CUDA_TRY(cudaGetLastError());
  return GBFEM_OK;
}

static int grid1(long long n) { return stream_grid(n); }

static int conv_in_fwd(gbfem_cnn_s* c, cudaStream_t s) {
  switch (c->cin0) {
    case 32: return launch_conv<32, C, 1, true, bf16>(c->x0, c->L[0].wb, c->a0, c->N[0], s);
    case 80: return launch_conv<80, C, 1, true, bf16>(c->x0, c->L[0].wb, c->a0, c->N[0], s);
    case 128: return launch_conv<128, C, 1, true, bf16>(c->x0, c->L[0].wb, c->a0, c->N[0], s);
  }
  return set_error(GBFEM_ERR_NOT_IMPLEMENTED, "gbfem_cnn: input width");
}
static int conv_out_fwd(gbfem_cnn_s* c, cudaStream_t s) {
  switch (c->cout0) {
    case 32: return launch_conv<C, 32, 1, false, float>(c->d1, c->L[8].wb, c->y, c->N[0], s);
    case 64: return launch_conv<C, 64, 1, false, float>(c->d1, c->L[8].wb, c->y, c->N[0], s);
    case 128: return launch_conv<C, 128, 1, false, float>(c->d1, c->L[8].wb, c->y, c->N[0], s);
  }
  return set_error(GBFEM_ERR_NOT_IMPLEMENTED, "gbfem_cnn: output width");
}

static int cnn_forward(gbfem_cnn_s* c, cudaStream_t s) {
  const int* N = c->N;
  GBFEM_TRY(conv_in_fwd(c, s));
  GBFEM_TRY((launch_conv27<true>(c, c->a0, c->L[1].wb, c->s1, N[0], s)));
  pool_fwd_kernel<<<grid1(c->P[1] * C), 256, 0, s>>>(c->s1, c->p1, N[0], C);
  GBFEM_TRY((launch_conv27<true>(c, c->p1, c->L[2].wb, c->s2, N[1], s)));
  pool_fwd_kernel<<<grid1(c->P[2] * C), 256, 0, s>>>(c->s2, c->p2, N[1], C);
  GBFEM_TRY((launch_conv27<true>(c, c->p2, c->L[3].wb, c->s3, N[2], s)));
  pool_fwd_kernel<<<grid1(c->P[3] * C), 256, 0, s>>>(c->s3, c->p3, N[2], C);
  GBFEM_TRY((launch_conv27<true>(c, c->p3, c->L[4].wb, c->b4, N[3], s)));
  up_add_kernel<<<grid1(c->P[2] * C), 256, 0, s>>>(c->b4, c->s3, c->u3, N[2], C);
  GBFEM_TRY((launch_conv27<true>(c, c->u3, c->L[5].wb, c->d3, N[2], s)));
  up_add_kernel<<<grid1(c->P[1] * C), 256, 0, s>>>(c->d3, c->s2, c->u2, N[1], C);
  GBFEM_TRY((launch_conv27<true>(c, c->u2, c->L[6].wb, c->d2, N[1], s)));
  up_add_kernel<<<grid1(c->P[0] * C), 256, 0, s>>>(c->d2, c->s1, c->u1, N[0], C);
  GBFEM_TRY((launch_conv27<true>(c, c->u1, c->L[7].wb, c->d1, N[0], s)));
  GBFEM_TRY(conv_out_fwd(c, s));
  GBFEM_CUDA_TRY(cudaGetLastError());
  return GBFEM_OK;
}

// Backward from dy (BF16 [P0][cout0]) into every L[i].g.  Level of each
// tensor in brackets; G[l][0..1] are the two gradient buffers of level l.
static int cnn_backward(gbfem_cnn_s* c, cudaStream_t s) {
  const int* N = c->N;
  const long long* P = c->P;
  bf16 *G00 = c->G[0][0], *G01 = c->G[0][1], *G10 = c->G[1][0], *G11 = c->G[1][1];
  bf16 *G20 = c->G[2][0], *G21 = c->G[2][1], *G30 = c->G[3][0], *G31 = c->G[3][1];
  // y = W8 d1 [0]:  dW8;  G00 = (W8^T dy) * (d1 > 0)
  switch (c->cout0) {
    case 32:
      GBFEM_TRY((launch_wgrad<C, 32, 1>(c, c->d1, c->dy, c->L[8].g, N[0], s)));
      GBFEM_TRY((launch_conv<32, C, 1, false, bf16>(c->dy, c->L[8].wbt, G00, N[0], s)));
      break;
    case 64:
      GBFEM_TRY((launch_wgrad<C, 64, 1>(c, c->d1, c->dy, c->L[8].g, N[0], s)));
      GBFEM_TRY((launch_conv<64, C, 1, false, bf16>(c->dy, c->L[8].wbt, G00, N[0], s)));
      break;
    case 128:
      GBFEM_TRY((launch_wgrad<C, 128, 1>(c, c->d1, c->dy, c->L[8].g, N[0], s)));
      GBFEM_TRY((launch_conv<128, C, 1, false, bf16>(c->dy, c->L[8].wbt, G00, N[0], s)));
      break;
    default: return set_error(GBFEM_ERR_NOT_IMPLEMENTED, "gbfem_cnn: output width");
  }
  relu_mask_kernel<<<grid1(P[0] * C), 256, 0, s>>>(G00, c->d1, P[0] * C);
  // d1 = relu(W7 * u1) [0]:  dW7;  G01 = du1 = W7^T * G00
  GBFEM_TRY((launch_wgrad<C, C, 27>(c, c->u1, G00, c->L[7].g, N[0], s)));
  GBFEM_TRY((launch_conv27<false>(c, G00, c->L[7].wbt, G01, N[0], s)));
  // u1 = up(d2) + s1:  G10 = dd2 = downsum(du1) * (d2 > 0) [1]
  up_bwd_mask_kernel<<<grid1(P[1] * C), 256, 0, s>>>(G01, c->d2, G10, N[0], C);
  // d2 = relu(W6 * u2) [1]:  dW6;  G11 = du2
  GBFEM_TRY((launch_wgrad<C, C, 27>(c, c->u2, G10, c->L[6].g, N[1], s)));
  GBFEM_TRY((launch_conv27<false>(c, G10, c->L[6].wbt, G11, N[1], s)));
  // u2 = up(d3) + s2:  G20 = dd3 [2]
  up_bwd_mask_kernel<<<grid1(P[2] * C), 256, 0, s>>>(G11, c->d3, G20, N[1], C);
  // d3 = relu(W5 * u3) [2]:  dW5;  G21 = du3
  GBFEM_TRY((launch_wgrad<C, C, 27>(c, c->u3, G20, c->L[5].g, N[2], s)));
  GBFEM_TRY((launch_conv27<false>(c, G20, c->L[5].wbt, G21, N[2], s)));
  // u3 = up(b4) + s3:  G30 = db4 [3]
  up_bwd_mask_kernel<<<grid1(P[3] * C), 256, 0, s>>>(G21, c->b4, G30, N[2], C);
  // b4 = relu(W4 * p3) [3]:  dW4;  G31 = dp3
  GBFEM_TRY((launch_wgrad<C, C, 27>(c, c->p3, G30, c->L[4].g, N[3], s)));
  GBFEM_TRY((launch_conv27<false>(c, G30, c->L[4].wbt, G31, N[3], s)));
  // p3 = pool(s3):  G20 = ds3 = (du3 + pool_back(dp3)) * (s3 > 0) [2]
  pool_bwd_add_mask_kernel<<<grid1(P[2] * C), 256, 0, s>>>(G21, G31, c->s3, G20, N[2], C);
  // s3 = relu(W3 * p2) [2]:  dW3;  G21 = dp2
  GBFEM_TRY((launch_wgrad<C, C, 27>(c, c->p2, G20, c->L[3].g, N[2], s)));
  GBFEM_TRY((launch_conv27<false>(c, G20, c->L[3].wbt, G21, N[2], s)));
  // p2 = pool(s2):  G10 = ds2 = (du2 + pool_back(dp2)) * (s2 > 0) [1]
  pool_bwd_add_mask_kernel<<<grid1(P[1] * C), 256, 0, s>>>(G11, G21, c->s2, G10, N[1], C);
  // s2 = relu(W2 * p1) [1]:  dW2;  G11 = dp1
  GBFEM_TRY((launch_wgrad<C, C, 27>(c, c->p1, G10, c->L[2].g, N[1], s)));
  GBFEM_TRY((launch_conv27<false>(c, G10, c->L[2].wbt, G11, N[1], s)));
  // p1 = pool(s1):  G00 = ds1 = (du1 + pool_back(dp1)) * (s1 > 0) [0]
  pool_bwd_add_mask_kernel<<<grid1(P[0] * C), 256, 0, s>>>(G01, G11, c->s1, G00, N[0], C);
  // s1 = relu(W1 * a0) [0]:  dW1;  G01 = da0 = (W1^T * ds1) * (a0 > 0)
  GBFEM_TRY((launch_wgrad<C, C, 27>(c, c->a0, G00, c->L[1].g, N[0], s)));
  GBFEM_TRY((launch_conv27<false>(c, G00, c->L[1].wbt, G01, N[0], s)));
  relu_mask_kernel<<<grid1(P[0] * C), 256, 0, s>>>(G01, c->a0, P[0] * C);
  // a0 = relu(W0 x0) [0]:  dW0
  switch (c->cin0) {
    case 32: GBFEM_TRY((launch_wgrad<32, C, 1>(c, c->x0, G01, c->L[0].g, N[0], s))); break;
    case 80: GBFEM_TRY((launch_wgrad<80, C, 1>(c, c->x0, G01, c->L[0].g, N[0], s))); break;
    case 128: GBFEM_TRY((launch_wgrad<128, C, 1>(c, c->x0, G01, c->L[0].g, N[0], s))); break;
    default: return set_error(GBFEM_ERR_NOT_IMPLEMENTED, "gbfem_cnn: input width");
  }
  GBFEM_CUDA_TRY(cudaGetLastError());
  return GBFEM_OK;
}

static int refresh_bf16(gbfem_cnn_s* c, cudaStream_t s) {
  for (int i = 0; i < NLAYER; ++i) {
    Layer& l = c->L[i];
    refresh_bf16_kernel<<<grid1(l.nw), 256, 0, s>>>(l.w, l.wb, l.wbt, l.taps, l.cout, l.cin);
  }
  GBFEM_CUDA_TRY(cudaGetLastError());
  return GBFEM_OK;
}

// Values the normalisation rms(r) = sqrt(rr / nnorm) is taken over: every
// dof, or in coarse mode the cell means only.
static long long cnn_nnorm(const gbfem_cnn_s* c) { return c->coarse ? c->P[0] : c->ndofs; }

template <typename T>
static int cnn_input(gbfem_cnn_s* c, const void* r, cudaStream_t s) {
  if (c->coarse)
    coarse_sumsq_kernel<T><<<1, 256, 0, s>>>(static_cast<const T*>(r), c->nloc, c->P[0], c->d_rr);
  else
  {
    const int np = grid1(c->ndofs / kEwUnroll);
    sumsq_partial_kernel<T><<<np, 256, 0, s>>>(static_cast<const T*>(r), unsigned(c->ndofs), c->d_partial);
    sum_partials_kernel<<<1, 256, 0, s>>>(c->d_partial, np, c->d_rr);
  }
  assemble_input_kernel<T><<<grid1(c->P[0] * c->cin0 / 2 / kEwUnroll), 256, 0, s>>>(static_cast<const T*>(r), c->logk, c->d_rr,
                                                                    cnn_nnorm(c), c->nloc, c->cin0, c->P[0], c->coarse,
                                                                    c->x0);
  GBFEM_CUDA_TRY(cudaGetLastError());
  return GBFEM_OK;
}

static int cnn_apply(gbfem_cnn_s* c, int precision, const void* r, void* z, int accumulate, cudaStream_t s) {
  if (precision == GBFEM_F64) GBFEM_TRY(cnn_input<double>(c, r, s));
  else GBFEM_TRY(cnn_input<float>(c, r, s));
  GBFEM_TRY(cnn_forward(c, s));
  if (precision == GBFEM_F64)
    emit_output_kernel<double><<<grid1(c->ndofs / kEwUnroll), 256, 0, s>>>(c->y, c->d_rr, cnn_nnorm(c), c->nloc, c->cout0, c->P[0],
                                                               c->S, accumulate, c->coarse, static_cast<double*>(z));
  else
    emit_output_kernel<float><<<grid1(c->ndofs / kEwUnroll), 256, 0, s>>>(c->y, c->d_rr, cnn_nnorm(c), c->nloc, c->cout0, c->P[0],
                                                              c->S, accumulate, c->coarse, static_cast<float*>(z));
  GBFEM_CUDA_TRY(cudaGetLastError());
  return GBFEM_OK;
}

// forward + loss + backward (gradients in L[i].g); loss to *loss (synchronises)
static int cnn_loss_grad(gbfem_cnn_s* c, int precision, const void* r, const void* target, double* loss,
                         cudaStream_t s) {
  if (precision == GBFEM_F64) GBFEM_TRY(cnn_input<double>(c, r, s));
  else GBFEM_TRY(cnn_input<float>(c, r, s));
  GBFEM_TRY(cnn_forward(c, s));
  const long long ny = c->P[0] * c->cout0;
  if (precision == GBFEM_F64)
    loss_grad_kernel<double><<<grid1(ny), 256, 0, s>>>(c->y, static_cast<const double*>(target), c->d_rr,
                                                       cnn_nnorm(c), c->nloc, c->cout0, c->P[0], c->S, c->coarse,
                                                       c->diff, c->dy);
  else
    loss_grad_kernel<float><<<grid1(ny), 256, 0, s>>>(c->y, static_cast<const float*>(target), c->d_rr,
                                                      cnn_nnorm(c), c->nloc, c->cout0, c->P[0], c->S, c->coarse,
                                                      c->diff, c->dy);
  GBFEM_CUDA_TRY(cudaGetLastError());
  GBFEM_TRY(cnn_backward(c, s));
  if (loss) {
    GBFEM_TRY(dot_device(GBFEM_F32, ny, c->diff, c->diff, c->d_loss, c->d_partial, s));
    GBFEM_CUDA_TRY(cudaMemcpyAsync(c->h_loss, c->d_loss, sizeof(double), cudaMemcpyDeviceToHost, s));
    GBFEM_CUDA_TRY(cudaStreamSynchronize(s));
    *loss = c->h_loss[0] / double(c->coarse ? c->P[0] : c->P[0] * c->nloc);
  }
  return GBFEM_OK;
}

struct LearnedCtx {
  gbfem_cnn_s* cnn;
  gbfem_preconditioner bj;  // not owned
  gbfem_operator op;        // not owned; NULL = additive form
  void* t = nullptr;        // work vectors of the two-level form
  void* at = nullptr;
  double* dots = nullptr;   // n.r, n.An (device)
  double* partial = nullptr;
  ~LearnedCtx() {
    if (t) cudaFree(t);
    if (at) cudaFree(at);
    if (dots) cudaFree(dots);
    if (partial) cudaFree(partial);
  }
};

template <typename T>
__global__ void learned_add_kernel(long long n, const T* __restrict__ a, T* __restrict__ z) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    z[i] += a[i];
}

// z *= alpha, t = r - alpha az with alpha = (n.r) / (n.An), or 0 where n.An
// is not positive (every thread computes alpha from the two device dots)
template <typename T>
__global__ void learned_scale_kernel(long long n, const double* __restrict__ dots, const T* __restrict__ r,
                                     const T* __restrict__ az, T* __restrict__ z, T* __restrict__ t) {
  const double b = dots[1];
  const double alpha = (b > 0.0 && isfinite(b) && isfinite(dots[0])) ? dots[0] / b : 0.0;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    z[i] = T(alpha * double(z[i]));
    t[i] = T(double(r[i]) - alpha * double(az[i]));
  }
}

// Additive:   z = BJ(r) + NN(r)
// Two-level:  n = NN(r) (coarse mode: the shape of the error's cell means),
//             z = alpha n with the Galerkin-optimal alpha = n.r / n.An (the
//             A-norm projection of the error onto span{n}), then one
//             block-Jacobi smoothing step z += BJ(r - A z).  A network whose
//             output does not correlate with the error gives alpha ~ 0, i.e.
//             block Jacobi.
static int ext_learned_apply(void* ctx, const void* r, void* z, cudaStream_t s) {
  LearnedCtx* lc = static_cast<LearnedCtx*>(ctx);
  gbfem_cnn_s* c = lc->cnn;
  const int prec = lc->bj ? lc->bj->precision : GBFEM_F64;
  if (!lc->op) {
    if (lc->bj) GBFEM_TRY(precond_apply(lc->bj, r, z, s));
    else GBFEM_CUDA_TRY(cudaMemsetAsync(z, 0, size_t(c->ndofs) * (prec == GBFEM_F64 ? 8 : 4), s));
    return cnn_apply(c, prec, r, z, 1, s);
  }
  GBFEM_TRY(cnn_apply(c, prec, r, z, 0, s));
  GBFEM_TRY(gbfem_operator_apply(lc->op, z, lc->at, s));
  const long long n = c->ndofs;
  GBFEM_TRY(dot_device(prec, n, z, r, lc->dots, lc->partial, s));
  GBFEM_TRY(dot_device(prec, n, z, lc->at, lc->dots + 1, lc->partial, s));
  if (prec == GBFEM_F64) {
    learned_scale_kernel<double><<<grid1(n), 256, 0, s>>>(n, lc->dots, (const double*)r, (const double*)lc->at,
                                                          (double*)z, (double*)lc->t);
  } else {
    learned_scale_kernel<float><<<grid1(n), 256, 0, s>>>(n, lc->dots, (const float*)r, (const float*)lc->at,
                                                         (float*)z, (float*)lc->t);
  }
  GBFEM_TRY(precond_apply(lc->bj, lc->t, lc->at, s));
  if (prec == GBFEM_F64) learned_add_kernel<double><<<grid1(n), 256, 0, s>>>(n, (const double*)lc->at, (double*)z);
  else learned_add_kernel<float><<<grid1(n), 256, 0, s>>>(n, (const float*)lc->at, (float*)z);
  GBFEM_CUDA_TRY(cudaGetLastError());
  return GBFEM_OK;
}

static void ext_learned_destroy(void* ctx) { delete static_cast<LearnedCtx*>(ctx); }

extern "C" {

int gbfem_cnn_create(int order, int cells, uint64_t seed, gbfem_cnn* out) {
  if (!out) return set_error(GBFEM_ERR_INVALID, "gbfem_cnn_create: null out");
  *out = nullptr;
  if (order < 1 || order > 4) return set_error(GBFEM_ERR_INVALID, "gbfem_cnn_create: order 1..4");
  if (cells < 8 || cells % 8) return set_error(GBFEM_ERR_INVALID, "gbfem_cnn_create: cells must be a multiple of 8");
  if (cells > 256)  // the elementwise kernels index with 32 bits
    return set_error(GBFEM_ERR_NOT_IMPLEMENTED, "gbfem_cnn_create: at most 256 cells per direction");
  auto* c = new (std::nothrow) gbfem_cnn_s();
  if (!c) return set_error(GBFEM_ERR_INVALID, "out of host memory");
  const int n = order + 1;
  c->nloc = n * n * n;
  c->cin0 = c->nloc + 1 <= 32 ? 32 : (c->nloc + 1 <= 80 ? 80 : 128);
  c->cout0 = c->nloc <= 32 ? 32 : (c->nloc <= 64 ? 64 : 128);
  for (int l = 0; l < 4; ++l) {
    c->N[l] = cells >> l;
    c->P[l] = (long long)c->N[l] * c->N[l] * c->N[l];
  }
  c->ndofs = c->P[0] * c->nloc;
  int rc = GBFEM_OK;
  auto A = [&](void** p, size_t b) { if (rc == GBFEM_OK) rc = cnn_alloc(c, p, b); };
  // layers
  for (int i = 0; i < NLAYER; ++i) {
    Layer& l = c->L[i];
    l.taps = (i == 0 || i == 8) ? 1 : 27;
    l.cin = i == 0 ? c->cin0 : C;
    l.cout = i == 8 ? c->cout0 : C;
    l.nw = (long long)l.taps * l.cin * l.cout;
    A((void**)&l.w, l.nw * 4);
    A((void**)&l.g, l.nw * 4);
    A((void**)&l.m, l.nw * 4);
    A((void**)&l.v, l.nw * 4);
    A((void**)&l.wb, l.nw * 2);
    A((void**)&l.wbt, l.nw * 2);
  }
  const size_t b16 = 2;
  A((void**)&c->x0, c->P[0] * c->cin0 * b16);
  bf16** lv0[] = {&c->a0, &c->s1, &c->u1, &c->d1};
  for (auto p : lv0) A((void**)p, c->P[0] * C * b16);
  bf16** lv1[] = {&c->p1, &c->s2, &c->u2, &c->d2};
  for (auto p : lv1) A((void**)p, c->P[1] * C * b16);
  bf16** lv2[] = {&c->p2, &c->s3, &c->u3, &c->d3};
  for (auto p : lv2) A((void**)p, c->P[2] * C * b16);
  bf16** lv3[] = {&c->p3, &c->b4};
  for (auto p : lv3) A((void**)p, c->P[3] * C * b16);
  for (int l = 0; l < 4; ++l)
    for (int k = 0; k < 2; ++k) A((void**)&c->G[l][k], c->P[l] * C * b16);
  A((void**)&c->y, c->P[0] * c->cout0 * 4);
  A((void**)&c->dy, c->P[0] * c->cout0 * b16);
  A((void**)&c->diff, c->P[0] * c->cout0 * 4);
  long long wp = 0;
  for (int l = 0; l < 4; ++l) {
    const long long nch = (c->P[l] + wgrad_chunk(c->P[l]) - 1) / wgrad_chunk(c->P[l]);
    const long long need = nch * (l == 0 ? std::max<long long>(27LL * C * C, (long long)C * std::max(c->cin0, c->cout0))
                                         : 27LL * C * C);
    wp = std::max(wp, need);
  }
  c->wpart_elems = wp;
  A((void**)&c->wpart, wp * 4);
  A((void**)&c->logk, c->P[0] * 4);
  A((void**)&c->d_rr, 64);
  A((void**)&c->d_loss, 64);
  A((void**)&c->status, 64);
  // partials of the loss reduction (gbfem's dot) and of the input's sum of
  // squares (one per block of sumsq_partial_kernel, at most stream_grid(ndofs))
  A((void**)&c->d_partial, sizeof(double) * (std::max<long long>(dot_num_partials(std::max(c->ndofs, c->P[0] * c->cout0)),
                                                                  stream_grid(c->ndofs)) + 8));
  if (rc == GBFEM_OK) {
    cudaError_t e = cudaMallocHost(&c->h_loss, 64);
    if (e != cudaSuccess) rc = set_cuda_error(e, "gbfem_cnn_create");
  }
  if (rc) { gbfem_cnn_destroy(c); return rc; }
  // He initialisation (seeded, host), zero Adam state
  uint64_t st = seed;
  for (int i = 0; i < NLAYER && rc == GBFEM_OK; ++i) {
    Layer& l = c->L[i];
    std::vector<float> w(l.nw);
    const double fan_in = double(l.taps) * (i == 0 ? (c->nloc + 1) : l.cin);
    const double sd = (i == 8 ? 0.1 : 1.0) * std::sqrt(2.0 / fan_in);
    for (long long e = 0; e < l.nw; ++e) {
      const double u1 = u01(st), u2 = u01(st);
      w[e] = float(sd * std::sqrt(-2.0 * std::log(u1)) * std::cos(6.283185307179586 * u2));
    }
    if (i == 0)  // padded input channels carry no weight
      for (int co = 0; co < l.cout; ++co)
        for (int ci = c->nloc + 1; ci < l.cin; ++ci) w[(long long)co * l.cin + ci] = 0.f;
    if (i == 8)  // padded output channels carry no weight
      for (int co = c->nloc; co < l.cout; ++co)
        for (int ci = 0; ci < l.cin; ++ci) w[(long long)co * l.cin + ci] = 0.f;
    cudaError_t e = cudaMemcpy(l.w, w.data(), l.nw * 4, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemset(l.m, 0, l.nw * 4);
    if (e == cudaSuccess) e = cudaMemset(l.v, 0, l.nw * 4);
    if (e == cudaSuccess) e = cudaMemset(l.g, 0, l.nw * 4);
    if (e != cudaSuccess) rc = set_cuda_error(e, "gbfem_cnn_create: init");
  }
  if (rc == GBFEM_OK) {
    cudaError_t e = cudaMemset(c->status, 0, sizeof(int));
    if (e != cudaSuccess) rc = set_cuda_error(e, "gbfem_cnn_create");
  }
  // tensor maps of the 3x3x3 convolutions' inputs (forward, backward-data)
  {
    const bf16* in[] = {c->a0, c->p1, c->p2, c->p3, c->u3, c->u2, c->u1, c->G[0][0], c->G[1][0], c->G[2][0], c->G[3][0]};
    const int lv[] = {0, 1, 2, 3, 2, 1, 0, 0, 1, 2, 3};
    for (int k = 0; k < 11 && rc == GBFEM_OK; ++k) rc = conv_map(c, in[k], c->N[lv[k]]);
  }
  if (rc == GBFEM_OK) {
    logkappa_kernel<double><<<grid1(c->P[0]), 256>>>(nullptr, c->nloc, c->P[0], c->logk);
    rc = refresh_bf16(c, nullptr);
  }
  if (rc == GBFEM_OK) {
    cudaError_t e = cudaDeviceSynchronize();
    if (e != cudaSuccess) rc = set_cuda_error(e, "gbfem_cnn_create");
  }
  if (rc) { gbfem_cnn_destroy(c); return rc; }
  *out = c;
  return GBFEM_OK;
}

int gbfem_cnn_destroy(gbfem_cnn c) {
  if (!c) return GBFEM_OK;
  for (void* p : c->allocs) cudaFree(p);
  if (c->h_loss) cudaFreeHost(c->h_loss);
  delete c;
  return GBFEM_OK;
}

int gbfem_cnn_set_kappa(gbfem_cnn c, int precision, const void* kappa, void* stream) {
  if (!c) return set_error(GBFEM_ERR_INVALID, "gbfem_cnn_set_kappa: null cnn");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (precision == GBFEM_F64 || !kappa)
    logkappa_kernel<double><<<grid1(c->P[0]), 256, 0, s>>>(static_cast<const double*>(kappa), c->nloc, c->P[0], c->logk);
  else
    logkappa_kernel<float><<<grid1(c->P[0]), 256, 0, s>>>(static_cast<const float*>(kappa), c->nloc, c->P[0], c->logk);
  GBFEM_CUDA_TRY(cudaGetLastError());
  return GBFEM_OK;
}

int gbfem_cnn_set_conv_engine(gbfem_cnn c, int engine) {
  if (!c || (engine != GBFEM_CNN_CONV_TENSOR_CORE && engine != GBFEM_CNN_CONV_MMA_SYNC))
    return set_error(GBFEM_ERR_INVALID, "gbfem_cnn_set_conv_engine: invalid argument");
  c->conv_engine = engine;
  return GBFEM_OK;
}

int gbfem_cnn_status(gbfem_cnn c, int* status) {
  if (!c || !status) return set_error(GBFEM_ERR_INVALID, "gbfem_cnn_status: null argument");
  GBFEM_CUDA_TRY(cudaMemcpy(status, c->status, sizeof(int), cudaMemcpyDeviceToHost));
  return GBFEM_OK;
}

int gbfem_cnn_set_coarse(gbfem_cnn c, int coarse) {
  if (!c) return set_error(GBFEM_ERR_INVALID, "gbfem_cnn_set_coarse: null cnn");
  c->coarse = coarse ? 1 : 0;
  return GBFEM_OK;
}

int gbfem_cnn_set_output_scale(gbfem_cnn c, double scale) {
  if (!c || !(scale > 0)) return set_error(GBFEM_ERR_INVALID, "gbfem_cnn_set_output_scale: bad argument");
  c->S = float(scale);
  return GBFEM_OK;
}

int gbfem_cnn_get_output_scale(gbfem_cnn c, double* scale) {
  if (!c || !scale) return set_error(GBFEM_ERR_INVALID, "null argument");
  *scale = c->S;
  return GBFEM_OK;
}

int gbfem_cnn_forward(gbfem_cnn c, int precision, const void* r, void* z, int accumulate, void* stream) {
  if (!c || !r || !z) return set_error(GBFEM_ERR_INVALID, "gbfem_cnn_forward: null argument");
  return cnn_apply(c, precision, r, z, accumulate, static_cast<cudaStream_t>(stream));
}

int gbfem_cnn_loss_grad(gbfem_cnn c, int precision, const void* r, const void* target, double* loss, void* stream) {
  if (!c || !r || !target) return set_error(GBFEM_ERR_INVALID, "gbfem_cnn_loss_grad: null argument");
  return cnn_loss_grad(c, precision, r, target, loss, static_cast<cudaStream_t>(stream));
}

int gbfem_cnn_train_step(gbfem_cnn c, int precision, const void* r, const void* target, double lr, double* loss,
                         void* stream) {
  if (!c || !r || !target) return set_error(GBFEM_ERR_INVALID, "gbfem_cnn_train_step: null argument");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  GBFEM_TRY(cnn_loss_grad(c, precision, r, target, loss, s));
  c->adam_t += 1;
  const float b1 = 0.9f, b2 = 0.999f;
  const float c1 = float(1.0 / (1.0 - std::pow(double(b1), c->adam_t)));
  const float c2 = float(1.0 / (1.0 - std::pow(double(b2), c->adam_t)));
  for (int i = 0; i < NLAYER; ++i) {
    Layer& l = c->L[i];
    adam_kernel<<<grid1(l.nw), 256, 0, s>>>(l.w, l.g, l.m, l.v, l.nw, float(lr), b1, b2, 1e-8f, c1, c2);
  }
  GBFEM_CUDA_TRY(cudaGetLastError());
  return refresh_bf16(c, s);
}

int gbfem_cnn_train_step_grad(gbfem_cnn c, int precision, const void* r, const void* grad_z, double lr,
                              void* stream) {
  if (!c || !r || !grad_z) return set_error(GBFEM_ERR_INVALID, "gbfem_cnn_train_step_grad: null argument");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (precision == GBFEM_F64) GBFEM_TRY(cnn_input<double>(c, r, s));
  else GBFEM_TRY(cnn_input<float>(c, r, s));
  GBFEM_TRY(cnn_forward(c, s));
  const long long ny = c->P[0] * c->cout0;
  if (precision == GBFEM_F64)
    grad_from_dofs_kernel<double><<<grid1(ny), 256, 0, s>>>(static_cast<const double*>(grad_z), c->d_rr, cnn_nnorm(c),
                                                            c->nloc, c->cout0, c->P[0], c->S, c->coarse, c->dy);
  else
    grad_from_dofs_kernel<float><<<grid1(ny), 256, 0, s>>>(static_cast<const float*>(grad_z), c->d_rr, cnn_nnorm(c),
                                                           c->nloc, c->cout0, c->P[0], c->S, c->coarse, c->dy);
  GBFEM_CUDA_TRY(cudaGetLastError());
  GBFEM_TRY(cnn_backward(c, s));
  c->adam_t += 1;
  const float b1 = 0.9f, b2 = 0.999f;
  const float c1 = float(1.0 / (1.0 - std::pow(double(b1), c->adam_t)));
  const float c2 = float(1.0 / (1.0 - std::pow(double(b2), c->adam_t)));
  for (int i = 0; i < NLAYER; ++i) {
    Layer& l = c->L[i];
    adam_kernel<<<grid1(l.nw), 256, 0, s>>>(l.w, l.g, l.m, l.v, l.nw, float(lr), b1, b2, 1e-8f, c1, c2);
  }
  GBFEM_CUDA_TRY(cudaGetLastError());
  return refresh_bf16(c, s);
}

int gbfem_cnn_num_params(gbfem_cnn c, int64_t* n) {
  if (!c || !n) return set_error(GBFEM_ERR_INVALID, "null argument");
  long long t = 0;
  for (int i = 0; i < NLAYER; ++i) t += c->L[i].nw;
  *n = t;
  return GBFEM_OK;
}

// which = 0: weights, 1: gradients; host FP32 arrays in layer order, [taps][cout][cin]
static int cnn_copy_params(gbfem_cnn c, float* host, int which, bool to_device) {
  long long off = 0;
  for (int i = 0; i < NLAYER; ++i) {
    Layer& l = c->L[i];
    float* d = which == 0 ? l.w : l.g;
    cudaError_t e = to_device ? cudaMemcpy(d, host + off, l.nw * 4, cudaMemcpyHostToDevice)
                              : cudaMemcpy(host + off, d, l.nw * 4, cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return set_cuda_error(e, "gbfem_cnn params");
    off += l.nw;
  }
  if (to_device && which == 0) {
    GBFEM_TRY(refresh_bf16(c, nullptr));
    GBFEM_CUDA_TRY(cudaDeviceSynchronize());
  }
  return GBFEM_OK;
}

int gbfem_cnn_get_params(gbfem_cnn c, float* host) { return c && host ? cnn_copy_params(c, host, 0, false) : set_error(GBFEM_ERR_INVALID, "null"); }
int gbfem_cnn_set_params(gbfem_cnn c, const float* host) { return c && host ? cnn_copy_params(c, const_cast<float*>(host), 0, true) : set_error(GBFEM_ERR_INVALID, "null"); }
int gbfem_cnn_get_grads(gbfem_cnn c, float* host) { return c && host ? cnn_copy_params(c, host, 1, false) : set_error(GBFEM_ERR_INVALID, "null"); }

int gbfem_cnn_save(gbfem_cnn c, const char* path) {
  if (!c || !path) return set_error(GBFEM_ERR_INVALID, "gbfem_cnn_save: null argument");
  int64_t n;
  gbfem_cnn_num_params(c, &n);
  std::vector<float> w(n);
  GBFEM_TRY(cnn_copy_params(c, w.data(), 0, false));
  FILE* f = std::fopen(path, "wb");
  if (!f) return set_error(GBFEM_ERR_INVALID, std::string("gbfem_cnn_save: cannot open ") + path);
  const int32_t hdr[6] = {0x4742434E, 1, c->nloc, c->cin0, c->cout0, C};
  bool ok = std::fwrite(hdr, sizeof(hdr), 1, f) == 1 && std::fwrite(&c->S, sizeof(float), 1, f) == 1 &&
            std::fwrite(&n, sizeof(n), 1, f) == 1 && std::fwrite(w.data(), 4, n, f) == size_t(n);
  std::fclose(f);
  return ok ? GBFEM_OK : set_error(GBFEM_ERR_INVALID, "gbfem_cnn_save: write failed");
}

int gbfem_cnn_load(gbfem_cnn c, const char* path) {
  if (!c || !path) return set_error(GBFEM_ERR_INVALID, "gbfem_cnn_load: null argument");
  FILE* f = std::fopen(path, "rb");
  if (!f) return set_error(GBFEM_ERR_INVALID, std::string("gbfem_cnn_load: cannot open ") + path);
  int32_t hdr[6];
  float S = 0;
  int64_t n = 0, want;
  gbfem_cnn_num_params(c, &want);
  bool ok = std::fread(hdr, sizeof(hdr), 1, f) == 1 && std::fread(&S, sizeof(float), 1, f) == 1 &&
            std::fread(&n, sizeof(n), 1, f) == 1;
  ok = ok && hdr[0] == 0x4742434E && hdr[1] == 1 && hdr[2] == c->nloc && hdr[3] == c->cin0 && hdr[4] == c->cout0 &&
       hdr[5] == C && n == want && std::isfinite(S) && S > 0;
  std::vector<float> w(ok ? n : 0);
  if (ok) ok = std::fread(w.data(), 4, n, f) == size_t(n);
  std::fclose(f);
  if (ok)
    for (float x : w)
      if (!std::isfinite(x)) { ok = false; break; }
  if (!ok) return set_error(GBFEM_ERR_INVALID, std::string("gbfem_cnn_load: not a valid network file for this space: ") + path);
  c->S = S;
  return cnn_copy_params(c, w.data(), 0, true);
}

int gbfem_preconditioner_learned_create(gbfem_cnn c, gbfem_preconditioner bj, gbfem_operator op,
                                        gbfem_preconditioner* out) {
  if (!c || !out) return set_error(GBFEM_ERR_INVALID, "gbfem_preconditioner_learned_create: null argument");
  if (bj && bj->n != c->ndofs) return set_error(GBFEM_ERR_INVALID, "learned preconditioner: size mismatch");
  if (op && (!bj || op->ndofs != c->ndofs || op->precision != bj->precision))
    return set_error(GBFEM_ERR_INVALID, "learned preconditioner: the two-level form needs bj and a matching op");
  *out = nullptr;
  auto* pc = new (std::nothrow) gbfem_preconditioner_s();
  if (!pc) return set_error(GBFEM_ERR_INVALID, "out of host memory");
  pc->kind = PcKind::External;
  pc->precision = bj ? bj->precision : GBFEM_F64;
  pc->n = c->ndofs;
  pc->nloc = c->nloc;
  pc->owns_data = false;
  auto* lc = new (std::nothrow) LearnedCtx{c, bj, op};
  if (!lc) { delete pc; return set_error(GBFEM_ERR_INVALID, "out of host memory"); }
  if (op) {
    const size_t bytes = size_t(c->ndofs) * (bj->precision == GBFEM_F64 ? 8 : 4);
    cudaError_t e = cudaMalloc(&lc->t, bytes);
    if (e == cudaSuccess) e = cudaMalloc(&lc->at, bytes);
    if (e == cudaSuccess) e = cudaMalloc(&lc->dots, 2 * sizeof(double));
    if (e == cudaSuccess) e = cudaMalloc(&lc->partial, sizeof(double) * (dot_num_partials(c->ndofs) + 8));
    if (e != cudaSuccess) {
      delete lc;
      delete pc;
      return set_cuda_error(e, "learned preconditioner: work vectors");
    }
  }
  pc->ext_apply = ext_learned_apply;
  pc->ext_destroy = ext_learned_destroy;
  pc->ext_ctx = lc;
  pc->fallback = bj;
  *out = pc;
  return GBFEM_OK;
}

}  // extern "C"
