// BLAS-1 on dof vectors: the operations of DiscreteFunctionDefault used by
// the Krylov loops (function/common/discretefunction.hh:781-901) and the
// scalar product of function/common/scalarproducts.hh:101-127.
//
// The reference sums dot products sequentially.  Here a dot product is a
// two-pass tree: pass 1 gives one FP64 partial per chunk of the vector, pass 2
// reduces the partials in one CTA.  The chunking depends only on n, so the
// result is bitwise reproducible, independent of device and stream.  FP32
// vectors are accumulated in FP64: the convergence dot products stay FP64 in
// the mixed-precision solver.
#include <cuda_runtime.h>
#include <mutex>
#include <vector>

#include "blas.cuh"
#include "gbfem_internal.cuh"

namespace gbfem {

constexpr int kMaxPartials = 1024;

int dot_num_partials(long long n) {
  long long p = (n + 8191) / 8192;
  if (p < 1) p = 1;
  if (p > kMaxPartials) p = kMaxPartials;
  return int(p);
}

template <typename T>
__global__ void __launch_bounds__(kRedThreads) dot_partial_kernel(const T* __restrict__ x, const T* __restrict__ y,
                                                                  long long n, long long chunk, double* partial) {
  const long long b0 = (long long)blockIdx.x * chunk;
  long long b1 = b0 + chunk;
  if (b1 > n) b1 = n;
  DotAcc<T> acc;
  for (long long i = b0 + threadIdx.x; i < b1; i += kRedThreads) acc.add(x[i], y[i]);
  const double s = block_sum(acc.value());
  if (threadIdx.x == 0) partial[blockIdx.x] = s;
}

__global__ void __launch_bounds__(kRedThreads) dot_final_kernel(const double* __restrict__ partial, int np,
                                                                double* out) {
  const double s = dot_final_sum(partial, np);
  if (threadIdx.x == 0) *out = s;
}

// Per-device scratch of the library's own reductions.
struct Scratch {
  double* partial = nullptr;  // kMaxPartials partial sums
  double* result = nullptr;   // 64 result slots
};
static std::mutex g_scratch_mu;
static std::vector<Scratch> g_scratch;

int library_scratch(double** partial, double** result) {
  int dev = 0;
  GBFEM_CUDA_TRY(cudaGetDevice(&dev));
  std::lock_guard<std::mutex> lk(g_scratch_mu);
  if (int(g_scratch.size()) <= dev) g_scratch.resize(dev + 1);
  Scratch& s = g_scratch[dev];
  if (!s.partial) {
    GBFEM_CUDA_TRY(cudaMalloc(&s.partial, sizeof(double) * kMaxPartials));
    GBFEM_CUDA_TRY(cudaMalloc(&s.result, sizeof(double) * 64));
  }
  *partial = s.partial;
  if (result) *result = s.result;
  return GBFEM_OK;
}

int dot_partial_device(int precision, long long n, const void* x, const void* y, double* d_partial, int* npo,
                       cudaStream_t s) {
  const int np = dot_num_partials(n);
  const long long chunk = (n + np - 1) / np;
  if (precision == GBFEM_F64)
    dot_partial_kernel<double><<<np, kRedThreads, 0, s>>>(static_cast<const double*>(x),
                                                         static_cast<const double*>(y), n, chunk, d_partial);
  else
    dot_partial_kernel<float><<<np, kRedThreads, 0, s>>>(static_cast<const float*>(x),
                                                        static_cast<const float*>(y), n, chunk, d_partial);
  GBFEM_CUDA_TRY(cudaGetLastError());
  *npo = np;
  return GBFEM_OK;
}

struct DotPairs {
  const void* x[kMaxDotPairs];
  const void* y[kMaxDotPairs];
};

// dot_partial_kernel for pair blockIdx.y: the same chunk, thread order and
// block reduction, so partial[l np + b] is bitwise the single dot's partial b
template <typename T>
__global__ void __launch_bounds__(kRedThreads) multi_dot_partial_kernel(const __grid_constant__ DotPairs pr, long long n,
                                                                        long long chunk, int np, double* partial) {
  const T* __restrict__ x = static_cast<const T*>(pr.x[blockIdx.y]);
  const T* __restrict__ y = static_cast<const T*>(pr.y[blockIdx.y]);
  const long long b0 = (long long)blockIdx.x * chunk;
  long long b1 = b0 + chunk;
  if (b1 > n) b1 = n;
  DotAcc<T> acc;
  for (long long i = b0 + threadIdx.x; i < b1; i += kRedThreads) acc.add(x[i], y[i]);
  const double s = block_sum(acc.value());
  if (threadIdx.x == 0) partial[(long long)blockIdx.y * np + blockIdx.x] = s;
}

__global__ void __launch_bounds__(kRedThreads) multi_dot_final_kernel(const double* __restrict__ partial, int np,
                                                                      double* out) {
  const double s = dot_final_sum(partial + (long long)blockIdx.x * np, np);
  if (threadIdx.x == 0) out[blockIdx.x] = s;
}

struct AxpyTerms {
  double a[kMaxDotPairs];
  const void* x[kMaxDotPairs];
};

// y = a_0 x_0 + 1 y, then a_1 x_1 + 1 y, ...: the arithmetic of k
// successive y = a x + b y updates with b = 1, in one pass over y
template <typename T>
__global__ void multi_axpy_kernel(long long n, int k, const __grid_constant__ AxpyTerms t, T* __restrict__ y) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    T acc = y[i];
    for (int l = 0; l < k; ++l) acc = T(t.a[l]) * static_cast<const T*>(t.x[l])[i] + T(1.0) * acc;
    y[i] = acc;
  }
}

int multi_dot_device(int precision, long long n, int k, const void* const* xs, const void* const* ys, double* d_out,
                     double* d_partial, cudaStream_t s) {
  if (k <= 0) return GBFEM_OK;
  if (k > kMaxDotPairs) return set_error(GBFEM_ERR_INVALID, "multi_dot: too many pairs");
  const int np = dot_num_partials(n);
  const long long chunk = (n + np - 1) / np;
  DotPairs pr{};
  for (int l = 0; l < k; ++l) {
    pr.x[l] = xs[l];
    pr.y[l] = ys[l];
  }
  const dim3 grid{unsigned(np), unsigned(k), 1u};
  if (precision == GBFEM_F64)
    multi_dot_partial_kernel<double><<<grid, kRedThreads, 0, s>>>(pr, n, chunk, np, d_partial);
  else
    multi_dot_partial_kernel<float><<<grid, kRedThreads, 0, s>>>(pr, n, chunk, np, d_partial);
  multi_dot_final_kernel<<<unsigned(k), kRedThreads, 0, s>>>(d_partial, np, d_out);
  GBFEM_CUDA_TRY(cudaGetLastError());
  return GBFEM_OK;
}

int multi_axpy_device(int precision, long long n, int k, const double* a, const void* const* xs, void* y,
                      cudaStream_t s) {
  if (k <= 0) return GBFEM_OK;
  if (k > kMaxDotPairs) return set_error(GBFEM_ERR_INVALID, "multi_axpy: too many terms");
  AxpyTerms t{};
  for (int l = 0; l < k; ++l) {
    t.a[l] = a[l];
    t.x[l] = xs[l];
  }
  if (precision == GBFEM_F64)
    multi_axpy_kernel<double><<<stream_grid(n), 256, 0, s>>>(n, k, t, static_cast<double*>(y));
  else
    multi_axpy_kernel<float><<<stream_grid(n), 256, 0, s>>>(n, k, t, static_cast<float*>(y));
  GBFEM_CUDA_TRY(cudaGetLastError());
  return GBFEM_OK;
}

int dot_device(int precision, long long n, const void* x, const void* y, double* d_out, double* d_partial,
               cudaStream_t s) {
  const int np = dot_num_partials(n);
  const long long chunk = (n + np - 1) / np;
  if (precision == GBFEM_F64)
    dot_partial_kernel<double><<<np, kRedThreads, 0, s>>>(static_cast<const double*>(x),
                                                         static_cast<const double*>(y), n, chunk, d_partial);
  else
    dot_partial_kernel<float><<<np, kRedThreads, 0, s>>>(static_cast<const float*>(x),
                                                        static_cast<const float*>(y), n, chunk, d_partial);
  dot_final_kernel<<<1, kRedThreads, 0, s>>>(d_partial, np, d_out);
  GBFEM_CUDA_TRY(cudaGetLastError());
  return GBFEM_OK;
}

template <typename T>
__global__ void axpy_kernel(long long n, T alpha, const T* __restrict__ x, T* __restrict__ y) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    y[i] = fma(alpha, x[i], y[i]);
}
template <typename T>
__global__ void scal_kernel(long long n, T alpha, T* __restrict__ x) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    x[i] *= alpha;
}
template <typename TX, typename TY>
__global__ void convert_kernel(long long n, const TX* __restrict__ x, TY* __restrict__ y) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    y[i] = TY(x[i]);
}

int stream_grid(long long n) {
  long long b = (n + 255) / 256;
  const long long cap = 152LL * 16;  // a few waves on the 152-SM part; loops cover the rest
  if (b > cap) b = cap;
  if (b < 1) b = 1;
  return int(b);
}

}  // namespace gbfem

using namespace gbfem;

extern "C" {

int gbfem_dot(int precision, int64_t n, const void* x, const void* y, double* result, void* stream) {
  if (!result || (n > 0 && (!x || !y))) return set_error(GBFEM_ERR_INVALID, "gbfem_dot: null argument");
  if (n <= 0) { *result = 0.0; return GBFEM_OK; }
  double *partial, *res;
  GBFEM_TRY(library_scratch(&partial, &res));
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  GBFEM_TRY(dot_device(precision, n, x, y, res, partial, s));
  GBFEM_CUDA_TRY(cudaMemcpyAsync(result, res, sizeof(double), cudaMemcpyDeviceToHost, s));
  GBFEM_CUDA_TRY(cudaStreamSynchronize(s));
  return GBFEM_OK;
}

int gbfem_axpy(int precision, int64_t n, double alpha, const void* x, void* y, void* stream) {
  if (n <= 0) return GBFEM_OK;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (precision == GBFEM_F64)
    axpy_kernel<double><<<stream_grid(n), 256, 0, s>>>(n, alpha, static_cast<const double*>(x), static_cast<double*>(y));
  else
    axpy_kernel<float><<<stream_grid(n), 256, 0, s>>>(n, float(alpha), static_cast<const float*>(x), static_cast<float*>(y));
  GBFEM_CUDA_TRY(cudaGetLastError());
  return GBFEM_OK;
}

int gbfem_scal(int precision, int64_t n, double alpha, void* x, void* stream) {
  if (n <= 0) return GBFEM_OK;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (precision == GBFEM_F64)
    scal_kernel<double><<<stream_grid(n), 256, 0, s>>>(n, alpha, static_cast<double*>(x));
  else
    scal_kernel<float><<<stream_grid(n), 256, 0, s>>>(n, float(alpha), static_cast<float*>(x));
  GBFEM_CUDA_TRY(cudaGetLastError());
  return GBFEM_OK;
}

int gbfem_copy(int precision, int64_t n, const void* x, void* y, void* stream) {
  if (n <= 0) return GBFEM_OK;
  const size_t bytes = size_t(n) * (precision == GBFEM_F64 ? 8 : 4);
  GBFEM_CUDA_TRY(cudaMemcpyAsync(y, x, bytes, cudaMemcpyDeviceToDevice, static_cast<cudaStream_t>(stream)));
  return GBFEM_OK;
}

int gbfem_convert(int64_t n, int px, const void* x, int py, void* y, void* stream) {
  if (n <= 0) return GBFEM_OK;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (px == py) return gbfem_copy(px, n, x, y, stream);
  if (px == GBFEM_F64)
    convert_kernel<double, float><<<stream_grid(n), 256, 0, s>>>(n, static_cast<const double*>(x), static_cast<float*>(y));
  else
    convert_kernel<float, double><<<stream_grid(n), 256, 0, s>>>(n, static_cast<const float*>(x), static_cast<double*>(y));
  GBFEM_CUDA_TRY(cudaGetLastError());
  return GBFEM_OK;
}

}  // extern "C"

namespace gbfem {

// Dot product over chunks of `chunk` elements (one partial each), launched
// on caller-provided scratch.  Used by the allocation-free entry point, which
// passes gbfem_dot's chunk wherever gbfem_dot's partition has <= 1024 chunks.
int dot_device_fixed_chunks(int precision, long long n, long long chunk, const void* x, const void* y,
                            double* d_out, double* d_partial, cudaStream_t s) {
  const long long np = (n + chunk - 1) / chunk;
  if (precision == GBFEM_F64)
    dot_partial_kernel<double><<<unsigned(np), kRedThreads, 0, s>>>(static_cast<const double*>(x),
                                                                   static_cast<const double*>(y), n, chunk, d_partial);
  else
    dot_partial_kernel<float><<<unsigned(np), kRedThreads, 0, s>>>(static_cast<const float*>(x),
                                                                  static_cast<const float*>(y), n, chunk, d_partial);
  dot_final_kernel<<<1, kRedThreads, 0, s>>>(d_partial, int(np), d_out);
  GBFEM_CUDA_TRY(cudaGetLastError());
  return GBFEM_OK;
}

}  // namespace gbfem
