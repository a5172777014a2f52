// Device-side BLAS-1 helpers shared by the solvers.
#pragma once
#include <cuda_runtime.h>

#include "convert.cuh"

namespace gbfem {

// Number of FP64 partial sums pass 1 of a dot product of length n writes.
// Pass 1 runs dot_num_partials(n) CTAs of kRedThreads threads; CTA b sums the
// chunk [b c, min(n, (b+1) c)), c = ceil(n / partials), thread t the elements
// b c + t + k kRedThreads in order, then block_sum.  Kernels that fuse a dot
// product into other work reproduce exactly this order (bitwise the same sum).
int dot_num_partials(long long n);
constexpr int kRedThreads = 256;

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  return v;
}

// A thread's share of a dot product, sum of x_i y_i in its fixed order.
// FP64 vectors: FP64 fma.  FP32 vectors: each product is formed exactly as
// p + e (p = x y rounded, e = fma(x, y, -p)) and the terms are summed in
// float-float (Knuth's two-sum for p, the errors and e into a second float),
// all on the FP32 pipe -- an FP64 product per element would bind on this
// GPU's narrow FP64 pipe -- and widened to FP64 once per thread.  The sum
// carries about 48 significant bits per thread share; the products keep
// the FP32 exponent range.
template <typename T> struct DotAcc;
template <> struct DotAcc<double> {
  double s = 0.0;
  __device__ __forceinline__ void add(double a, double b) { s = fma(a, b, s); }
  __device__ __forceinline__ double value() const { return s; }
};
template <> struct DotAcc<float> {
  float s = 0.f, c = 0.f;
  __device__ __forceinline__ void add(float a, float b) {
    const float p = a * b;
    const float e = fmaf(a, b, -p);
    const float t = s + p;
    const float bp = t - s;
    c += ((s - (t - bp)) + (p - bp)) + e;
    s = t;
  }
  __device__ __forceinline__ double value() const { return f32_to_f64(s) + f32_to_f64(c); }
};

// Fixed-shape block reduction of one value per thread (kRedThreads threads);
// the result is valid in thread 0.
__device__ __forceinline__ double block_sum(double v) {
  __shared__ double red[kRedThreads / 32];
  v = warp_sum(v);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (lane == 0) red[wid] = v;
  __syncthreads();
  double r = 0.0;
  if (wid == 0) {
    r = lane < kRedThreads / 32 ? red[lane] : 0.0;
    r = warp_sum(r);
  }
  __syncthreads();
  return r;
}

// Pass 2 of a dot product, as a device function for kernels that continue
// with the result: every thread of the (single, kRedThreads-thread) CTA
// calls it; the sum is valid in thread 0.
__device__ __forceinline__ double dot_final_sum(const double* __restrict__ partial, int np) {
  double s = 0.0;
  for (int i = threadIdx.x; i < np; i += kRedThreads) s += partial[i];
  return block_sum(s);
}

// Pass 1 only (partials into d_partial); returns through *np the count.
int dot_partial_device(int precision, long long n, const void* x, const void* y, double* d_partial, int* np,
                       cudaStream_t s);
// d_out[0] = x . y (FP64 accumulate), asynchronously on stream s.
// d_partial must hold dot_num_partials(n) doubles.
int dot_device(int precision, long long n, const void* x, const void* y, double* d_out, double* d_partial,
               cudaStream_t s);
// Dot product over fixed chunks of `chunk` elements on caller-provided
// scratch (ceil(n/chunk) partials).
int dot_device_fixed_chunks(int precision, long long n, long long chunk, const void* x, const void* y,
                            double* d_out, double* d_partial, cudaStream_t s);
// Up to kMaxDotPairs dot products x_l . y_l in one pass 1 (a 2-D grid:
// chunks x pairs) and one pass 2, each with exactly gbfem_dot's partition and
// summation order, so every result is bitwise the single dot's.  d_partial
// must hold k * dot_num_partials(n) doubles, d_out k doubles.
constexpr int kMaxDotPairs = 32;
int multi_dot_device(int precision, long long n, int k, const void* const* xs, const void* const* ys, double* d_out,
                     double* d_partial, cudaStream_t s);
// y = y + sum_l a_l x_l (l = 0..k-1 in order, k <= kMaxDotPairs), one pass.
int multi_axpy_device(int precision, long long n, int k, const double* a, const void* const* xs, void* y,
                      cudaStream_t s);
// The library's per-device scratch (allocated on first use).
int library_scratch(double** partial, double** result);
// Grid size of the grid-stride streaming kernels.
int stream_grid(long long n);

}  // namespace gbfem
