// FMA-throughput microbenchmark for the FP64 and FP32 pipes (built into
// lib/libgbfem_bench.so for bench.py; not part of the library's C-ABI).
//
// The roofline of the matrix-free operator apply needs the arithmetic peak of
// the pipe it runs on, and the HBM copy peak alone does not give it.  Each
// thread runs CHAINS independent FMA chains for `iters` iterations, so the
// pipe, not the dependency latency, limits the rate.  The result is written
// to `out` so the compiler cannot remove the chains.  Returns 0, or the CUDA
// error code.
#include <cuda_runtime.h>

#define PEAK_TRY(expr)                          \
  do {                                          \
    cudaError_t _e = (expr);                    \
    if (_e != cudaSuccess) return int(_e);      \
  } while (0)

namespace gbfem_bench {

template <typename T, int CHAINS>
__global__ void fma_chain_kernel(T* out, int iters, T a, T b) {
  T acc[CHAINS];
#pragma unroll
  for (int c = 0; c < CHAINS; ++c) acc[c] = T(threadIdx.x + c);
  for (int it = 0; it < iters; ++it) {
#pragma unroll
    for (int c = 0; c < CHAINS; ++c) acc[c] = fma(acc[c], a, b);
  }
  T s = 0;
#pragma unroll
  for (int c = 0; c < CHAINS; ++c) s += acc[c];
  out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

template <typename T>
static int run_peak(int sm_count, double* tflops) {
  const int threads = 256, blocks_per_sm = 8, chains = 8;
  const int blocks = sm_count * blocks_per_sm;
  const int iters = sizeof(T) == 8 ? 1024 : 16384;
  T* out = nullptr;
  PEAK_TRY(cudaMalloc(&out, sizeof(T) * blocks * threads));
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  // warm-up
  fma_chain_kernel<T, chains><<<blocks, threads>>>(out, iters / 8, T(0.999999), T(1e-7));
  cudaEventRecord(e0);
  const int reps = 3;
  for (int r = 0; r < reps; ++r)
    fma_chain_kernel<T, chains><<<blocks, threads>>>(out, iters, T(0.999999), T(1e-7));
  cudaEventRecord(e1);
  cudaError_t err = cudaEventSynchronize(e1);
  float ms = 0.f;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(out);
  if (err != cudaSuccess) return int(err);
  const double fmas = double(reps) * blocks * threads * double(iters) * chains;
  *tflops = 2.0 * fmas / (ms * 1e-3) / 1e12;
  return 0;
}

}  // namespace gbfem_bench

extern "C" int gbfem_bench_fma_peaks(double* fp64_tflops, double* fp32_tflops) {
  using namespace gbfem_bench;
  int dev = 0, sms = 0;
  PEAK_TRY(cudaGetDevice(&dev));
  PEAK_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  int rc = run_peak<double>(sms, fp64_tflops);
  if (rc) return rc;
  return run_peak<float>(sms, fp32_tflops);
}
