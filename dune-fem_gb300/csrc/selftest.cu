// Device self-tests of helpers that restate hardware behaviour.
#include <cuda_runtime.h>
#include <cstdint>

#include "convert.cuh"
#include "gbfem_internal.cuh"

namespace gbfem {
namespace {

__device__ __forceinline__ uint64_t splitmix(uint64_t& s) {
  uint64_t z = (s += 0x9E3779B97F4A7C15ull);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

// every thread draws bit patterns (uniform bits, and values near the
// binary32 range limits and rounding ties) and compares the integer
// conversions with the hardware's
__global__ void k_conversions(uint64_t n, uint64_t seed, unsigned long long* mismatches) {
  unsigned long long bad = 0;
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
    uint64_t s = seed ^ (i * 0x2545F4914F6CDD1Dull);
    const uint64_t r = splitmix(s);
    uint64_t bits;
    switch (i & 3) {
      case 0: bits = r; break;  // any pattern
      case 1: bits = (r & 0x800FFFFFFFFFFFFFull) | (uint64_t(874 + (splitmix(s) % 300)) << 52); break;  // near f32 limits
      case 2: bits = (r & 0x800FFFFFE0000000ull) | (uint64_t(1023 - 20 + (splitmix(s) % 40)) << 52) |
                     (splitmix(s) & 1 ? 0x10000000ull : 0ull);  // ties and near-ties
              break;
      default: bits = (r & 0x800FFFFFFFFFFFFFull) | (uint64_t(splitmix(s) % 2047) << 52); break;
    }
    const double d = __longlong_as_double(static_cast<long long>(bits));
    const float a = f64_to_f32_rn(d), b = __double2float_rn(d);
    if (!((a != a && b != b) || __float_as_uint(a) == __float_as_uint(b))) ++bad;
    const float f = __uint_as_float(uint32_t(r >> 32));
    const double x = f32_to_f64(f), y = double(f);
    if (!((x != x && y != y) || __double_as_longlong(x) == __double_as_longlong(y))) ++bad;
  }
  if (bad) atomicAdd(mismatches, bad);
}

}  // namespace
}  // namespace gbfem

using namespace gbfem;

extern "C" int gbfem_selftest_conversions(uint64_t n, uint64_t seed, uint64_t* mismatches) {
  if (!mismatches) return set_error(GBFEM_ERR_INVALID, "gbfem_selftest_conversions: null argument");
  unsigned long long* d = nullptr;
  GBFEM_CUDA_TRY(cudaMalloc(&d, sizeof(unsigned long long)));
  cudaError_t e = cudaMemset(d, 0, sizeof(unsigned long long));
  if (e == cudaSuccess) {
    k_conversions<<<152 * 8, 256>>>(n, seed, d);
    e = cudaGetLastError();
  }
  unsigned long long h = 0;
  if (e == cudaSuccess) e = cudaMemcpy(&h, d, sizeof(h), cudaMemcpyDeviceToHost);
  cudaFree(d);
  if (e != cudaSuccess) return set_cuda_error(e, "gbfem_selftest_conversions");
  *mismatches = h;
  return GBFEM_OK;
}
