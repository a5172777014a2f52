// Allocation-free variant of the deterministic dot product.
//
// Some callers cannot let the library call cudaMalloc: a solver host that
// hands all of HBM to its own memory pool at start-up (a library cudaMalloc
// then fails or fragments the pool), or a latency-critical loop that cannot
// afford the device synchronisation cudaMalloc may imply.  gbfem_dot keeps
// its partial sums in scratch the library allocates on first use; this
// entry point keeps them in a fixed array in the library's own device
// memory instead, so it never allocates.
//
// The scratch is a file-scope __device__ array: every GPU that loads
// libgbfem holds it (kNoAllocScratchDoubles doubles, about 512 KB) until the
// process exits.  In host code the array's name is only a host-side
// stand-in, so its device address is looked up once per device with
// cudaGetSymbolAddress and that address is what the kernels receive.
#include <cuda_runtime.h>
#include <mutex>

#include "blas.cuh"
#include "gbfem_internal.cuh"

namespace gbfem {

// One partial sum per chunk of at most 8192 elements: np = ceil(n / 8192)
// partials of ceil(n / np) elements each.  Up to 1024 partials this is
// exactly gbfem_dot's partition (dot_num_partials), so for n <= 1024 * 8192
// the two entry points return bitwise the same sum; beyond that gbfem_dot
// stops at 1024 longer chunks and this one keeps chunks of <= 8192.  At most
// 65536 partials, so n <= 65536 * 8192 = 536,870,912 elements.
constexpr long long kNoAllocChunk = 8192;
constexpr long long kNoAllocMaxPartials = 65536;
constexpr long long kNoAllocMaxN = kNoAllocChunk * kNoAllocMaxPartials;
// partials, then one result slot (padded to a 256-byte line)
constexpr long long kNoAllocScratchDoubles = kNoAllocMaxPartials + 32;

static __device__ __align__(256) double g_dot_noalloc_scratch[kNoAllocScratchDoubles];

constexpr int kMaxDevices = 64;
static std::mutex g_noalloc_mu;
static double* g_noalloc_ptr[kMaxDevices] = {};

// Device address of the scratch array on the current device, looked up
// once per device (with that device current).  The cached address belongs to
// the device's current context: after cudaDeviceReset the library's module is
// loaded again and the address must not be reused, so callers that reset a
// device must not call this entry point afterwards in the same process.
static int noalloc_scratch(double** out) {
  int dev = 0;
  GBFEM_CUDA_TRY(cudaGetDevice(&dev));
  if (dev < 0 || dev >= kMaxDevices) return set_error(GBFEM_ERR_INVALID, "gbfem_dot_noalloc: device index too large");
  std::lock_guard<std::mutex> lk(g_noalloc_mu);
  if (!g_noalloc_ptr[dev]) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_dot_noalloc_scratch);
    if (e != cudaSuccess) return set_cuda_error(e, "gbfem_dot_noalloc: cudaGetSymbolAddress");
    g_noalloc_ptr[dev] = static_cast<double*>(p);
  }
  *out = g_noalloc_ptr[dev];
  return GBFEM_OK;
}

}  // namespace gbfem

using namespace gbfem;

extern "C" int gbfem_dot_noalloc(int precision, int64_t n, const void* x, const void* y, double* result,
                                 void* stream) {
  if (!result || (n > 0 && (!x || !y))) return set_error(GBFEM_ERR_INVALID, "gbfem_dot_noalloc: null argument");
  if (precision != GBFEM_F64 && precision != GBFEM_F32)
    return set_error(GBFEM_ERR_INVALID, "gbfem_dot_noalloc: precision must be GBFEM_F64 or GBFEM_F32");
  if (n > kNoAllocMaxN)
    return set_error(GBFEM_ERR_INVALID, "gbfem_dot_noalloc: n = " + std::to_string((long long)n) +
                                            " exceeds the maximum of " + std::to_string(kNoAllocMaxN) +
                                            " elements (fixed scratch of 65536 partial sums)");
  if (n <= 0) {
    *result = 0.0;
    return GBFEM_OK;
  }
  double* scratch = nullptr;
  GBFEM_TRY(noalloc_scratch(&scratch));
  double* partial = scratch;
  double* res = scratch + kNoAllocMaxPartials;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  // Pass 1 overwrites every partial it uses and pass 2 overwrites the result
  // slot, so nothing left by an earlier call needs clearing.
  const long long np = (n + kNoAllocChunk - 1) / kNoAllocChunk;
  const long long chunk = (n + np - 1) / np;
  GBFEM_TRY(dot_device_fixed_chunks(precision, n, chunk, x, y, res, partial, s));
  GBFEM_CUDA_TRY(cudaMemcpyAsync(result, res, sizeof(double), cudaMemcpyDeviceToHost, s));
  GBFEM_CUDA_TRY(cudaStreamSynchronize(s));
  return GBFEM_OK;
}
