// Error reporting, device memory and version entry points of libgbfem.
#include <cuda_runtime.h>
#include <cstdio>
#include <string>

#include "gbfem_internal.cuh"

namespace gbfem {

static thread_local std::string g_last_error;

int set_error(int code, const std::string& msg) {
  g_last_error = msg;
  return code;
}

int set_cuda_error(cudaError_t err, const char* where) {
  if (err == cudaErrorNoDevice || err == cudaErrorInsufficientDriver)
    return set_error(GBFEM_ERR_NO_DEVICE, std::string("no CUDA device: ") + cudaGetErrorString(err));
  return set_error(GBFEM_ERR_CUDA, std::string(where) + ": " + cudaGetErrorString(err));
}

}  // namespace gbfem

extern "C" {

const char* gbfem_last_error(void) { return gbfem::g_last_error.c_str(); }

int gbfem_version(void) { return 100; }

int gbfem_malloc(void** ptr, size_t bytes) {
  if (!ptr) return gbfem::set_error(GBFEM_ERR_INVALID, "gbfem_malloc: null ptr");
  *ptr = nullptr;
  if (bytes == 0) return GBFEM_OK;
  GBFEM_CUDA_TRY(cudaMalloc(ptr, bytes));
  return GBFEM_OK;
}

int gbfem_free(void* ptr) {
  if (ptr) GBFEM_CUDA_TRY(cudaFree(ptr));
  return GBFEM_OK;
}

int gbfem_memcpy_h2d(void* dst, const void* src, size_t bytes) {
  if (bytes) GBFEM_CUDA_TRY(cudaMemcpy(dst, src, bytes, cudaMemcpyHostToDevice));
  return GBFEM_OK;
}

int gbfem_memcpy_d2h(void* dst, const void* src, size_t bytes) {
  if (bytes) GBFEM_CUDA_TRY(cudaMemcpy(dst, src, bytes, cudaMemcpyDeviceToHost));
  return GBFEM_OK;
}

int gbfem_memset(void* ptr, int value, size_t bytes) {
  if (bytes) GBFEM_CUDA_TRY(cudaMemset(ptr, value, bytes));
  return GBFEM_OK;
}

int gbfem_synchronize(void) {
  GBFEM_CUDA_TRY(cudaDeviceSynchronize());
  return GBFEM_OK;
}

}  // extern "C"
