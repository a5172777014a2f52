// Internal helpers shared by the translation units of libgbfem:
// error reporting (status codes + a thread-local message, the C-ABI's
// replacement for DUNE_THROW) and small device utilities.
#pragma once
#include <cuda_runtime.h>
#include <cstddef>
#include <cstdint>
#include <string>

#include "../../include/gbfem.h"

namespace gbfem {

// Records `msg` as the calling thread's last error and returns `code`.
int set_error(int code, const std::string& msg);
// Records a CUDA runtime error and returns GBFEM_ERR_CUDA.
int set_cuda_error(cudaError_t err, const char* where);

}  // namespace gbfem

#define GBFEM_CUDA_TRY(expr)                                      \
  do {                                                            \
    cudaError_t _e = (expr);                                      \
    if (_e != cudaSuccess) return ::gbfem::set_cuda_error(_e, #expr); \
  } while (0)

#define GBFEM_TRY(expr)            \
  do {                             \
    int _rc = (expr);              \
    if (_rc != 0) return _rc;      \
  } while (0)
