// Device-side BLAS-1 helpers shared by the solvers.
#pragma once
#include <cuda_runtime.h>

namespace gbfem {

// Number of FP64 partial sums pass 1 of a dot product of length n writes.
int dot_num_partials(long long n);
// d_out[0] = x . y (FP64 accumulate), asynchronously on stream s.
// d_partial must hold dot_num_partials(n) doubles.
int dot_device(int precision, long long n, const void* x, const void* y, double* d_out, double* d_partial,
               cudaStream_t s);
// Dot product over fixed chunks of `chunk` elements on caller-provided
// scratch (ceil(n/chunk) partials).
int dot_device_fixed_chunks(int precision, long long n, long long chunk, const void* x, const void* y,
                            double* d_out, double* d_partial, cudaStream_t s);
// The library's per-device scratch (allocated on first use).
int library_scratch(double** partial, double** result);
// Grid size of the grid-stride streaming kernels.
int stream_grid(long long n);

}  // namespace gbfem
