// Launch wrappers for the device kernels (implemented in the .cu files).
#pragma once
#include <cuda_runtime.h>
#include <stddef.h>

#include <algorithm>

namespace a2ds {
int launch_axpy(double *y, double alpha, const double *x, size_t n, cudaStream_t s);
int launch_spmv_f64(int nrows, const int *rowp, const int *cols, const double *vals,
                    const double *x, double *y, cudaStream_t s);
}  // namespace a2ds
