// 6x6-block CSR kernels: row-only Dirichlet treatment, value copy/axpy and
// the block SpMV in FP64 and FP32.
//
// Reference counterparts: BCSRMat::zeroRow (src/bpmat/BCSRMat.cpp:2005),
// BCSRMat::copyValues/axpy (:2375, :2430), BCSRMatVecMult6
// (src/bpmat/BCSRMatMult6.cpp:82).
#include "a2ds_internal.h"
#include "kernels.h"

namespace a2ds {

// One thread per (BC entry, block of its row, block row index ii): zero the
// masked rows of every block in the row, identity on the diagonal block.
__global__ void k_apply_bc_rows(double *vals, const int *rowp, const int *cols,
                                const int *bc_rows, const int *bc_masks, int nbc) {
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  int b = t / 6, ii = t % 6;
  if (b >= nbc) return;
  const int row = bc_rows[b], mask = bc_masks[b];
  if (!(mask & (1 << ii))) return;
  for (int jp = rowp[row]; jp < rowp[row + 1]; jp++) {
    double *a = vals + (size_t)jp * 36 + ii * 6;
#pragma unroll
    for (int jj = 0; jj < 6; jj++) a[jj] = 0.0;
    if (cols[jp] == row) a[ii] = 1.0;
  }
}

int launch_apply_bc_rows(double *vals, const int *rowp, const int *cols, const int *bc_rows,
                         const int *bc_masks, int nbc, cudaStream_t s) {
  if (nbc <= 0) return 0;
  int n = 6 * nbc;
  k_apply_bc_rows<<<(n + 255) / 256, 256, 0, s>>>(vals, rowp, cols, bc_rows, bc_masks, nbc);
  A2DS_CUDA_TRY(cudaGetLastError());
  return 0;
}

__global__ void k_axpy(double *y, double alpha, const double *x, size_t n) {
  size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  size_t stride = (size_t)gridDim.x * blockDim.x;
  for (; i < n; i += stride) y[i] += alpha * x[i];
}

int launch_axpy(double *y, double alpha, const double *x, size_t n, cudaStream_t s) {
  if (!n) return 0;
  int blocks = (int)std::min<size_t>((n + 255) / 256, 152 * 16);
  k_axpy<<<blocks, 256, 0, s>>>(y, alpha, x, n);
  A2DS_CUDA_TRY(cudaGetLastError());
  return 0;
}

// y = A x: one warp per block row.  Lanes 0..29 form five groups of six;
// lane (g, i) takes blocks g, g+5, ... of the row and forms the dot product
// of row i of each block (six contiguous values) with the matching six
// entries of x, so every FMA issued is useful and no accumulator is indexed
// dynamically.  The five group partial sums are combined through shared
// memory.
template <typename TV, typename TX>
__global__ void __launch_bounds__(256) k_bcsr_spmv(int nrows, const int *__restrict__ rowp,
                                                   const int *__restrict__ cols,
                                                   const TV *__restrict__ vals,
                                                   const TX *__restrict__ x, TX *__restrict__ y) {
  __shared__ TX part[8][32];
  const int wib = threadIdx.x >> 5;
  const int warp = blockIdx.x * 8 + wib;
  const int lane = threadIdx.x & 31;
  TX acc = 0;
  if (warp < nrows && lane < 30) {
    const int g = lane / 6, i = lane - 6 * g;
    const int start = rowp[warp], end = rowp[warp + 1];
    for (int jp = start + g; jp < end; jp += 5) {
      const TV *a = vals + (size_t)jp * 36 + 6 * i;
      const TX *xv = x + (size_t)cols[jp] * 6;
#pragma unroll
      for (int j = 0; j < 6; j++) acc += (TX)a[j] * xv[j];
    }
  }
  part[wib][lane] = acc;
  __syncwarp();
  if (warp < nrows && lane < 6) {
    TX v = part[wib][lane] + part[wib][lane + 6] + part[wib][lane + 12] +
           part[wib][lane + 18] + part[wib][lane + 24];
    y[(size_t)warp * 6 + lane] = v;
  }
}

int launch_spmv_f64(int nrows, const int *rowp, const int *cols, const double *vals,
                    const double *x, double *y, cudaStream_t s) {
  if (nrows <= 0) return 0;
  int blocks = (nrows * 32 + 255) / 256;
  k_bcsr_spmv<double, double><<<blocks, 256, 0, s>>>(nrows, rowp, cols, vals, x, y);
  A2DS_CUDA_TRY(cudaGetLastError());
  return 0;
}

int launch_spmv_f32(int nrows, const int *rowp, const int *cols, const float *vals,
                    const float *x, float *y, cudaStream_t s) {
  if (nrows <= 0) return 0;
  int blocks = (nrows * 32 + 255) / 256;
  k_bcsr_spmv<float, float><<<blocks, 256, 0, s>>>(nrows, rowp, cols, vals, x, y);
  A2DS_CUDA_TRY(cudaGetLastError());
  return 0;
}

}  // namespace a2ds
