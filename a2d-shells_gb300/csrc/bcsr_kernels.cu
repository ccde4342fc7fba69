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

// y = A x, one warp per block row: lanes 0..29 form five groups of six;
// lane (g, i) takes blocks g, g+5, ... of the row and forms the dot product
// of row i of each block (six contiguous values) with the matching six
// entries of x, so every FMA issued is useful and no accumulator is indexed
// dynamically; the five group partial sums are combined through shared
// memory.  FP64 values are read with 16-byte loads: lane (g, i) reads row
// i of a block as three double2 (a block row of 48 bytes, 16-byte aligned
// since blocks are 288 bytes) and the six x entries as three double2; the
// row's column indices are read once by the warp (lane l holds column
// start + l) and handed to the groups by shuffles, so no group waits on an
// index load before its gather.  Two passes cover the usual 6-10 block rows
// of Quad4 meshes.
__global__ void __launch_bounds__(256) k_bcsr_spmv_f64(int nrows, const int *__restrict__ rowp,
                                                       const int *__restrict__ cols,
                                                       const double *__restrict__ vals,
                                                       const double *__restrict__ x,
                                                       double *__restrict__ y) {
  __shared__ double part[8][32];
  const int wib = threadIdx.x >> 5;
  const int row = blockIdx.x * 8 + wib;
  const int lane = threadIdx.x & 31;
  if (row >= nrows) return;  // whole warp
  const int g = lane / 6, i = lane - 6 * g;
  const int start = rowp[row], end = rowp[row + 1];
  double acc = 0.0;
  for (int base = start; base < end; base += 32) {
    const int myc = base + lane < end ? cols[base + lane] : 0;
    const int nb = min(32, end - base);
    for (int k = 0; k < nb; k += 5) {
      const int slot = k + g;  // this group's block, if any
      const int c = __shfl_sync(0xffffffffu, myc, slot < 32 ? slot : 0);
      if (lane < 30 && slot < nb) {
        const double2 *a = reinterpret_cast<const double2 *>(vals + (size_t)(base + slot) * 36 + 6 * i);
        const double2 *xv = reinterpret_cast<const double2 *>(x + (size_t)c * 6);
        const double2 a0 = a[0], a1 = a[1], a2 = a[2];
        const double2 x0 = __ldg(xv), x1 = __ldg(xv + 1), x2 = __ldg(xv + 2);
        acc += a0.x * x0.x + a0.y * x0.y + a1.x * x1.x + a1.y * x1.y + a2.x * x2.x + a2.y * x2.y;
      }
    }
  }
  part[wib][lane] = lane < 30 ? acc : 0.0;
  __syncwarp();
  if (lane < 6)
    y[(size_t)row * 6 + lane] = part[wib][lane] + part[wib][lane + 6] + part[wib][lane + 12] +
                                part[wib][lane + 18] + part[wib][lane + 24];
}

int launch_spmv_f64(int nrows, const int *rowp, const int *cols, const double *vals,
                    const double *x, double *y, cudaStream_t s) {
  if (nrows <= 0) return 0;
  int blocks = (nrows * 32 + 255) / 256;
  k_bcsr_spmv_f64<<<blocks, 256, 0, s>>>(nrows, rowp, cols, vals, x, y);
  A2DS_CUDA_TRY(cudaGetLastError());
  return 0;
}

}  // namespace a2ds
