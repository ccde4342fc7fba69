// Multi-vector (block) kernels for the block Lanczos iteration; a block of p
// vectors is stored row-major (n6 x p).  p in {1, 2, 4, 8, 16}.
#pragma once
#include <cuda_runtime.h>
#include <stddef.h>

#include <algorithm>

namespace a2ds {
// Y = A X (B == NULL) or Y = B - A X for a 6x6-block CSR matrix.
int blk_spmm(int nrows, const int *rowp, const int *cols, const double *vals, const double *X,
             const double *B, double *Y, int p, cudaStream_t s);
// Zero the Dirichlet DOFs of every vector of the block.
int blk_zero_bc(double *X, int p, const int *bc_rows, const int *bc_masks, int nbc,
                cudaStream_t s);
// H[b] = Q_b^T W (p x p, row c1 = column of Q_b) for b < nb, Q_b = Q + b * bstride.
int blk_dots(const double *Q, int nb, size_t bstride, const double *W, size_t n6, int p,
             double *H, cudaStream_t s);
// W -= sum_b Q_b H[b] (H on the device).
int blk_sub(double *W, const double *Q, int nb, size_t bstride, const double *H, size_t n6, int p,
            cudaStream_t s);
// Y_o = sum_b Q_b C_{b,o} for o < nout (each n6 x p, at Y + o ostride):
// Y_o[i][c2] = sum_{b, c1} Q_b[i][c1] C[(b p + c1) (nout p) + o p + c2].
int blk_mul(const double *Q, int nb, size_t bstride, const double *C, int nout, size_t ostride,
            size_t n6, int p, double *Y, cudaStream_t s);
// X <- X M, M p x p row-major on the device.
int blk_rmul(double *X, const double *M, size_t n6, int p, cudaStream_t s);
// out[k] (contiguous, length n6) = sum_{b, c} column c of Q_b times C[(b p + c) nout + k].
int blk_combine(const double *Q, int nb, size_t bstride, int p, const double *C, int nout,
                size_t n6, double *out, cudaStream_t s);
// Y += X (n values).
int blk_add(double *Y, const double *X, size_t n, cudaStream_t s);

// Column-wise forms (column c of one block only meets column c of another;
// p independent Krylov spaces in lockstep; p a power of 2 up to 16):
// out[b p + c] = sum_i Q_b[i][c] W[i][c] for b < nb (out zeroed first).
int col_dots(const double *Q, int nb, size_t bstride, const double *W, size_t n6, int p,
             double *out, cudaStream_t s);
// W[i][c] += sign * sum_b Q_b[i][c] h[b p + c], nb <= 64, h on the device.
int col_axpy(double *W, const double *Q, int nb, size_t bstride, const double *h, size_t n6,
             int p, double sign, cudaStream_t s);
// W[i][c] /= sqrt(nrm2[c]) where nrm2[c] > 0 (nrm2 on the device).
int col_unit(double *W, const double *nrm2, size_t n6, int p, cudaStream_t s);
}  // namespace a2ds
