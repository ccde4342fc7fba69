// Multi-vector (block) kernels for the block Lanczos iteration; a block of p
// vectors is stored row-major (n6 x p).  p in {1, 2, 4, 8, 16}.
#pragma once
#include <cuda_runtime.h>
#include <stddef.h>

#include <algorithm>

namespace a2ds {
struct df64;  // double-float value (df64.h)
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

// Double-float Krylov passes (krylov_df.cu): the inner GMRES of the
// mixed-precision solves on the FP32 pipe.  Vectors are df64 (n6 x p,
// row-major like the FP64 blocks) or FP32; coefficients FP64 on the device.
int df_from_f64(df64 *out, const double *in, size_t n, cudaStream_t s);
int df_hi(float *out, const df64 *in, size_t n, cudaStream_t s);  // the FP32 rounding
int df_from_f32(df64 *out, const float *in, size_t n, cudaStream_t s);
int f64_to_f32(float *y, const double *x, size_t n, cudaStream_t s);
// W = A Z, A df64 6x6 blocks in the mesh pattern, Z FP32.
int df_spmm(int nrows, const int *rowp, const int *cols, const df64 *vals, const float *Z,
            df64 *W, int p, cudaStream_t s);
// out[b p + c] = sum_i Q_b[i][c] W[i][c] (out zeroed first).
int df_col_dots(const df64 *Q, int nb, size_t bstride, const df64 *W, size_t n6, int p,
                double *out, cudaStream_t s);
// W[i][c] += sign sum_b Q_b[i][c] h[b p + c]; hscratch: 64 x 16 df64 on the device.
int df_col_axpy(df64 *W, const df64 *Q, int nb, size_t bstride, const double *h, size_t n6,
                int p, double sign, df64 *hscratch, cudaStream_t s);
int df_col_unit(df64 *W, const double *nrm2, size_t n6, int p, cudaStream_t s);
// Y[i][c] += sum_b Z_b[i][c] y[b p + c] in FP64 (Z df64).
int df_col_axpy_f64(double *Y, const df64 *Z, int nb, size_t bstride, const double *y,
                    size_t n6, int p, cudaStream_t s);
int df_diff(df64 *T, const df64 *V, const df64 *AZ, size_t n, cudaStream_t s);  // T = V - AZ
// H_b = Y_b^T T (p x p per block b < nb; Y FP32, T df64).
int df_blk_dots(const float *Y, int nb, size_t bstride, const df64 *T, size_t n6, int p,
                double *H, cudaStream_t s);
// Z -= sum_b Y_b H_b and AZ -= sum_b AY_b H_b (Z, AZ df64; Y FP32).
int df_defl_sub(df64 *Z, const float *Y, df64 *AZ, const df64 *AY, int nb, size_t bstride,
                const double *H, size_t n6, int p, cudaStream_t s);
}  // namespace a2ds
