// Multi-vector kernels of the block Lanczos iteration.  A block of p
// vectors of length n6 is stored row-major (n6 x p): entry (i, c) at
// i * p + c, the layout the triangular solves take for p right-hand sides.
// All of these are HBM-bound streams over the blocks, except blk_spmm
// (72 p flops per 6x6 block against 292 bytes: FP64-pipe bound for p >= 4).
#include "a2ds_internal.h"
#include "block.h"

namespace a2ds {

static int grid_for(size_t n, int per = 256) {
  return (int)std::min<size_t>((n + per - 1) / per, (size_t)152 * 16);
}

// Y = A X or Y = B - A X; one warp per block row.  For 6P < 32 the warp
// splits into G groups of 6P lanes that stride over the row's blocks (partial
// sums reduced in shared memory); for larger P each lane owns NPASS outputs.
template <int P>
__global__ void __launch_bounds__(256) k_blk_spmm(int nrows, const int *__restrict__ rowp,
                                                  const int *__restrict__ cols,
                                                  const double *__restrict__ vals,
                                                  const double *__restrict__ X,
                                                  const double *__restrict__ B,
                                                  double *__restrict__ Y) {
  constexpr int NOUT = 6 * P;
  constexpr int G = NOUT >= 32 ? 1 : 32 / NOUT;
  constexpr int NPASS = (NOUT + 31) / 32;
  __shared__ double part[8][G > 1 ? G * NOUT : 1];
  const int wib = threadIdx.x >> 5;
  const int row = blockIdx.x * 8 + wib;
  const int lane = threadIdx.x & 31;
  if (row >= nrows) return;
  const int g = G > 1 ? lane / NOUT : 0;
  const bool live = G > 1 ? lane < G * NOUT : true;
  double acc[NPASS];
#pragma unroll
  for (int q = 0; q < NPASS; q++) acc[q] = 0.0;
  const int kb = rowp[row], ke = rowp[row + 1];
  if (live)
    for (int k = kb + g; k < ke; k += G) {
      const double *a = vals + (size_t)k * 36;
      const double *x = X + (size_t)cols[k] * NOUT;
#pragma unroll
      for (int q = 0; q < NPASS; q++) {
        const int o = G > 1 ? lane - g * NOUT : lane + 32 * q;
        if (o < NOUT) {
          const int d = o / P, c = o - P * d;
          double s = 0.0;
#pragma unroll
          for (int b = 0; b < 6; b++) s += a[6 * d + b] * x[b * P + c];
          acc[q] += s;
        }
      }
    }
  if (G > 1) {
    if (live) part[wib][lane] = acc[0];
    __syncwarp();
    if (lane < NOUT) {
      double v = 0.0;
#pragma unroll
      for (int gg = 0; gg < G; gg++) v += part[wib][gg * NOUT + lane];
      const size_t idx = (size_t)row * NOUT + lane;
      Y[idx] = B ? B[idx] - v : v;
    }
    return;
  }
#pragma unroll
  for (int q = 0; q < NPASS; q++) {
    const int o = lane + 32 * q;
    if (o < NOUT) {
      const size_t idx = (size_t)row * NOUT + o;
      Y[idx] = B ? B[idx] - acc[q] : acc[q];
    }
  }
}

int blk_spmm(int nrows, const int *rowp, const int *cols, const double *vals, const double *X,
             const double *B, double *Y, int p, cudaStream_t s) {
  const int grid = (nrows + 7) / 8;
  switch (p) {
    case 1: k_blk_spmm<1><<<grid, 256, 0, s>>>(nrows, rowp, cols, vals, X, B, Y); break;
    case 2: k_blk_spmm<2><<<grid, 256, 0, s>>>(nrows, rowp, cols, vals, X, B, Y); break;
    case 4: k_blk_spmm<4><<<grid, 256, 0, s>>>(nrows, rowp, cols, vals, X, B, Y); break;
    case 8: k_blk_spmm<8><<<grid, 256, 0, s>>>(nrows, rowp, cols, vals, X, B, Y); break;
    case 16: k_blk_spmm<16><<<grid, 256, 0, s>>>(nrows, rowp, cols, vals, X, B, Y); break;
    default: return fail(A2DS_ERR_ARG, "block size must be 1, 2, 4, 8 or 16");
  }
  A2DS_CUDA_TRY(cudaGetLastError());
  return 0;
}

__global__ void k_blk_zero_bc(double *X, int p, const int *__restrict__ bc_rows,
                              const int *__restrict__ bc_masks, int nbc) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nbc * 6 * p) return;
  const int c = t % p, k = (t / p) % 6, b = t / (6 * p);
  if (bc_masks[b] & (1 << k)) X[((size_t)bc_rows[b] * 6 + k) * p + c] = 0.0;
}

int blk_zero_bc(double *X, int p, const int *bc_rows, const int *bc_masks, int nbc,
                cudaStream_t s) {
  if (nbc <= 0) return 0;
  k_blk_zero_bc<<<(nbc * 6 * p + 255) / 256, 256, 0, s>>>(X, p, bc_rows, bc_masks, nbc);
  A2DS_CUDA_TRY(cudaGetLastError());
  return 0;
}

// H[b][c1][c2] += sum_i Q_b[i][c1] W[i][c2]; blockIdx.y = b.  Threads hold
// one (c1, c2) pair and stride over rows; per-CTA partials go to H with one
// atomic per pair.
__global__ void __launch_bounds__(256) k_blk_dots(const double *__restrict__ Q, size_t bstride,
                                                  const double *__restrict__ W, size_t n6, int p,
                                                  double *__restrict__ H) {
  __shared__ double red[256];
  const int pp = p * p;
  const int rpi = blockDim.x / pp;  // rows per CTA iteration
  const int t = threadIdx.x;
  const int pair = t % pp, lr = t / pp;
  const int c1 = pair / p, c2 = pair % p;
  const double *Qb = Q + (size_t)blockIdx.y * bstride;
  double acc = 0.0;
  if (lr < rpi)
    for (size_t i = (size_t)blockIdx.x * rpi + lr; i < n6; i += (size_t)gridDim.x * rpi)
      acc += Qb[i * p + c1] * W[i * p + c2];
  red[t] = acc;
  __syncthreads();
  if (lr == 0) {
    double v = 0.0;
    for (int r = 0; r < rpi; r++) v += red[r * pp + pair];
    atomicAdd(&H[(size_t)blockIdx.y * pp + pair], v);
  }
}

int blk_dots(const double *Q, int nb, size_t bstride, const double *W, size_t n6, int p,
             double *H, cudaStream_t s) {
  if (p < 1 || p > 16) return fail(A2DS_ERR_ARG, "block size must be <= 16");
  A2DS_CUDA_TRY(cudaMemsetAsync(H, 0, (size_t)nb * p * p * sizeof(double), s));
  dim3 grid((unsigned)std::min<size_t>((n6 + 255) / 256, 152 * 2), (unsigned)nb);
  k_blk_dots<<<grid, 256, 0, s>>>(Q, bstride, W, n6, p, H);
  A2DS_CUDA_TRY(cudaGetLastError());
  return 0;
}

// W[i][c2] -= sum_b sum_c1 Q_b[i][c1] H_b[c1][c2]; H staged in shared memory.
__global__ void __launch_bounds__(256) k_blk_sub(double *__restrict__ W,
                                                 const double *__restrict__ Q, int nb,
                                                 size_t bstride, const double *__restrict__ H,
                                                 size_t n6, int p) {
  extern __shared__ double sH[];
  const int nh = nb * p * p;
  for (int k = threadIdx.x; k < nh; k += blockDim.x) sH[k] = H[k];
  __syncthreads();
  const size_t total = n6 * p;
  for (size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x; t < total;
       t += (size_t)gridDim.x * blockDim.x) {
    const size_t i = t / p;
    const int c2 = (int)(t - i * p);
    double acc = 0.0;
    for (int b = 0; b < nb; b++) {
      const double *q = Q + (size_t)b * bstride + i * p;
      const double *h = sH + (size_t)b * p * p + c2;
      for (int c1 = 0; c1 < p; c1++) acc += q[c1] * h[c1 * p];
    }
    W[t] -= acc;
  }
}

int blk_sub(double *W, const double *Q, int nb, size_t bstride, const double *H, size_t n6, int p,
            cudaStream_t s) {
  const size_t smem = (size_t)nb * p * p * sizeof(double);
  if (smem > 200 * 1024) return fail(A2DS_ERR_ARG, "block Lanczos basis too large for blk_sub");
  static bool configured = false;
  if (!configured) {
    A2DS_CUDA_TRY(cudaFuncSetAttribute(k_blk_sub, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       200 * 1024));
    configured = true;
  }
  k_blk_sub<<<grid_for(n6 * p), 256, smem, s>>>(W, Q, nb, bstride, H, n6, p);
  A2DS_CUDA_TRY(cudaGetLastError());
  return 0;
}

// Y_o = sum_b Q_b C_{b,o} for the output blocks o < nout (n6 x p each, at
// Y + o ostride): Y_o[i][c2] = sum_{b, c1} Q_b[i][c1] C[(b p + c1) (nout p)
// + o p + c2]; C staged in shared memory, one thread per (i, c2).
__global__ void __launch_bounds__(256) k_blk_mul(const double *__restrict__ Q, int nb,
                                                 size_t bstride, const double *__restrict__ C,
                                                 int nout, size_t ostride, size_t n6, int p,
                                                 double *__restrict__ Y) {
  extern __shared__ double sC[];
  const int ld = nout * p, nc = nb * p * ld;
  for (int k = threadIdx.x; k < nc; k += blockDim.x) sC[k] = C[k];
  __syncthreads();
  const size_t total = n6 * p;
  for (size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x; t < total;
       t += (size_t)gridDim.x * blockDim.x) {
    const size_t i = t / p;
    const int c2 = (int)(t - i * p);
    for (int o = 0; o < nout; o++) {
      double acc = 0.0;
      for (int b = 0; b < nb; b++) {
        const double *q = Q + (size_t)b * bstride + i * p;
        const double *c = sC + (size_t)(b * p) * ld + o * p + c2;
        for (int c1 = 0; c1 < p; c1++) acc += q[c1] * c[(size_t)c1 * ld];
      }
      Y[(size_t)o * ostride + t] = acc;
    }
  }
}

int blk_mul(const double *Q, int nb, size_t bstride, const double *C, int nout, size_t ostride,
            size_t n6, int p, double *Y, cudaStream_t s) {
  const size_t smem = (size_t)nb * p * nout * p * sizeof(double);
  if (nb < 1 || nout < 1) return 0;
  if (smem > 200 * 1024) return fail(A2DS_ERR_ARG, "blk_mul: coefficient table too large");
  static bool configured = false;
  if (!configured) {
    A2DS_CUDA_TRY(cudaFuncSetAttribute(k_blk_mul, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       200 * 1024));
    configured = true;
  }
  k_blk_mul<<<grid_for(n6 * p), 256, smem, s>>>(Q, nb, bstride, C, nout, ostride, n6, p, Y);
  A2DS_CUDA_TRY(cudaGetLastError());
  return 0;
}

// X <- X M (M p x p), one thread per row.
template <int P>
__global__ void k_blk_rmul(double *__restrict__ X, const double *__restrict__ M, size_t n6) {
  __shared__ double sM[P * P];
  for (int k = threadIdx.x; k < P * P; k += blockDim.x) sM[k] = M[k];
  __syncthreads();
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n6;
       i += (size_t)gridDim.x * blockDim.x) {
    double x[P];
#pragma unroll
    for (int c = 0; c < P; c++) x[c] = X[i * P + c];
#pragma unroll
    for (int c2 = 0; c2 < P; c2++) {
      double v = 0.0;
#pragma unroll
      for (int c1 = 0; c1 < P; c1++) v += x[c1] * sM[c1 * P + c2];
      X[i * P + c2] = v;
    }
  }
}

int blk_rmul(double *X, const double *M, size_t n6, int p, cudaStream_t s) {
  const int grid = grid_for(n6);
  switch (p) {
    case 1: k_blk_rmul<1><<<grid, 256, 0, s>>>(X, M, n6); break;
    case 2: k_blk_rmul<2><<<grid, 256, 0, s>>>(X, M, n6); break;
    case 4: k_blk_rmul<4><<<grid, 256, 0, s>>>(X, M, n6); break;
    case 8: k_blk_rmul<8><<<grid, 256, 0, s>>>(X, M, n6); break;
    case 16: k_blk_rmul<16><<<grid, 256, 0, s>>>(X, M, n6); break;
    default: return fail(A2DS_ERR_ARG, "block size must be 1, 2, 4, 8 or 16");
  }
  A2DS_CUDA_TRY(cudaGetLastError());
  return 0;
}

// out[k][i] = sum_{b, c} Q_b[i][c] C[(b p + c) nout + k], out contiguous per k.
__global__ void __launch_bounds__(256) k_blk_combine(const double *__restrict__ Q, int nb,
                                                     size_t bstride, int p,
                                                     const double *__restrict__ C, int nout,
                                                     size_t n6, double *__restrict__ out) {
  extern __shared__ double sC[];
  const int nc = nb * p * nout;
  for (int k = threadIdx.x; k < nc; k += blockDim.x) sC[k] = C[k];
  __syncthreads();
  const size_t total = n6 * nout;
  for (size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x; t < total;
       t += (size_t)gridDim.x * blockDim.x) {
    const size_t i = t / nout;
    const int k = (int)(t - i * nout);
    double acc = 0.0;
    for (int b = 0; b < nb; b++) {
      const double *q = Q + (size_t)b * bstride + i * p;
      for (int c = 0; c < p; c++) acc += q[c] * sC[(b * p + c) * nout + k];
    }
    out[(size_t)k * n6 + i] = acc;
  }
}

int blk_combine(const double *Q, int nb, size_t bstride, int p, const double *C, int nout,
                size_t n6, double *out, cudaStream_t s) {
  const size_t smem = (size_t)nb * p * nout * sizeof(double);
  if (smem > 200 * 1024) return fail(A2DS_ERR_ARG, "too many Ritz vectors for blk_combine");
  static bool configured = false;
  if (!configured) {
    A2DS_CUDA_TRY(cudaFuncSetAttribute(k_blk_combine,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024));
    configured = true;
  }
  k_blk_combine<<<grid_for(n6 * nout), 256, smem, s>>>(Q, nb, bstride, p, C, nout, n6, out);
  A2DS_CUDA_TRY(cudaGetLastError());
  return 0;
}

// ---------------------------------------------------- column-wise kernels
// Each column of an n6 x p block carries its own Krylov space (p GMRES
// solves in lockstep), so these kernels pair column c only with column c.
// Grid strides are multiples of p (256-thread CTAs, p <= 16), so a thread
// keeps one column for its whole walk.

// out[b p + c] += sum_i Q_b[i][c] W[i][c] for b in [8 blockIdx.y, +8) and b < nb.
__global__ void __launch_bounds__(256) k_col_dots(const double *__restrict__ Q, int nb,
                                                  size_t bstride, const double *__restrict__ W,
                                                  size_t n6, int p, double *__restrict__ out) {
  __shared__ double red[8][8][16];
  const int b0 = blockIdx.y * 8;
  const int nbl = min(8, nb - b0);
  double acc[8];
#pragma unroll
  for (int k = 0; k < 8; k++) acc[k] = 0.0;
  const size_t total = n6 * p;
  for (size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x; e < total;
       e += (size_t)gridDim.x * blockDim.x) {
    const double w = W[e];
#pragma unroll
    for (int k = 0; k < 8; k++)
      if (k < nbl) acc[k] += Q[(size_t)(b0 + k) * bstride + e] * w;
  }
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
  for (int k = 0; k < 8; k++) {
    double v = acc[k];
    for (int o = 16; o >= p; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if (lane < p) red[wid][k][lane] = v;
  }
  __syncthreads();
  if (threadIdx.x < 8 * p) {
    const int k = threadIdx.x / p, c = threadIdx.x % p;
    if (k < nbl) {
      double v = 0.0;
      for (int w = 0; w < (int)(blockDim.x >> 5); w++) v += red[w][k][c];
      atomicAdd(&out[(size_t)(b0 + k) * p + c], v);
    }
  }
}

int col_dots(const double *Q, int nb, size_t bstride, const double *W, size_t n6, int p,
             double *out, cudaStream_t s) {
  if (p < 1 || p > 16 || (p & (p - 1))) return fail(A2DS_ERR_ARG, "block size must be 1..16, a power of 2");
  if (nb < 1) return 0;
  A2DS_CUDA_TRY(cudaMemsetAsync(out, 0, (size_t)nb * p * sizeof(double), s));
  dim3 grid((unsigned)std::min<size_t>((n6 * p + 255) / 256, 152 * 4), (unsigned)((nb + 7) / 8));
  k_col_dots<<<grid, 256, 0, s>>>(Q, nb, bstride, W, n6, p, out);
  A2DS_CUDA_TRY(cudaGetLastError());
  return 0;
}

// W[i][c] -= sum_b Q_b[i][c] h[b p + c]   (sign = -1), or
// W[i][c] += sum_b Q_b[i][c] h[b p + c]   (sign = +1); h on the device.
__global__ void __launch_bounds__(256) k_col_axpy(double *__restrict__ W,
                                                  const double *__restrict__ Q, int nb,
                                                  size_t bstride, const double *__restrict__ h,
                                                  size_t n6, int p, double sign) {
  __shared__ double sh[64 * 16];
  for (int k = threadIdx.x; k < nb * p; k += blockDim.x) sh[k] = sign * h[k];
  __syncthreads();
  const size_t total = n6 * p;
  for (size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x; e < total;
       e += (size_t)gridDim.x * blockDim.x) {
    const int c = (int)(e & (size_t)(p - 1));
    double acc = 0.0;
    for (int b = 0; b < nb; b++) acc += Q[(size_t)b * bstride + e] * sh[b * p + c];
    W[e] += acc;
  }
}

int col_axpy(double *W, const double *Q, int nb, size_t bstride, const double *h, size_t n6,
             int p, double sign, cudaStream_t s) {
  if (nb < 1) return 0;
  if (nb > 64 || p > 16 || (p & (p - 1))) return fail(A2DS_ERR_ARG, "col_axpy: too many blocks");
  k_col_axpy<<<grid_for(n6 * p), 256, 0, s>>>(W, Q, nb, bstride, h, n6, p, sign);
  A2DS_CUDA_TRY(cudaGetLastError());
  return 0;
}

// W[i][c] /= sqrt(nrm2[c]) (columns with nrm2[c] == 0 are left as they are).
// (The p scale factors are formed once per CTA: FP64 square roots and
// divisions per element would bound the kernel by the FP64 pipe.)
__global__ void k_col_unit(double *__restrict__ W, const double *__restrict__ nrm2, size_t n6,
                           int p) {
  __shared__ double sc[16];
  if (threadIdx.x < p) {
    const double q = nrm2[threadIdx.x];
    sc[threadIdx.x] = q > 0.0 ? 1.0 / sqrt(q) : 1.0;
  }
  __syncthreads();
  const size_t total = n6 * p;
  for (size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x; e < total;
       e += (size_t)gridDim.x * blockDim.x)
    W[e] *= sc[e & (size_t)(p - 1)];
}

int col_unit(double *W, const double *nrm2, size_t n6, int p, cudaStream_t s) {
  k_col_unit<<<grid_for(n6 * p), 256, 0, s>>>(W, nrm2, n6, p);
  A2DS_CUDA_TRY(cudaGetLastError());
  return 0;
}

__global__ void k_blk_add(double *__restrict__ Y, const double *__restrict__ X, size_t n) {
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x)
    Y[i] += X[i];
}

int blk_add(double *Y, const double *X, size_t n, cudaStream_t s) {
  k_blk_add<<<grid_for(n), 256, 0, s>>>(Y, X, n);
  A2DS_CUDA_TRY(cudaGetLastError());
  return 0;
}

}  // namespace a2ds
