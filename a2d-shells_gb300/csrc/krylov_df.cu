// Double-float Krylov kernels: the inner GMRES of the mixed-precision
// shift-invert solves on the FP32 pipe.
//
// On GB300 the FP64 pipe issues ~1/60 of the FP32 rate, so the FP64 passes
// of GMRES -- the block product A Z and the Gram-Schmidt dots and updates --
// are bound by FP64 FMAs (~0.55 T/s, one FMA per 8 bytes caps a pass near
// 4.4 TB/s), not by memory.  Here the Arnoldi vectors and the shifted
// operator are double-float (df64: an unevaluated sum hi + lo of two FP32
// values, a ~48-bit significand, the same 8 bytes as FP64), and every
// product is an exact FP32 product (FMA error term) plus the cross terms,
// accumulated by two-sum: ~10 FP32 operations per FMA, so the passes become
// memory-bound.  The preconditioned vectors Z start as the FP32 factor's
// output (the product A Z reads them as FP32) and are kept as df64, so that
// the deflation's correction z + Y c and A z + (A Y) c stay consistent:
// flexible GMRES needs A Z formed from exactly the Z it keeps.  A rounding unit of ~2^-48 instead of 2^-53 puts the floor of
// the attainable relative residual near 1e-12 on these matrices, well below
// the shift-invert solves' tolerance (1e-9).
#include "a2ds_internal.h"
#include "block.h"
#include "df64.h"

namespace a2ds {

static int grid_for_df(size_t n) {
  return (int)std::min<size_t>((n + 255) / 256, (size_t)152 * 16);
}

// (hi, lo) += a b for df64 a and FP32 b (exact leading product, the low
// part's product rounded), and for df64 a, b.
__device__ __forceinline__ void df_acc(float &hi, float &lo, df64 a, float b) {
  const float ph = __fmul_rn(a.hi, b);
  float pe = fmaf(a.hi, b, -ph);
  pe = fmaf(a.lo, b, pe);
  const float s = __fadd_rn(hi, ph);
  const float bb = __fsub_rn(s, hi);
  const float err = __fadd_rn(__fsub_rn(hi, __fsub_rn(s, bb)), __fsub_rn(ph, bb));
  hi = s;
  lo = __fadd_rn(lo, __fadd_rn(err, pe));
}
__device__ __forceinline__ void df_acc(float &hi, float &lo, df64 a, df64 b) {
  const float ph = __fmul_rn(a.hi, b.hi);
  float pe = fmaf(a.hi, b.hi, -ph);
  pe = fmaf(a.hi, b.lo, pe);
  pe = fmaf(a.lo, b.hi, pe);
  const float s = __fadd_rn(hi, ph);
  const float bb = __fsub_rn(s, hi);
  const float err = __fadd_rn(__fsub_rn(hi, __fsub_rn(s, bb)), __fsub_rn(ph, bb));
  hi = s;
  lo = __fadd_rn(lo, __fadd_rn(err, pe));
}
__device__ __forceinline__ double df_val(float hi, float lo) { return (double)hi + (double)lo; }

__device__ __forceinline__ df64 df_load(const df64 *p, size_t i) { return p[i]; }
__device__ __forceinline__ df64 df_load(const float *p, size_t i) { return df64{p[i], 0.0f}; }

// ------------------------------------------------------------ conversions
__global__ void k_df_from_f64(df64 *__restrict__ out, const double *__restrict__ in, size_t n) {
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x)
    out[i] = df_split(in[i]);
}
__global__ void k_df_hi(float *__restrict__ out, const df64 *__restrict__ in, size_t n) {
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x)
    out[i] = in[i].hi;
}
__global__ void k_df_split_small(df64 *__restrict__ out, const double *__restrict__ in, int n,
                                 double scale) {
  for (int i = threadIdx.x; i < n; i += blockDim.x) out[i] = df_split(scale * in[i]);
}

int df_from_f64(df64 *out, const double *in, size_t n, cudaStream_t s) {
  k_df_from_f64<<<grid_for_df(n), 256, 0, s>>>(out, in, n);
  A2DS_CUDA_TRY(cudaGetLastError());
  return 0;
}
int df_hi(float *out, const df64 *in, size_t n, cudaStream_t s) {
  k_df_hi<<<grid_for_df(n), 256, 0, s>>>(out, in, n);
  A2DS_CUDA_TRY(cudaGetLastError());
  return 0;
}
__global__ void k_df_from_f32(df64 *__restrict__ out, const float *__restrict__ in, size_t n) {
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x)
    out[i] = df64{in[i], 0.0f};
}
int df_from_f32(df64 *out, const float *in, size_t n, cudaStream_t s) {
  k_df_from_f32<<<grid_for_df(n), 256, 0, s>>>(out, in, n);
  A2DS_CUDA_TRY(cudaGetLastError());
  return 0;
}

// ------------------------------------------------------- block product
// W = A Z (A df64 6x6 blocks, Z FP32, W df64), one warp per block row, the
// same lane layout as the FP64 block product: for 6P < 32, G groups of 6P
// lanes stride over the row's blocks; otherwise each lane owns NPASS outputs.
template <int P>
__global__ void __launch_bounds__(256) k_df_spmm(int nrows, const int *__restrict__ rowp,
                                                 const int *__restrict__ cols,
                                                 const df64 *__restrict__ vals,
                                                 const float *__restrict__ Z,
                                                 df64 *__restrict__ W) {
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
  float hi[NPASS], lo[NPASS];
#pragma unroll
  for (int q = 0; q < NPASS; q++) hi[q] = lo[q] = 0.0f;
  const int kb = rowp[row], ke = rowp[row + 1];
  if (live)
    for (int k = kb + g; k < ke; k += G) {
      const df64 *a = vals + (size_t)k * 36;
      const float *x = Z + (size_t)cols[k] * NOUT;
#pragma unroll
      for (int q = 0; q < NPASS; q++) {
        const int o = G > 1 ? lane - g * NOUT : lane + 32 * q;
        if (o < NOUT) {
          const int d = o / P, c = o - P * d;
#pragma unroll
          for (int b = 0; b < 6; b++) df_acc(hi[q], lo[q], a[6 * d + b], x[b * P + c]);
        }
      }
    }
  if constexpr (G > 1) {
    // the G partial sums of an output are added in FP64 (a few per row)
    if (live) part[wib][lane] = df_val(hi[0], lo[0]);
    __syncwarp();
    if (lane < NOUT) {
      double v = 0.0;
#pragma unroll
      for (int gg = 0; gg < G; gg++) v += part[wib][gg * NOUT + lane];
      W[(size_t)row * NOUT + lane] = df_split(v);
    }
  } else {
#pragma unroll
    for (int q = 0; q < NPASS; q++) {
      const int o = lane + 32 * q;
      if (o < NOUT) {
        const float s = __fadd_rn(hi[q], lo[q]);
        W[(size_t)row * NOUT + o] = df64{s, __fsub_rn(lo[q], __fsub_rn(s, hi[q]))};
      }
    }
  }
}

int df_spmm(int nrows, const int *rowp, const int *cols, const df64 *vals, const float *Z,
            df64 *W, int p, cudaStream_t s) {
  const int grid = (nrows + 7) / 8;
  switch (p) {
    case 1: k_df_spmm<1><<<grid, 256, 0, s>>>(nrows, rowp, cols, vals, Z, W); break;
    case 2: k_df_spmm<2><<<grid, 256, 0, s>>>(nrows, rowp, cols, vals, Z, W); break;
    case 4: k_df_spmm<4><<<grid, 256, 0, s>>>(nrows, rowp, cols, vals, Z, W); break;
    case 8: k_df_spmm<8><<<grid, 256, 0, s>>>(nrows, rowp, cols, vals, Z, W); break;
    case 16: k_df_spmm<16><<<grid, 256, 0, s>>>(nrows, rowp, cols, vals, Z, W); break;
    default: return fail(A2DS_ERR_ARG, "block size must be 1, 2, 4, 8 or 16");
  }
  A2DS_CUDA_TRY(cudaGetLastError());
  return 0;
}

// ---------------------------------------------------- column-wise passes
// Column c of one block only meets column c of another (p Krylov spaces in
// lockstep); grid strides are multiples of p, so a thread keeps its column.

// out[b p + c] = sum_i Q_b[i][c] W[i][c] for b in [8 blockIdx.y, +8), b < nb
// (out zeroed first): df64 sums per thread, FP64 across threads.
template <typename TQ>
__global__ void __launch_bounds__(256) k_df_col_dots(const TQ *__restrict__ Q, int nb,
                                                     size_t bstride, const df64 *__restrict__ W,
                                                     size_t n6, int p, double *__restrict__ out) {
  __shared__ double red[8][8][16];
  const int b0 = blockIdx.y * 8;
  const int nbl = min(8, nb - b0);
  float hi[8], lo[8];
#pragma unroll
  for (int k = 0; k < 8; k++) hi[k] = lo[k] = 0.0f;
  const size_t total = n6 * p;
  for (size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x; e < total;
       e += (size_t)gridDim.x * blockDim.x) {
    const df64 w = W[e];
#pragma unroll
    for (int k = 0; k < 8; k++)
      if (k < nbl) df_acc(hi[k], lo[k], w, df_load(Q, (size_t)(b0 + k) * bstride + e));
  }
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
  for (int k = 0; k < 8; k++) {
    double v = df_val(hi[k], lo[k]);
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

template <typename TQ>
static int df_col_dots_t(const TQ *Q, int nb, size_t bstride, const df64 *W, size_t n6, int p,
                         double *out, cudaStream_t s) {
  if (p < 1 || p > 16 || (p & (p - 1))) return fail(A2DS_ERR_ARG, "block size must be 1..16, a power of 2");
  if (nb < 1) return 0;
  A2DS_CUDA_TRY(cudaMemsetAsync(out, 0, (size_t)nb * p * sizeof(double), s));
  dim3 grid((unsigned)std::min<size_t>((n6 * p + 255) / 256, 152 * 4), (unsigned)((nb + 7) / 8));
  k_df_col_dots<TQ><<<grid, 256, 0, s>>>(Q, nb, bstride, W, n6, p, out);
  A2DS_CUDA_TRY(cudaGetLastError());
  return 0;
}
int df_col_dots(const df64 *Q, int nb, size_t bstride, const df64 *W, size_t n6, int p,
                double *out, cudaStream_t s) {
  return df_col_dots_t(Q, nb, bstride, W, n6, p, out, s);
}

// W[e] += sum_b Q_b[e] h[b p + c] (h: df64 coefficients, sign already in).
__global__ void __launch_bounds__(256) k_df_col_axpy(df64 *__restrict__ W,
                                                     const df64 *__restrict__ Q, int nb,
                                                     size_t bstride, const df64 *__restrict__ h,
                                                     size_t n6, int p) {
  __shared__ df64 sh[64 * 16];
  for (int k = threadIdx.x; k < nb * p; k += blockDim.x) sh[k] = h[k];
  __syncthreads();
  const size_t total = n6 * p;
  for (size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x; e < total;
       e += (size_t)gridDim.x * blockDim.x) {
    const int c = (int)(e & (size_t)(p - 1));
    const df64 w = W[e];
    float hi = w.hi, lo = w.lo;
    for (int b = 0; b < nb; b++) df_acc(hi, lo, Q[(size_t)b * bstride + e], sh[b * p + c]);
    const float s = __fadd_rn(hi, lo);
    W[e] = df64{s, __fsub_rn(lo, __fsub_rn(s, hi))};
  }
}

int df_col_axpy(df64 *W, const df64 *Q, int nb, size_t bstride, const double *h, size_t n6,
                int p, double sign, df64 *hscratch, cudaStream_t s) {
  if (nb < 1) return 0;
  if (nb > 64 || p > 16 || (p & (p - 1))) return fail(A2DS_ERR_ARG, "df_col_axpy: too many blocks");
  k_df_split_small<<<1, 256, 0, s>>>(hscratch, h, nb * p, sign);
  k_df_col_axpy<<<grid_for_df(n6 * p), 256, 0, s>>>(W, Q, nb, bstride, hscratch, n6, p);
  A2DS_CUDA_TRY(cudaGetLastError());
  return 0;
}

// W[i][c] *= 1 / sqrt(nrm2[c]) (columns with nrm2[c] == 0 left as they are).
__global__ void k_df_col_unit(df64 *__restrict__ W, const double *__restrict__ nrm2, size_t n6,
                              int p) {
  __shared__ df64 sc[16];
  if (threadIdx.x < p) {
    const double q = nrm2[threadIdx.x];
    sc[threadIdx.x] = df_split(q > 0.0 ? 1.0 / sqrt(q) : 1.0);
  }
  __syncthreads();
  const size_t total = n6 * p;
  for (size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x; e < total;
       e += (size_t)gridDim.x * blockDim.x) {
    float hi = 0.0f, lo = 0.0f;
    df_acc(hi, lo, W[e], sc[e & (size_t)(p - 1)]);
    const float s = __fadd_rn(hi, lo);
    W[e] = df64{s, __fsub_rn(lo, __fsub_rn(s, hi))};
  }
}

int df_col_unit(df64 *W, const double *nrm2, size_t n6, int p, cudaStream_t s) {
  k_df_col_unit<<<grid_for_df(n6 * p), 256, 0, s>>>(W, nrm2, n6, p);
  A2DS_CUDA_TRY(cudaGetLastError());
  return 0;
}

// Y[e] += sum_b Z_b[e] y[b p + c] in FP64 (Z df64: the update of the
// solution by the kept preconditioned vectors, once per cycle).
__global__ void __launch_bounds__(256) k_df_col_axpy_f64(double *__restrict__ Y,
                                                         const df64 *__restrict__ Z, int nb,
                                                         size_t bstride,
                                                         const double *__restrict__ y,
                                                         size_t n6, int p) {
  __shared__ double sy[64 * 16];
  for (int k = threadIdx.x; k < nb * p; k += blockDim.x) sy[k] = y[k];
  __syncthreads();
  const size_t total = n6 * p;
  for (size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x; e < total;
       e += (size_t)gridDim.x * blockDim.x) {
    const int c = (int)(e & (size_t)(p - 1));
    double acc = 0.0;
    for (int b = 0; b < nb; b++) {
      const df64 z = Z[(size_t)b * bstride + e];
      acc += ((double)z.hi + (double)z.lo) * sy[b * p + c];
    }
    Y[e] += acc;
  }
}

int df_col_axpy_f64(double *Y, const df64 *Z, int nb, size_t bstride, const double *y,
                    size_t n6, int p, cudaStream_t s) {
  if (nb < 1) return 0;
  if (nb > 64 || p > 16) return fail(A2DS_ERR_ARG, "df_col_axpy_f64: too many blocks");
  k_df_col_axpy_f64<<<grid_for_df(n6 * p), 256, 0, s>>>(Y, Z, nb, bstride, y, n6, p);
  A2DS_CUDA_TRY(cudaGetLastError());
  return 0;
}

// ------------------------------------------------------------ deflation
// T = V - AZ (df64).
__global__ void k_df_diff(df64 *__restrict__ T, const df64 *__restrict__ V,
                          const df64 *__restrict__ AZ, size_t n) {
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x) {
    const df64 v = V[i], a = AZ[i];
    const float s = __fsub_rn(v.hi, a.hi);
    const float bb = __fsub_rn(s, v.hi);
    const float err = __fadd_rn(__fsub_rn(v.hi, __fsub_rn(s, bb)), __fsub_rn(-a.hi, bb));
    const float lo = __fadd_rn(err, __fsub_rn(v.lo, a.lo));
    const float h = __fadd_rn(s, lo);
    T[i] = df64{h, __fsub_rn(lo, __fsub_rn(h, s))};
  }
}
int df_diff(df64 *T, const df64 *V, const df64 *AZ, size_t n, cudaStream_t s) {
  k_df_diff<<<grid_for_df(n), 256, 0, s>>>(T, V, AZ, n);
  A2DS_CUDA_TRY(cudaGetLastError());
  return 0;
}

// H[b][c1][c2] = sum_i Y_b[i][c1] T[i][c2] (Y FP32, T df64; H zeroed
// first, FP64 output); blockIdx.y = b.
__global__ void __launch_bounds__(256) k_df_blk_dots(const float *__restrict__ Y, size_t bstride,
                                                     const df64 *__restrict__ T, size_t n6,
                                                     int p, double *__restrict__ H) {
  __shared__ double red[256];
  const int pp = p * p;
  const int rpi = blockDim.x / pp;
  const int t = threadIdx.x;
  const int pair = t % pp, lr = t / pp;
  const int c1 = pair / p, c2 = pair % p;
  const float *Yb = Y + (size_t)blockIdx.y * bstride;
  float hi = 0.0f, lo = 0.0f;
  if (lr < rpi)
    for (size_t i = (size_t)blockIdx.x * rpi + lr; i < n6; i += (size_t)gridDim.x * rpi)
      df_acc(hi, lo, T[i * p + c2], Yb[i * p + c1]);
  red[t] = lr < rpi ? df_val(hi, lo) : 0.0;
  __syncthreads();
  if (lr == 0) {
    double v = 0.0;
    for (int r = 0; r < rpi; r++) v += red[r * pp + pair];
    atomicAdd(&H[(size_t)blockIdx.y * pp + pair], v);
  }
}
int df_blk_dots(const float *Y, int nb, size_t bstride, const df64 *T, size_t n6, int p,
                double *H, cudaStream_t s) {
  if (p < 1 || p > 16) return fail(A2DS_ERR_ARG, "block size must be <= 16");
  A2DS_CUDA_TRY(cudaMemsetAsync(H, 0, (size_t)nb * p * p * sizeof(double), s));
  dim3 grid((unsigned)std::min<size_t>((n6 + 255) / 256, 152 * 2), (unsigned)nb);
  k_df_blk_dots<<<grid, 256, 0, s>>>(Y, bstride, T, n6, p, H);
  A2DS_CUDA_TRY(cudaGetLastError());
  return 0;
}

// Z[i][c2] -= sum_b sum_c1 Y_b[i][c1] H_b[c1][c2] (df64 Z, FP32 Y; the
// preconditioner's correction) and AZ -= the same with AY (df64), one
// thread per (i, c2); H (FP64, on the device) staged as df64.
__global__ void __launch_bounds__(256) k_df_defl_sub(df64 *__restrict__ Z,
                                                     const float *__restrict__ Y,
                                                     df64 *__restrict__ AZ,
                                                     const df64 *__restrict__ AY, int nb,
                                                     size_t bstride, const double *__restrict__ H,
                                                     size_t n6, int p) {
  __shared__ df64 sH[16 * 16 * 4];
  const int nh = nb * p * p;
  for (int k = threadIdx.x; k < nh; k += blockDim.x) sH[k] = df_split(-H[k]);
  __syncthreads();
  const size_t total = n6 * p;
  for (size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x; t < total;
       t += (size_t)gridDim.x * blockDim.x) {
    const size_t i = t / p;
    const int c2 = (int)(t - i * p);
    const df64 z = Z[t], a = AZ[t];
    float zh = z.hi, zl = z.lo, hi = a.hi, lo = a.lo;
    for (int b = 0; b < nb; b++) {
      const size_t base = (size_t)b * bstride + i * p;
      for (int c1 = 0; c1 < p; c1++) {
        const df64 h = sH[(b * p + c1) * p + c2];
        df_acc(zh, zl, h, Y[base + c1]);
        df_acc(hi, lo, AY[base + c1], h);
      }
    }
    const float sz = __fadd_rn(zh, zl);
    Z[t] = df64{sz, __fsub_rn(zl, __fsub_rn(sz, zh))};
    const float s = __fadd_rn(hi, lo);
    AZ[t] = df64{s, __fsub_rn(lo, __fsub_rn(s, hi))};
  }
}
int df_defl_sub(df64 *Z, const float *Y, df64 *AZ, const df64 *AY, int nb, size_t bstride,
                const double *H, size_t n6, int p, cudaStream_t s) {
  if (nb * p * p > 16 * 16 * 4) return fail(A2DS_ERR_ARG, "df_defl_sub: too many coefficients");
  k_df_defl_sub<<<grid_for_df(n6 * p), 256, 0, s>>>(Z, Y, AZ, AY, nb, bstride, H, n6, p);
  A2DS_CUDA_TRY(cudaGetLastError());
  return 0;
}

// FP64 -> FP32 (the deflation vectors Y as the FP32 preconditioner uses them).
__global__ void k_f64_to_f32_df(float *__restrict__ y, const double *__restrict__ x, size_t n) {
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x)
    y[i] = (float)x[i];
}
int f64_to_f32(float *y, const double *x, size_t n, cudaStream_t s) {
  k_f64_to_f32_df<<<grid_for_df(n), 256, 0, s>>>(y, x, n);
  A2DS_CUDA_TRY(cudaGetLastError());
  return 0;
}

}  // namespace a2ds
