// Level-scheduled block ILU(k) / LU factorization and triangular solves for
// 6x6-block CSR matrices, FP64 or FP32.
//
// Numerics follow BCSRMatFactor6 (src/bpmat/BCSRMatFact6.cpp:946-1330):
// every L block becomes L_ij = A_ij D_j^{-1}, the row is updated with
// -L_ij U_jk on the ILU pattern, and each diagonal block is finally replaced
// by its inverse (partial pivoting, as BMatComputeInverse,
// src/bpmat/BCSRMatMult.cpp:308).  The solves follow BCSRMatApplyLower6 /
// BCSRMatApplyUpper6 (src/bpmat/BCSRMatMult6.cpp:319-416): unit-lower
// forward substitution, then backward substitution with the stored inverse
// diagonal.
//
// Parallel schedule (GB300-side, not the reference's):
// * factorization is right-looking by dependency levels.  For level l,
//   (1) the pivot kernel inverts the diagonal blocks of the level's rows
//   (final once every lower level has been applied), (2) the update kernel
//   runs one thread block per target row that has L entries in level-l
//   columns: it forms those L_ij and applies -L_ij U_j* to the row, one
//   thread per U block, locating each block column in the target row by a
//   binary search over the row's columns staged in shared memory.  Pivots of
//   one level never update each other's rows, and each target row is owned
//   by one block, so no atomics are needed.  Dense trailing separators are
//   thus updated by all their remaining rows in parallel at every level;
// * solves use one warp per row on wide levels and one 256-thread block per
//   row on narrow levels (the long rows of the dense tail), with nrhs
//   right-hand sides stored row-major (row, dof, rhs).
#include "a2ds_internal.h"
#include "ilu.h"

namespace a2ds {

constexpr int FACTOR_SMEM_COLS = 10240;  // column indices staged per target row
constexpr int NARROW_LEVEL = 48;         // levels with fewer rows solve block-per-row

template <typename T>
__device__ __forceinline__ int d_inv6(const T *A, T *Ainv) {
  T M[36], I[36];
#pragma unroll
  for (int k = 0; k < 36; k++) {
    M[k] = A[k];
    I[k] = (k % 7 == 0) ? T(1) : T(0);
  }
  int fail = 0;
#pragma unroll
  for (int c = 0; c < 6; c++) {
    int p = c;
    T best = fabs(M[6 * c + c]);
#pragma unroll
    for (int r = c + 1; r < 6; r++) {
      T v = fabs(M[6 * r + c]);
      if (v > best) {
        best = v;
        p = r;
      }
    }
    if (best == T(0)) {
      fail = c + 1;
      break;
    }
    if (p != c) {
#pragma unroll
      for (int k = 0; k < 6; k++) {
        T t = M[6 * c + k];
        M[6 * c + k] = M[6 * p + k];
        M[6 * p + k] = t;
        t = I[6 * c + k];
        I[6 * c + k] = I[6 * p + k];
        I[6 * p + k] = t;
      }
    }
    T inv = T(1) / M[6 * c + c];
#pragma unroll
    for (int k = 0; k < 6; k++) {
      M[6 * c + k] *= inv;
      I[6 * c + k] *= inv;
    }
#pragma unroll
    for (int r = 0; r < 6; r++) {
      if (r == c) continue;
      T f = M[6 * r + c];
#pragma unroll
      for (int k = 0; k < 6; k++) {
        M[6 * r + k] -= f * M[6 * c + k];
        I[6 * r + k] -= f * I[6 * c + k];
      }
    }
  }
#pragma unroll
  for (int k = 0; k < 36; k++) Ainv[k] = I[k];
  return fail;
}

// Copy the values of A (+ alpha2 A2) into the factor pattern, zero elsewhere.
template <typename T>
__global__ void k_scatter_into_factor(int n, const int *__restrict__ rowp,
                                      const int *__restrict__ cols, const double *__restrict__ A,
                                      const double *__restrict__ A2, double alpha2,
                                      const int *__restrict__ frowp, const int *__restrict__ fcols,
                                      T *__restrict__ F) {
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (warp >= n) return;
  const int i = warp;
  const int fs = frowp[i], fe = frowp[i + 1];
  for (int idx = lane; idx < (fe - fs) * 36; idx += 32) F[(size_t)fs * 36 + idx] = T(0);
  __syncwarp();
  const int s = rowp[i], e = rowp[i + 1];
  for (int jp = s; jp < e; jp++) {
    const int c = cols[jp];
    int lo = fs, hi = fe - 1;
    while (lo < hi) {
      int mid = (lo + hi) >> 1;
      if (fcols[mid] < c)
        lo = mid + 1;
      else
        hi = mid;
    }
    for (int k = lane; k < 36; k += 32) {
      double v = A[(size_t)jp * 36 + k];
      if (A2) v += alpha2 * A2[(size_t)jp * 36 + k];
      F[(size_t)lo * 36 + k] = T(v);
    }
  }
}

template <typename T>
__global__ void k_factor_pivot(const int *__restrict__ rows, int nrows,
                               const int *__restrict__ fdiag, T *__restrict__ F,
                               int *__restrict__ status) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= nrows) return;
  const int j = rows[r];
  T *D = F + (size_t)fdiag[j] * 36;
  T inv[36];
  if (d_inv6<T>(D, inv)) atomicMax(status, j + 1);
#pragma unroll
  for (int k = 0; k < 36; k++) D[k] = inv[k];
}

template <typename T>
__global__ void __launch_bounds__(128) k_factor_update(
    const int *__restrict__ task_row, const int *__restrict__ task_ptr,
    const int *__restrict__ task_jp, int ntasks, const int *__restrict__ frowp,
    const int *__restrict__ fcols, const int *__restrict__ fdiag, T *__restrict__ F) {
  extern __shared__ int s_cols[];
  __shared__ T Lij[36];
  const int t = blockIdx.x;
  if (t >= ntasks) return;
  const int i = task_row[t];
  const int rs = frowp[i], re = frowp[i + 1], len = re - rs;
  const bool staged = len <= FACTOR_SMEM_COLS;
  if (staged)
    for (int k = threadIdx.x; k < len; k += blockDim.x) s_cols[k] = fcols[rs + k];
  __syncthreads();
  const int *colsrc = staged ? s_cols : fcols + rs;
  for (int q = task_ptr[t]; q < task_ptr[t + 1]; q++) {
    const int jp = task_jp[q];
    const int j = fcols[jp];
    T *Aij = F + (size_t)jp * 36;
    T v = 0;
    if (threadIdx.x < 36) {
      const T *Dinv = F + (size_t)fdiag[j] * 36;
      const int a = threadIdx.x / 6, b = threadIdx.x % 6;
#pragma unroll
      for (int k = 0; k < 6; k++) v += Aij[6 * a + k] * Dinv[6 * k + b];
    }
    __syncthreads();
    if (threadIdx.x < 36) {
      Aij[threadIdx.x] = v;
      Lij[threadIdx.x] = v;
    }
    __syncthreads();
    const int us = fdiag[j] + 1, ue = frowp[j + 1];
    const int lo0 = jp + 1 - rs;
    for (int pu = us + threadIdx.x; pu < ue; pu += blockDim.x) {
      const int c = fcols[pu];
      int lo = lo0, hi = len - 1;
      while (lo < hi) {
        int mid = (lo + hi) >> 1;
        if (colsrc[mid] < c)
          lo = mid + 1;
        else
          hi = mid;
      }
      if (lo < len && colsrc[lo] == c) {
        const T *U = F + (size_t)pu * 36;
        T *Aik = F + (size_t)(rs + lo) * 36;
        T u[36];
#pragma unroll
        for (int k = 0; k < 36; k++) u[k] = U[k];
#pragma unroll
        for (int a = 0; a < 6; a++) {
#pragma unroll
          for (int b = 0; b < 6; b++) {
            T s = 0;
#pragma unroll
            for (int k = 0; k < 6; k++) s += Lij[6 * a + k] * u[6 * k + b];
            Aik[6 * a + b] -= s;
          }
        }
      }
    }
    __syncthreads();
  }
}

// ---------------------------------------------------------------- solves
// Forward substitution, one warp per row: y_i = x_i - sum_{k<diag} L_ik y_k
template <typename T, typename TV>
__global__ void __launch_bounds__(256) k_lower_warp(const int *__restrict__ rows, int nrows,
                                                    const int *__restrict__ frowp,
                                                    const int *__restrict__ fcols,
                                                    const int *__restrict__ fdiag,
                                                    const T *__restrict__ F, const TV *x, TV *y,
                                                    int nrhs) {
  __shared__ TV part[8][30];
  const int wib = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int wr = blockIdx.x * 8 + wib;
  const bool live = wr < nrows;
  const int i = live ? rows[wr] : 0;
  const int g = lane / 6, ii = lane - 6 * (lane / 6);
  for (int rhs = 0; rhs < nrhs; rhs++) {
    TV acc = 0;
    if (live && lane < 30) {
      const int s = frowp[i], e = fdiag[i];
      for (int k = s + g; k < e; k += 5) {
        const T *a = F + (size_t)k * 36 + 6 * ii;
        const TV *yv = y + (size_t)fcols[k] * 6 * nrhs + rhs;
#pragma unroll
        for (int c = 0; c < 6; c++) acc += (TV)a[c] * yv[c * nrhs];
      }
    }
    if (lane < 30) part[wib][lane] = acc;
    __syncwarp();
    if (live && lane < 6) {
      TV v = part[wib][lane] + part[wib][lane + 6] + part[wib][lane + 12] + part[wib][lane + 18] +
             part[wib][lane + 24];
      const size_t o = ((size_t)i * 6 + lane) * nrhs + rhs;
      y[o] = x[o] - v;
    }
    __syncwarp();
  }
}

// Backward substitution, one warp per row: y_i = D_i^{-1}(y_i - sum U_ik y_k)
template <typename T, typename TV>
__global__ void __launch_bounds__(256) k_upper_warp(const int *__restrict__ rows, int nrows,
                                                    const int *__restrict__ frowp,
                                                    const int *__restrict__ fcols,
                                                    const int *__restrict__ fdiag,
                                                    const T *__restrict__ F, TV *y, int nrhs) {
  __shared__ TV part[8][30];
  __shared__ TV z[8][6];
  const int wib = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int wr = blockIdx.x * 8 + wib;
  const bool live = wr < nrows;
  const int i = live ? rows[wr] : 0;
  const int g = lane / 6, ii = lane - 6 * (lane / 6);
  for (int rhs = 0; rhs < nrhs; rhs++) {
    TV acc = 0;
    if (live && lane < 30) {
      const int s = fdiag[i] + 1, e = frowp[i + 1];
      for (int k = s + g; k < e; k += 5) {
        const T *a = F + (size_t)k * 36 + 6 * ii;
        const TV *yv = y + (size_t)fcols[k] * 6 * nrhs + rhs;
#pragma unroll
        for (int c = 0; c < 6; c++) acc += (TV)a[c] * yv[c * nrhs];
      }
    }
    if (lane < 30) part[wib][lane] = acc;
    __syncwarp();
    if (live && lane < 6) {
      TV v = part[wib][lane] + part[wib][lane + 6] + part[wib][lane + 12] + part[wib][lane + 18] +
             part[wib][lane + 24];
      z[wib][lane] = y[((size_t)i * 6 + lane) * nrhs + rhs] - v;
    }
    __syncwarp();
    if (live && lane < 6) {
      const T *Dinv = F + (size_t)fdiag[i] * 36 + 6 * lane;
      TV v = 0;
#pragma unroll
      for (int c = 0; c < 6; c++) v += (TV)Dinv[c] * z[wib][c];
      y[((size_t)i * 6 + lane) * nrhs + rhs] = v;
    }
    __syncwarp();
  }
}

// Long rows: one 256-thread block per row; 42 groups of six threads stride
// over the row's blocks, partial sums reduced in shared memory.
template <typename T, typename TV, bool UPPER>
__global__ void __launch_bounds__(256) k_tri_block(const int *__restrict__ rows, int nrows,
                                                   const int *__restrict__ frowp,
                                                   const int *__restrict__ fcols,
                                                   const int *__restrict__ fdiag,
                                                   const T *__restrict__ F, const TV *x, TV *y,
                                                   int nrhs) {
  __shared__ TV part[256];
  __shared__ TV z[6];
  const int r = blockIdx.x;
  if (r >= nrows) return;
  const int i = rows[r];
  const int t = threadIdx.x;
  const int g = t / 6, ii = t - 6 * (t / 6);
  const int s = UPPER ? fdiag[i] + 1 : frowp[i];
  const int e = UPPER ? frowp[i + 1] : fdiag[i];
  for (int rhs = 0; rhs < nrhs; rhs++) {
    TV acc = 0;
    if (t < 252) {
      for (int k = s + g; k < e; k += 42) {
        const T *a = F + (size_t)k * 36 + 6 * ii;
        const TV *yv = y + (size_t)fcols[k] * 6 * nrhs + rhs;
#pragma unroll
        for (int c = 0; c < 6; c++) acc += (TV)a[c] * yv[c * nrhs];
      }
    }
    part[t] = acc;
    __syncthreads();
    // reduce the 42 groups: threads 0..5 sum their row
    if (t < 6) {
      TV v = 0;
      for (int gg = 0; gg < 42; gg++) v += part[6 * gg + t];
      const size_t o = ((size_t)i * 6 + t) * nrhs + rhs;
      if (UPPER)
        z[t] = y[o] - v;
      else
        y[o] = x[o] - v;
    }
    __syncthreads();
    if (UPPER && t < 6) {
      const T *Dinv = F + (size_t)fdiag[i] * 36 + 6 * t;
      TV v = 0;
#pragma unroll
      for (int c = 0; c < 6; c++) v += (TV)Dinv[c] * z[c];
      y[((size_t)i * 6 + t) * nrhs + rhs] = v;
    }
    __syncthreads();
  }
}

// ------------------------------------------------------ dense-tail solves
// Rows [s, n) (the trailing separators, where levels hold a handful of long
// rows) are solved column-oriented: once a tail pivot's value is final its
// column is pushed into every later row in parallel (one thread per block
// entry, atomic adds because pivots of one level may share target rows).

// Pull the head part of every tail row: y_i = x_i - sum_{j < s} L_ij y_j.
template <typename T, typename TV>
__global__ void __launch_bounds__(256) k_tail_pull(int s, int d, const int *__restrict__ frowp,
                                                   const int *__restrict__ fcols,
                                                   const int *__restrict__ lsplit,
                                                   const T *__restrict__ F, const TV *x, TV *y,
                                                   int nrhs) {
  __shared__ TV part[8][30];
  const int wib = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int r = blockIdx.x * 8 + wib;
  const bool live = r < d;
  const int i = s + (live ? r : 0);
  const int g = lane / 6, ii = lane - 6 * (lane / 6);
  for (int rhs = 0; rhs < nrhs; rhs++) {
    TV acc = 0;
    if (live && lane < 30) {
      const int b = frowp[i], e = lsplit[r];
      for (int k = b + g; k < e; k += 5) {
        const T *a = F + (size_t)k * 36 + 6 * ii;
        const TV *yv = y + (size_t)fcols[k] * 6 * nrhs + rhs;
#pragma unroll
        for (int c = 0; c < 6; c++) acc += (TV)a[c] * yv[c * nrhs];
      }
    }
    if (lane < 30) part[wib][lane] = acc;
    __syncwarp();
    if (live && lane < 6) {
      TV v = part[wib][lane] + part[wib][lane + 6] + part[wib][lane + 12] + part[wib][lane + 18] +
             part[wib][lane + 24];
      const size_t o = ((size_t)i * 6 + lane) * nrhs + rhs;
      y[o] = x[o] - v;
    }
    __syncwarp();
  }
}

// Push the columns of one tail level.  Entry e: (target row, factor position,
// pivot row).  Lower: y_i -= L_ij y_j.  Upper: z_i -= U_ij D_j^{-1} z_j
// (the pivot's final value is formed on the fly; z_j itself is replaced by
// D_j^{-1} z_j only after all tail levels, by k_tail_finalize).
template <typename T, typename TV, bool UPPER>
__global__ void __launch_bounds__(256) k_tail_push(const int *__restrict__ erow,
                                                   const int *__restrict__ epos,
                                                   const int *__restrict__ ecol, int ne,
                                                   const int *__restrict__ fdiag,
                                                   const T *__restrict__ F, TV *y, int nrhs) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= ne) return;
  const int i = erow[e], p = epos[e], j = ecol[e];
  const T *A = F + (size_t)p * 36;
  for (int rhs = 0; rhs < nrhs; rhs++) {
    TV w[6];
#pragma unroll
    for (int b = 0; b < 6; b++) w[b] = y[((size_t)j * 6 + b) * nrhs + rhs];
    if (UPPER) {
      const T *Dinv = F + (size_t)fdiag[j] * 36;
      TV v[6];
#pragma unroll
      for (int a = 0; a < 6; a++) {
        TV sacc = 0;
#pragma unroll
        for (int b = 0; b < 6; b++) sacc += (TV)Dinv[6 * a + b] * w[b];
        v[a] = sacc;
      }
#pragma unroll
      for (int a = 0; a < 6; a++) w[a] = v[a];
    }
#pragma unroll
    for (int a = 0; a < 6; a++) {
      TV sacc = 0;
#pragma unroll
      for (int b = 0; b < 6; b++) sacc += (TV)A[6 * a + b] * w[b];
      atomicAdd(&y[((size_t)i * 6 + a) * nrhs + rhs], -sacc);
    }
  }
}

// y_j = D_j^{-1} z_j for every tail row (after the upper tail pushes).
template <typename T, typename TV>
__global__ void k_tail_finalize(int s, int d, const int *__restrict__ fdiag,
                                const T *__restrict__ F, TV *y, int nrhs) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= d) return;
  const int j = s + r;
  const T *Dinv = F + (size_t)fdiag[j] * 36;
  for (int rhs = 0; rhs < nrhs; rhs++) {
    TV z[6];
#pragma unroll
    for (int b = 0; b < 6; b++) z[b] = y[((size_t)j * 6 + b) * nrhs + rhs];
#pragma unroll
    for (int a = 0; a < 6; a++) {
      TV v = 0;
#pragma unroll
      for (int b = 0; b < 6; b++) v += (TV)Dinv[6 * a + b] * z[b];
      y[((size_t)j * 6 + a) * nrhs + rhs] = v;
    }
  }
}

// ------------------------------------------------------------ launchers
template <typename T>
int factor_scatter(int n, const int *rowp, const int *cols, const double *A, const double *A2,
                   double alpha2, const int *frowp, const int *fcols, T *F, cudaStream_t s) {
  k_scatter_into_factor<T><<<(n * 32 + 255) / 256, 256, 0, s>>>(n, rowp, cols, A, A2, alpha2,
                                                               frowp, fcols, F);
  A2DS_CUDA_TRY(cudaGetLastError());
  return 0;
}

template <typename T>
int factor_levels(const Factor &f, T *F, int *status, cudaStream_t s, long long *launches) {
  const LevelSchedule &L = f.flv;
  static bool configured = false;
  const int smem = FACTOR_SMEM_COLS * (int)sizeof(int);
  if (!configured) {
    A2DS_CUDA_TRY(cudaFuncSetAttribute(k_factor_update<T>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
    configured = true;
  }
  for (int lv = 0; lv < L.nlevels; lv++) {
    const int cnt = L.ptr[lv + 1] - L.ptr[lv];
    k_factor_pivot<T><<<(cnt + 127) / 128, 128, 0, s>>>(L.d_rows.p + L.ptr[lv], cnt,
                                                        f.d_fdiag.p, F, status);
    const int t0 = f.task_level_ptr[lv], nt = f.task_level_ptr[lv + 1] - t0;
    if (nt > 0) {
      k_factor_update<T><<<nt, 128, smem, s>>>(f.d_task_row.p + t0, f.d_task_ptr.p + t0,
                                               f.d_task_jp.p, nt, f.d_frowp.p, f.d_fcols.p,
                                               f.d_fdiag.p, F);
    }
    if (launches) *launches += 1 + (nt > 0);
  }
  A2DS_CUDA_TRY(cudaGetLastError());
  return 0;
}

template <typename T, typename TV>
int solve_levels(const Factor &f, const T *F, const TV *x, TV *y, int nrhs, cudaStream_t s,
                 long long *launches) {
  const LevelSchedule &Lo = f.lower, &Up = f.upper;
  long long nl = 0;
  for (int lv = 0; lv < Lo.nlevels; lv++) {
    const int cnt = Lo.ptr[lv + 1] - Lo.ptr[lv];
    if (cnt < NARROW_LEVEL)
      k_tri_block<T, TV, false><<<cnt, 256, 0, s>>>(Lo.d_rows.p + Lo.ptr[lv], cnt, f.d_frowp.p,
                                                    f.d_fcols.p, f.d_fdiag.p, F, x, y, nrhs);
    else
      k_lower_warp<T, TV><<<(cnt + 7) / 8, 256, 0, s>>>(Lo.d_rows.p + Lo.ptr[lv], cnt,
                                                        f.d_frowp.p, f.d_fcols.p, f.d_fdiag.p, F,
                                                        x, y, nrhs);
    nl++;
  }
  const int ts = f.tail_s, d = f.n - f.tail_s;
  if (d > 0) {
    k_tail_pull<T, TV><<<(d + 7) / 8, 256, 0, s>>>(ts, d, f.d_frowp.p, f.d_fcols.p, f.d_lsplit.p,
                                                   F, x, y, nrhs);
    nl++;
    for (size_t lv = 0; lv + 1 < f.tl_ptr.size(); lv++) {
      const int e0 = f.tl_ptr[lv], ne = f.tl_ptr[lv + 1] - e0;
      if (ne <= 0) continue;
      k_tail_push<T, TV, false><<<(ne + 255) / 256, 256, 0, s>>>(
          f.d_tl_row.p + e0, f.d_tl_pos.p + e0, f.d_tl_col.p + e0, ne, f.d_fdiag.p, F, y, nrhs);
      nl++;
    }
    for (size_t lv = 0; lv + 1 < f.tu_ptr.size(); lv++) {
      const int e0 = f.tu_ptr[lv], ne = f.tu_ptr[lv + 1] - e0;
      if (ne <= 0) continue;
      k_tail_push<T, TV, true><<<(ne + 255) / 256, 256, 0, s>>>(
          f.d_tu_row.p + e0, f.d_tu_pos.p + e0, f.d_tu_col.p + e0, ne, f.d_fdiag.p, F, y, nrhs);
      nl++;
    }
    k_tail_finalize<T, TV><<<(d + 127) / 128, 128, 0, s>>>(ts, d, f.d_fdiag.p, F, y, nrhs);
    nl++;
  }
  for (int lv = 0; lv < Up.nlevels; lv++) {
    const int cnt = Up.ptr[lv + 1] - Up.ptr[lv];
    if (cnt < NARROW_LEVEL)
      k_tri_block<T, TV, true><<<cnt, 256, 0, s>>>(Up.d_rows.p + Up.ptr[lv], cnt, f.d_frowp.p,
                                                   f.d_fcols.p, f.d_fdiag.p, F, y, y, nrhs);
    else
      k_upper_warp<T, TV><<<(cnt + 7) / 8, 256, 0, s>>>(Up.d_rows.p + Up.ptr[lv], cnt,
                                                        f.d_frowp.p, f.d_fcols.p, f.d_fdiag.p, F,
                                                        y, nrhs);
  }
  if (launches) *launches += nl + Up.nlevels;
  A2DS_CUDA_TRY(cudaGetLastError());
  return 0;
}

template int factor_scatter<double>(int, const int *, const int *, const double *, const double *,
                                    double, const int *, const int *, double *, cudaStream_t);
template int factor_scatter<float>(int, const int *, const int *, const double *, const double *,
                                   double, const int *, const int *, float *, cudaStream_t);
template int factor_levels<double>(const Factor &, double *, int *, cudaStream_t, long long *);
template int factor_levels<float>(const Factor &, float *, int *, cudaStream_t, long long *);
template int solve_levels<double, double>(const Factor &, const double *, const double *, double *,
                                          int, cudaStream_t, long long *);
template int solve_levels<float, float>(const Factor &, const float *, const float *, float *, int,
                                        cudaStream_t, long long *);

// ------------------------------------------------------------- host side
void build_levels(int n, const std::vector<int> &frowp, const std::vector<int> &fcols,
                  const std::vector<int> &fdiag, bool upper, LevelSchedule &L,
                  std::vector<int> *level_of) {
  std::vector<int> lev(n, 0);
  int maxlev = 0;
  if (!upper) {
    for (int i = 0; i < n; i++) {
      int l = 0;
      for (int k = frowp[i]; k < fdiag[i]; k++) l = std::max(l, lev[fcols[k]] + 1);
      lev[i] = l;
      maxlev = std::max(maxlev, l);
    }
  } else {
    for (int i = n - 1; i >= 0; i--) {
      int l = 0;
      for (int k = fdiag[i] + 1; k < frowp[i + 1]; k++) l = std::max(l, lev[fcols[k]] + 1);
      lev[i] = l;
      maxlev = std::max(maxlev, l);
    }
  }
  L.nlevels = n ? maxlev + 1 : 0;
  L.ptr.assign(L.nlevels + 1, 0);
  for (int i = 0; i < n; i++) L.ptr[lev[i] + 1]++;
  for (int l = 0; l < L.nlevels; l++) L.ptr[l + 1] += L.ptr[l];
  L.rows.resize(n);
  std::vector<int> fill(L.ptr.begin(), L.ptr.end() - 1);
  for (int i = 0; i < n; i++) L.rows[fill[lev[i]]++] = i;
  if (level_of) *level_of = lev;
}

// Update tasks of the right-looking schedule: for level l, one task per
// target row i holding the positions of its L entries whose column is a
// level-l row (in increasing column order).  Built with a counting sort of
// the L entries by column level; within a level, entries stay in row order.
void build_update_tasks(Factor &f, const std::vector<int> &lev) {
  const int n = f.n;
  const int nl = f.flv.nlevels;
  {
    // every U block of row j updates each row with an L entry in column j
    // (exact for the complete LU, an upper bound for ILU(k))
    double blocks = 0.0;
    for (int i = 0; i < n; i++)
      for (int k = f.frowp[i]; k < f.fdiag[i]; k++) {
        const int j = f.fcols[k];
        blocks += 1.0 + (double)(f.frowp[j + 1] - f.fdiag[j] - 1);
      }
    f.flop_count = 432.0 * (blocks + (double)n);
  }
  std::vector<long long> cnt(nl + 1, 0);
  for (int i = 0; i < n; i++)
    for (int k = f.frowp[i]; k < f.fdiag[i]; k++) cnt[lev[f.fcols[k]] + 1]++;
  for (int l = 0; l < nl; l++) cnt[l + 1] += cnt[l];
  std::vector<int> bucket_row(cnt[nl]), bucket_jp(cnt[nl]);
  std::vector<long long> fill(cnt.begin(), cnt.end() - 1);
  for (int i = 0; i < n; i++)
    for (int k = f.frowp[i]; k < f.fdiag[i]; k++) {
      long long p = fill[lev[f.fcols[k]]]++;
      bucket_row[p] = i;
      bucket_jp[p] = k;
    }
  f.task_level_ptr.assign(nl + 1, 0);
  f.task_row.clear();
  f.task_ptr.assign(1, 0);
  for (int l = 0; l < nl; l++) {
    for (long long p = cnt[l]; p < cnt[l + 1]; p++) {
      if (p == cnt[l] || bucket_row[p] != bucket_row[p - 1]) {
        if (p != cnt[l]) f.task_ptr.push_back((int)p);
        f.task_row.push_back(bucket_row[p]);
      }
    }
    if (cnt[l + 1] > cnt[l]) f.task_ptr.push_back((int)cnt[l + 1]);
    f.task_level_ptr[l + 1] = (int)f.task_row.size();
  }
  f.task_jp = std::move(bucket_jp);
}

// Rows are split at s = the smallest row index among rows of the first
// narrow factor level (fewer than `narrow` rows); rows [s, n) are the dense
// tail.  Head solves are row-oriented by levels; the tail pulls its head
// couplings once, then pushes columns level by level (lower), and pushes
// D^{-1}-scaled columns in reverse level order (upper) before the head
// upper solve pulls the final tail values.
void build_solve_schedule(Factor &f, const std::vector<int> &lev, int narrow) {
  const int n = f.n;
  const LevelSchedule &F = f.flv;
  int first_narrow = F.nlevels;
  for (int l = 0; l < F.nlevels; l++)
    if (F.ptr[l + 1] - F.ptr[l] < narrow) {
      first_narrow = l;
      break;
    }
  int s = n;
  for (int i = 0; i < n; i++)
    if (lev[i] >= first_narrow) {
      s = i;
      break;
    }
  f.tail_s = s;
  const int d = n - s;
  // head lower: factor levels restricted to rows < s (empty levels dropped)
  {
    LevelSchedule &L = f.lower;
    std::vector<int> cnt(F.nlevels + 1, 0);
    for (int i = 0; i < s; i++) cnt[lev[i]]++;
    std::vector<int> remap(F.nlevels, -1);
    int nl = 0;
    for (int l = 0; l < F.nlevels; l++)
      if (cnt[l]) remap[l] = nl++;
    L.nlevels = nl;
    L.ptr.assign(nl + 1, 0);
    for (int i = 0; i < s; i++) L.ptr[remap[lev[i]] + 1]++;
    for (int l = 0; l < nl; l++) L.ptr[l + 1] += L.ptr[l];
    L.rows.resize(s);
    std::vector<int> fill(L.ptr.begin(), L.ptr.end() - 1);
    for (int i = 0; i < s; i++) L.rows[fill[remap[lev[i]]]++] = i;
  }
  // head upper: levels counting only head columns (tail values are final)
  {
    std::vector<int> ul(s, 0);
    int maxl = 0;
    for (int i = s - 1; i >= 0; i--) {
      int l = 0;
      for (int k = f.fdiag[i] + 1; k < f.frowp[i + 1]; k++) {
        int c = f.fcols[k];
        if (c < s) l = std::max(l, ul[c] + 1);
      }
      ul[i] = l;
      maxl = std::max(maxl, l);
    }
    LevelSchedule &U = f.upper;
    U.nlevels = s ? maxl + 1 : 0;
    U.ptr.assign(U.nlevels + 1, 0);
    for (int i = 0; i < s; i++) U.ptr[ul[i] + 1]++;
    for (int l = 0; l < U.nlevels; l++) U.ptr[l + 1] += U.ptr[l];
    U.rows.resize(s);
    std::vector<int> fill(U.ptr.begin(), U.ptr.end() - 1);
    for (int i = 0; i < s; i++) U.rows[fill[ul[i]]++] = i;
  }
  f.lsplit.assign(d, 0);
  f.tl_ptr.assign(1, 0);
  f.tu_ptr.assign(1, 0);
  f.tl_row.clear();
  f.tl_pos.clear();
  f.tl_col.clear();
  f.tu_row.clear();
  f.tu_pos.clear();
  f.tu_col.clear();
  if (d == 0) return;
  // lower tail: levels within the tail, push lists grouped by pivot level
  std::vector<int> tl(d, 0);
  int maxl = 0;
  for (int i = s; i < n; i++) {
    int k = f.frowp[i];
    while (k < f.fdiag[i] && f.fcols[k] < s) k++;
    f.lsplit[i - s] = k;
    int l = 0;
    for (; k < f.fdiag[i]; k++) l = std::max(l, tl[f.fcols[k] - s] + 1);
    tl[i - s] = l;
    maxl = std::max(maxl, l);
  }
  {
    std::vector<long long> cnt(maxl + 2, 0);
    for (int i = s; i < n; i++)
      for (int k = f.lsplit[i - s]; k < f.fdiag[i]; k++) cnt[tl[f.fcols[k] - s] + 1]++;
    for (int l = 0; l <= maxl; l++) cnt[l + 1] += cnt[l];
    const long long tot = cnt[maxl + 1];
    f.tl_row.resize(tot);
    f.tl_pos.resize(tot);
    f.tl_col.resize(tot);
    std::vector<long long> fill(cnt.begin(), cnt.end() - 1);
    for (int i = s; i < n; i++)
      for (int k = f.lsplit[i - s]; k < f.fdiag[i]; k++) {
        long long p = fill[tl[f.fcols[k] - s]]++;
        f.tl_row[p] = i;
        f.tl_pos[p] = k;
        f.tl_col[p] = f.fcols[k];
      }
    f.tl_ptr.resize(maxl + 2);
    for (int l = 0; l <= maxl + 1; l++) f.tl_ptr[l] = (int)cnt[l];
  }
  // upper tail: reverse levels, push lists grouped by pivot (column) level
  std::vector<int> tu(d, 0);
  maxl = 0;
  for (int i = n - 1; i >= s; i--) {
    int l = 0;
    for (int k = f.fdiag[i] + 1; k < f.frowp[i + 1]; k++) l = std::max(l, tu[f.fcols[k] - s] + 1);
    tu[i - s] = l;
    maxl = std::max(maxl, l);
  }
  {
    std::vector<long long> cnt(maxl + 2, 0);
    for (int i = s; i < n; i++)
      for (int k = f.fdiag[i] + 1; k < f.frowp[i + 1]; k++) cnt[tu[f.fcols[k] - s] + 1]++;
    for (int l = 0; l <= maxl; l++) cnt[l + 1] += cnt[l];
    const long long tot = cnt[maxl + 1];
    f.tu_row.resize(tot);
    f.tu_pos.resize(tot);
    f.tu_col.resize(tot);
    std::vector<long long> fill(cnt.begin(), cnt.end() - 1);
    for (int i = s; i < n; i++)
      for (int k = f.fdiag[i] + 1; k < f.frowp[i + 1]; k++) {
        long long p = fill[tu[f.fcols[k] - s]]++;
        f.tu_row[p] = i;
        f.tu_pos[p] = k;
        f.tu_col[p] = f.fcols[k];
      }
    f.tu_ptr.resize(maxl + 2);
    for (int l = 0; l <= maxl + 1; l++) f.tu_ptr[l] = (int)cnt[l];
  }
}

int upload_schedules(Factor &f, cudaStream_t s) {
  int rc;
  if ((rc = f.flv.d_rows.upload(f.flv.rows.data(), f.flv.rows.size(), s))) return rc;
  if ((rc = f.lower.d_rows.upload(f.lower.rows.data(), f.lower.rows.size(), s))) return rc;
  if ((rc = f.upper.d_rows.upload(f.upper.rows.data(), f.upper.rows.size(), s))) return rc;
  if ((rc = f.d_task_row.upload(f.task_row.data(), f.task_row.size(), s))) return rc;
  if ((rc = f.d_task_ptr.upload(f.task_ptr.data(), f.task_ptr.size(), s))) return rc;
  if ((rc = f.d_task_jp.upload(f.task_jp.data(), f.task_jp.size(), s))) return rc;
  if ((rc = f.d_lsplit.upload(f.lsplit.data(), f.lsplit.size(), s))) return rc;
  if ((rc = f.d_tl_row.upload(f.tl_row.data(), f.tl_row.size(), s))) return rc;
  if ((rc = f.d_tl_pos.upload(f.tl_pos.data(), f.tl_pos.size(), s))) return rc;
  if ((rc = f.d_tl_col.upload(f.tl_col.data(), f.tl_col.size(), s))) return rc;
  if ((rc = f.d_tu_row.upload(f.tu_row.data(), f.tu_row.size(), s))) return rc;
  if ((rc = f.d_tu_pos.upload(f.tu_pos.data(), f.tu_pos.size(), s))) return rc;
  if ((rc = f.d_tu_col.upload(f.tu_col.data(), f.tu_col.size(), s))) return rc;
  return 0;
}

}  // namespace a2ds
