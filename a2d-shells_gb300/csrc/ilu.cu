// Level-scheduled block ILU(k) / LU factorization and triangular solves for
// 6x6-block CSR matrices, FP64 or FP32.
//
// Numerics follow BCSRMatFactor6 (src/bpmat/BCSRMatFact6.cpp:946-1330):
// row i is eliminated left to right; each L block becomes
// L_ij = A_ij D_j^{-1} and updates the row with -L_ij U_jk on the pattern;
// the diagonal block is then replaced by its inverse (partial pivoting, as
// BMatComputeInverse, src/bpmat/BCSRMatMult.cpp:308).  The solves follow
// BCSRMatApplyLower6 / BCSRMatApplyUpper6 (src/bpmat/BCSRMatMult6.cpp:
// 319-416): unit-lower forward substitution, then backward substitution
// with the stored inverted diagonal.
//
// Parallel schedule (GPU-side): rows are grouped by dependency level on the
// host (a row's level is one more than the highest level among the rows its
// L (resp. U) part references); one launch per level, all rows of the level
// in parallel.  Factorization: one thread block per row; the block walks the
// row's L entries in order, forming L_ij with 36 threads and applying the
// U-row update with all threads (each update block located in row i by a
// binary search).  Solves: one warp per row, five groups of six lanes, the
// same dot-product layout as the SpMV kernel, with nrhs right-hand sides
// stored row-major (row, dof, rhs).
#include "a2ds_internal.h"
#include "ilu.h"

namespace a2ds {

template <typename T>
__device__ __forceinline__ int d_inv6(const T *A, T *Ainv) {
  // Gauss-Jordan with partial pivoting on a local copy
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

// Copy the values of A (pattern rowp/cols) into the factor pattern
// (frowp/fcols), zero elsewhere; optionally converting to T.  One warp per row.
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
    // locate c in the factor row (sorted): binary search by every lane
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
__global__ void __launch_bounds__(128) k_factor_level(const int *__restrict__ rows, int nrows,
                                                      const int *__restrict__ frowp,
                                                      const int *__restrict__ fcols,
                                                      const int *__restrict__ fdiag,
                                                      T *__restrict__ F, int *__restrict__ status) {
  __shared__ T d[36];
  __shared__ T D[36];
  const int r = blockIdx.x;
  if (r >= nrows) return;
  const int i = rows[r];
  const int rs = frowp[i], re = frowp[i + 1], di = fdiag[i];
  const int t = threadIdx.x;
  for (int jp = rs; jp < di; jp++) {
    const int j = fcols[jp];
    const T *Dj = F + (size_t)fdiag[j] * 36;
    T *Aij = F + (size_t)jp * 36;
    if (t < 36) {
      const int a = t / 6, b = t % 6;
      T v = 0;
#pragma unroll
      for (int k = 0; k < 6; k++) v += Aij[6 * a + k] * Dj[6 * k + b];
      d[t] = v;
    }
    __syncthreads();
    if (t < 36) Aij[t] = d[t];
    // row update over U part of row j: A_ik -= d * U_jk
    const int us = fdiag[j] + 1, ue = frowp[j + 1];
    const int nu = ue - us;
    for (int w = t; w < nu * 36; w += blockDim.x) {
      const int pu = us + w / 36, q = w % 36;
      const int c = fcols[pu];
      // binary search c in row i after jp
      int lo = jp + 1, hi = re - 1;
      while (lo < hi) {
        int mid = (lo + hi) >> 1;
        if (fcols[mid] < c)
          lo = mid + 1;
        else
          hi = mid;
      }
      if (lo < re && fcols[lo] == c) {
        const int a = q / 6, b = q % 6;
        const T *U = F + (size_t)pu * 36;
        T v = 0;
#pragma unroll
        for (int k = 0; k < 6; k++) v += d[6 * a + k] * U[6 * k + b];
        F[(size_t)lo * 36 + q] -= v;
      }
    }
    __syncthreads();
  }
  if (t < 36) D[t] = F[(size_t)di * 36 + t];
  __syncthreads();
  if (t == 0) {
    T inv[36];
    int fail = d_inv6<T>(D, inv);
    if (fail) atomicMax(status, i + 1);
#pragma unroll
    for (int k = 0; k < 36; k++) D[k] = inv[k];
  }
  __syncthreads();
  if (t < 36) F[(size_t)di * 36 + t] = D[t];
}

// Forward substitution for one level: y_i = x_i - sum_{k < diag} L_ik y_k
// (y may alias x).  Vectors hold nrhs right-hand sides, layout (row, dof, rhs).
template <typename T, typename TV>
__global__ void __launch_bounds__(256) k_lower_level(const int *__restrict__ rows, int nrows,
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

// Backward substitution for one level: y_i = D_i^{-1} (y_i - sum_{k > diag} U_ik y_k)
template <typename T, typename TV>
__global__ void __launch_bounds__(256) k_upper_level(const int *__restrict__ rows, int nrows,
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
int factor_levels(const LevelSchedule &L, const int *frowp, const int *fcols, const int *fdiag,
                  T *F, int *status, cudaStream_t s, long long *launches) {
  for (int lv = 0; lv < L.nlevels; lv++) {
    const int cnt = L.ptr[lv + 1] - L.ptr[lv];
    k_factor_level<T><<<cnt, 128, 0, s>>>(L.d_rows.p + L.ptr[lv], cnt, frowp, fcols, fdiag, F,
                                          status);
  }
  if (launches) *launches += L.nlevels;
  A2DS_CUDA_TRY(cudaGetLastError());
  return 0;
}

template <typename T, typename TV>
int solve_levels(const LevelSchedule &Lo, const LevelSchedule &Up, const int *frowp,
                 const int *fcols, const int *fdiag, const T *F, const TV *x, TV *y, int nrhs,
                 cudaStream_t s, long long *launches) {
  for (int lv = 0; lv < Lo.nlevels; lv++) {
    const int cnt = Lo.ptr[lv + 1] - Lo.ptr[lv];
    k_lower_level<T, TV><<<(cnt + 7) / 8, 256, 0, s>>>(Lo.d_rows.p + Lo.ptr[lv], cnt, frowp, fcols,
                                                      fdiag, F, x, y, nrhs);
  }
  for (int lv = 0; lv < Up.nlevels; lv++) {
    const int cnt = Up.ptr[lv + 1] - Up.ptr[lv];
    k_upper_level<T, TV><<<(cnt + 7) / 8, 256, 0, s>>>(Up.d_rows.p + Up.ptr[lv], cnt, frowp,
                                                      fcols, fdiag, F, y, nrhs);
  }
  if (launches) *launches += Lo.nlevels + Up.nlevels;
  A2DS_CUDA_TRY(cudaGetLastError());
  return 0;
}

template int factor_scatter<double>(int, const int *, const int *, const double *, const double *,
                                    double, const int *, const int *, double *, cudaStream_t);
template int factor_scatter<float>(int, const int *, const int *, const double *, const double *,
                                   double, const int *, const int *, float *, cudaStream_t);
template int factor_levels<double>(const LevelSchedule &, const int *, const int *, const int *,
                                   double *, int *, cudaStream_t, long long *);
template int factor_levels<float>(const LevelSchedule &, const int *, const int *, const int *,
                                  float *, int *, cudaStream_t, long long *);
template int solve_levels<double, double>(const LevelSchedule &, const LevelSchedule &,
                                          const int *, const int *, const int *, const double *,
                                          const double *, double *, int, cudaStream_t,
                                          long long *);
template int solve_levels<float, float>(const LevelSchedule &, const LevelSchedule &, const int *,
                                        const int *, const int *, const float *, const float *,
                                        float *, int, cudaStream_t, long long *);

// ------------------------------------------------------------- host side
void build_levels(int n, const std::vector<int> &frowp, const std::vector<int> &fcols,
                  const std::vector<int> &fdiag, bool upper, LevelSchedule &L) {
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
}

}  // namespace a2ds
