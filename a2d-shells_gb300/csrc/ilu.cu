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
// * the solves are in trisolve.cu.
#include "a2ds_internal.h"
#include "ilu.h"

namespace a2ds {

constexpr int FACTOR_SMEM_COLS = 10240;  // column indices staged per target row

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

// Invert the diagonal blocks of one level in place (6x6 Gauss-Jordan with
// partial pivoting, first maximum wins, as BMatComputeInverse).  Six lanes
// per block, one row of M and of the inverse each; pivot search, row swap
// and the pivot-row broadcast go through warp shuffles, so every value
// stays in registers and a level's blocks spread over many SMs (FP64
// throughput per SM is low on this part).  Arithmetic is the same
// operation sequence as the one-thread version, hence bit-identical.
template <typename T>
__global__ void __launch_bounds__(128) k_factor_pivot(const int *__restrict__ rows, int nrows,
                                                      const int *__restrict__ fdiag,
                                                      T *__restrict__ F, int *__restrict__ status) {
  const unsigned full = 0xffffffffu;
  const int lane = threadIdx.x & 31;
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (warp * 5 >= nrows) return;  // whole warp
  const int sub = lane / 6, r = lane - 6 * (lane / 6);
  const int idx = warp * 5 + sub;
  const bool live = sub < 5 && idx < nrows;
  const int base = sub < 5 ? 6 * sub : 0;
  const int j = live ? rows[idx] : 0;
  T *D = F + (size_t)(live ? fdiag[j] : 0) * 36;
  T m[6], v[6];
#pragma unroll
  for (int k = 0; k < 6; k++) {
    m[k] = live ? D[6 * r + k] : T(0);
    v[k] = (k == r) ? T(1) : T(0);
  }
  int fail = 0;
#pragma unroll
  for (int c = 0; c < 6; c++) {
    T bv = T(-1);
    int bp = c;
#pragma unroll
    for (int q = 0; q < 6; q++) {
      const T vq = __shfl_sync(full, fabs(m[c]), base + q);
      if (q >= c && vq > bv) {
        bv = vq;
        bp = q;
      }
    }
    if (bv == T(0) && !fail) fail = c + 1;  // singular; result unused
#pragma unroll
    for (int k = 0; k < 6; k++) {
      const T mc = __shfl_sync(full, m[k], base + c), mp = __shfl_sync(full, m[k], base + bp);
      const T vc = __shfl_sync(full, v[k], base + c), vp = __shfl_sync(full, v[k], base + bp);
      if (r == c) {
        m[k] = mp;
        v[k] = vp;
      } else if (r == bp) {
        m[k] = mc;
        v[k] = vc;
      }
    }
    const T piv = __shfl_sync(full, m[c], base + c);
    const T inv = piv != T(0) ? T(1) / piv : T(0);
    if (r == c) {
#pragma unroll
      for (int k = 0; k < 6; k++) {
        m[k] *= inv;
        v[k] *= inv;
      }
    }
    T pm[6], pv[6];
#pragma unroll
    for (int k = 0; k < 6; k++) {
      pm[k] = __shfl_sync(full, m[k], base + c);
      pv[k] = __shfl_sync(full, v[k], base + c);
    }
    if (r != c) {
      const T f = m[c];
#pragma unroll
      for (int k = 0; k < 6; k++) {
        m[k] -= f * pm[k];
        v[k] -= f * pv[k];
      }
    }
  }
  if (live) {
#pragma unroll
    for (int k = 0; k < 6; k++) D[6 * r + k] = v[k];
    if (fail && r == 0) atomicMax(status, j + 1);
  }
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
    k_factor_pivot<T><<<(cnt + 19) / 20, 128, 0, s>>>(L.d_rows.p + L.ptr[lv], cnt,
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

template int factor_scatter<double>(int, const int *, const int *, const double *, const double *,
                                    double, const int *, const int *, double *, cudaStream_t);
template int factor_scatter<float>(int, const int *, const int *, const double *, const double *,
                                   double, const int *, const int *, float *, cudaStream_t);
template int factor_levels<double>(const Factor &, double *, int *, cudaStream_t, long long *);
template int factor_levels<float>(const Factor &, float *, int *, cudaStream_t, long long *);

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
