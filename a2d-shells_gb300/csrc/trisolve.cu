// Block triangular solves with the LU / ILU(k) factor for R right-hand
// sides at once, and CUDA-graph replay of a whole solve.
//
// Numerics follow BCSRMatApplyLower6 / BCSRMatApplyUpper6
// (src/bpmat/BCSRMatMult6.cpp:319-416): unit-lower forward substitution
// y_i = x_i - sum_{k<i} L_ik y_k, then backward substitution
// y_i = D_i^{-1} (y_i - sum_{k>i} U_ik y_k) with the stored inverse diagonal.
//
// Vectors hold R right-hand sides row-major: entry (row, dof, rhs) at
// (row * 6 + dof) * R + rhs, so one factor block is loaded once and applied
// to all R vectors.  Rows of the head (levels with many rows) are solved one
// warp per row (five 6-lane groups stride over the row's blocks), narrow
// levels one 256-thread block per row, the middle of the tail
// column-oriented (each final pivot pushes its column into later rows with
// FP64 atomics), and the trailing separator rows as one dense block, panel
// by panel.  solve_graph() captures the whole launch sequence once per
// (factor, x, y, R) and replays it.
#include "a2ds_internal.h"
#include "ilu.h"

namespace a2ds {


// Partial sums of sum_k F_k[ii][:] y[fcols[k]] over k = kb + g, kb + g + step, ...
template <typename T, typename TV, int R>
__device__ __forceinline__ void row_partial(int kb, int ke, int g, int step, int ii,
                                            const int *__restrict__ fcols,
                                            const T *__restrict__ F, const TV *y, TV (&acc)[R]) {
  for (int k = kb + g; k < ke; k += step) {
    const T *a = F + (size_t)k * 36 + 6 * ii;
    TV av[6];
#pragma unroll
    for (int c = 0; c < 6; c++) av[c] = (TV)a[c];
    const TV *yv = y + (size_t)fcols[k] * 6 * R;
#pragma unroll
    for (int c = 0; c < 6; c++)
#pragma unroll
      for (int r = 0; r < R; r++) acc[r] += av[c] * yv[c * R + r];
  }
}

// Forward substitution, one warp per row of a level.
template <typename T, typename TV, int R>
__global__ void __launch_bounds__(256) k_lower_warp(const int *__restrict__ rows, int nrows,
                                                    const int *__restrict__ frowp,
                                                    const int *__restrict__ fcols,
                                                    const int *__restrict__ fdiag,
                                                    const T *__restrict__ F, const TV *x, TV *y) {
  __shared__ TV part[8][30][R];
  const int wib = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int wr = blockIdx.x * 8 + wib;
  if (wr >= nrows) return;  // whole warp leaves together
  const int i = rows[wr];
  const int g = lane / 6, ii = lane - 6 * g;
  TV acc[R];
#pragma unroll
  for (int r = 0; r < R; r++) acc[r] = 0;
  if (lane < 30) row_partial<T, TV, R>(frowp[i], fdiag[i], g, 5, ii, fcols, F, y, acc);
  if (lane < 30)
#pragma unroll
    for (int r = 0; r < R; r++) part[wib][lane][r] = acc[r];
  __syncwarp();
  for (int o = lane; o < 6 * R; o += 32) {
    const int d = o / R, r = o - R * d;
    TV v = part[wib][d][r] + part[wib][d + 6][r] + part[wib][d + 12][r] + part[wib][d + 18][r] +
           part[wib][d + 24][r];
    const size_t idx = ((size_t)i * 6 + d) * R + r;
    y[idx] = x[idx] - v;
  }
}

// Backward substitution, one warp per row of a level.
template <typename T, typename TV, int R>
__global__ void __launch_bounds__(256) k_upper_warp(const int *__restrict__ rows, int nrows,
                                                    const int *__restrict__ frowp,
                                                    const int *__restrict__ fcols,
                                                    const int *__restrict__ fdiag,
                                                    const T *__restrict__ F, TV *y) {
  __shared__ TV part[8][30][R];
  __shared__ TV z[8][6][R];
  const int wib = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int wr = blockIdx.x * 8 + wib;
  if (wr >= nrows) return;
  const int i = rows[wr];
  const int g = lane / 6, ii = lane - 6 * g;
  TV acc[R];
#pragma unroll
  for (int r = 0; r < R; r++) acc[r] = 0;
  if (lane < 30) row_partial<T, TV, R>(fdiag[i] + 1, frowp[i + 1], g, 5, ii, fcols, F, y, acc);
  if (lane < 30)
#pragma unroll
    for (int r = 0; r < R; r++) part[wib][lane][r] = acc[r];
  __syncwarp();
  for (int o = lane; o < 6 * R; o += 32) {
    const int d = o / R, r = o - R * d;
    TV v = part[wib][d][r] + part[wib][d + 6][r] + part[wib][d + 12][r] + part[wib][d + 18][r] +
           part[wib][d + 24][r];
    z[wib][d][r] = y[((size_t)i * 6 + d) * R + r] - v;
  }
  __syncwarp();
  const T *Dinv = F + (size_t)fdiag[i] * 36;
  for (int o = lane; o < 6 * R; o += 32) {
    const int d = o / R, r = o - R * d;
    TV v = 0;
#pragma unroll
    for (int c = 0; c < 6; c++) v += (TV)Dinv[6 * d + c] * z[wib][c][r];
    y[((size_t)i * 6 + d) * R + r] = v;
  }
}

// Long rows of narrow levels: one 256-thread block per row, 42 groups of
// six threads stride over the row's blocks.
template <typename T, typename TV, int R, bool UPPER>
__global__ void __launch_bounds__(256) k_tri_block(const int *__restrict__ rows, int nrows,
                                                   const int *__restrict__ frowp,
                                                   const int *__restrict__ fcols,
                                                   const int *__restrict__ fdiag,
                                                   const T *__restrict__ F, const TV *x, TV *y) {
  __shared__ TV part[252][R];
  __shared__ TV z[6][R];
  const int rr = blockIdx.x;
  if (rr >= nrows) return;
  const int i = rows[rr];
  const int t = threadIdx.x;
  const int g = t / 6, ii = t - 6 * g;
  const int kb = UPPER ? fdiag[i] + 1 : frowp[i];
  const int ke = UPPER ? frowp[i + 1] : fdiag[i];
  if (t < 252) {
    TV acc[R];
#pragma unroll
    for (int r = 0; r < R; r++) acc[r] = 0;
    row_partial<T, TV, R>(kb, ke, g, 42, ii, fcols, F, y, acc);
#pragma unroll
    for (int r = 0; r < R; r++) part[t][r] = acc[r];
  }
  __syncthreads();
  for (int o = t; o < 6 * R; o += blockDim.x) {
    const int d = o / R, r = o - R * d;
    TV v = 0;
    for (int gg = 0; gg < 42; gg++) v += part[6 * gg + d][r];
    const size_t idx = ((size_t)i * 6 + d) * R + r;
    if (UPPER)
      z[d][r] = y[idx] - v;
    else
      y[idx] = x[idx] - v;
  }
  if (!UPPER) return;
  __syncthreads();
  const T *Dinv = F + (size_t)fdiag[i] * 36;
  for (int o = t; o < 6 * R; o += blockDim.x) {
    const int d = o / R, r = o - R * d;
    TV v = 0;
#pragma unroll
    for (int c = 0; c < 6; c++) v += (TV)Dinv[6 * d + c] * z[c][r];
    y[((size_t)i * 6 + d) * R + r] = v;
  }
}

// ------------------------------------------------------------ tail solves
// Rows [s, n) are the trailing separators, where levels hold a handful of
// long rows.  Their head couplings are pulled once; then, tail level by tail
// level, the columns of final pivots are pushed into the later rows.

// y_i = x_i - sum_{j < s} L_ij y_j for every tail row i (one warp per row).
template <typename T, typename TV, int R>
__global__ void __launch_bounds__(256) k_tail_pull(int s, int d, const int *__restrict__ frowp,
                                                   const int *__restrict__ fcols,
                                                   const int *__restrict__ lsplit,
                                                   const T *__restrict__ F, const TV *x, TV *y) {
  __shared__ TV part[8][30][R];
  const int wib = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int rr = blockIdx.x * 8 + wib;
  if (rr >= d) return;
  const int i = s + rr;
  const int g = lane / 6, ii = lane - 6 * g;
  TV acc[R];
#pragma unroll
  for (int r = 0; r < R; r++) acc[r] = 0;
  if (lane < 30) row_partial<T, TV, R>(frowp[i], lsplit[rr], g, 5, ii, fcols, F, y, acc);
  if (lane < 30)
#pragma unroll
    for (int r = 0; r < R; r++) part[wib][lane][r] = acc[r];
  __syncwarp();
  for (int o = lane; o < 6 * R; o += 32) {
    const int dd = o / R, r = o - R * dd;
    TV v = part[wib][dd][r] + part[wib][dd + 6][r] + part[wib][dd + 12][r] +
           part[wib][dd + 18][r] + part[wib][dd + 24][r];
    const size_t idx = ((size_t)i * 6 + dd) * R + r;
    y[idx] = x[idx] - v;
  }
}

// One tail level's column pushes; thread (entry e, rhs r).  Entry e is
// (target row i, factor position p, pivot row j).  PUSH_L: y_i -= L_ij y_j.
// PUSH_U: y_i -= U_ij D_j^{-1} y_j (y_j itself is scaled by D_j^{-1} only
// after all tail levels, by k_tail_finalize).  PUSH_U_FINAL: y_i -= U_ij y_j
// with y_j already final (dense-block columns).
enum { PUSH_L = 0, PUSH_U = 1, PUSH_U_FINAL = 2 };
template <typename T, typename TV, int R, int MODE>
__global__ void __launch_bounds__(256) k_tail_push(const int *__restrict__ erow,
                                                   const int *__restrict__ epos,
                                                   const int *__restrict__ ecol, int ne,
                                                   const int *__restrict__ fdiag,
                                                   const T *__restrict__ F, TV *y) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  const int e = t / R, r = t - R * (t / R);
  if (e >= ne) return;
  const int i = erow[e], p = epos[e], j = ecol[e];
  const T *A = F + (size_t)p * 36;
  TV w[6];
#pragma unroll
  for (int b = 0; b < 6; b++) w[b] = y[((size_t)j * 6 + b) * R + r];
  if (MODE == PUSH_U) {
    const T *Dinv = F + (size_t)fdiag[j] * 36;
    TV v[6];
#pragma unroll
    for (int a = 0; a < 6; a++) {
      TV acc = 0;
#pragma unroll
      for (int b = 0; b < 6; b++) acc += (TV)Dinv[6 * a + b] * w[b];
      v[a] = acc;
    }
#pragma unroll
    for (int a = 0; a < 6; a++) w[a] = v[a];
  }
#pragma unroll
  for (int a = 0; a < 6; a++) {
    TV acc = 0;
#pragma unroll
    for (int b = 0; b < 6; b++) acc += (TV)A[6 * a + b] * w[b];
    atomicAdd(&y[((size_t)i * 6 + a) * R + r], -acc);
  }
}

// y_j = D_j^{-1} z_j for tail rows j in [s, s + d); thread (row, rhs).
template <typename T, typename TV, int R>
__global__ void k_tail_finalize(int s, int d, const int *__restrict__ fdiag,
                                const T *__restrict__ F, TV *y) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  const int rr = t / R, r = t - R * (t / R);
  if (rr >= d) return;
  const int j = s + rr;
  const T *Dinv = F + (size_t)fdiag[j] * 36;
  TV z[6];
#pragma unroll
  for (int b = 0; b < 6; b++) z[b] = y[((size_t)j * 6 + b) * R + r];
#pragma unroll
  for (int a = 0; a < 6; a++) {
    TV v = 0;
#pragma unroll
    for (int b = 0; b < 6; b++) v += (TV)Dinv[6 * a + b] * z[b];
    y[((size_t)j * 6 + a) * R + r] = v;
  }
}

// ------------------------------------------------------ dense trailing block
// The last dense_n block rows are solved as a dense (6 dense_n)^2 system,
// DENSE_PANEL block rows (PB6 unknowns) at a time: w = P_pp y_p with the
// precomputed inverse of the diagonal panel, then the rows beyond the panel
// (below it for L, above it for U) subtract M[rows, panel] w.  Two launches
// per panel instead of one per row, and the work of a panel is spread over
// the whole GPU.
constexpr int PB6 = 6 * DENSE_PANEL;

// Sum of v[r] over the warp for every r, spread over the lanes: halving
// exchanges (offsets 16, 8, ...) leave each lane one partial sum for RHS
// `rhs` (from its high lane bits), then the remaining offsets complete it;
// lanes with (lane & (32 / R - 1)) == 0 hold the R distinct totals.  R + 4
// shuffles per warp instead of 5 R.
template <typename TV, int R>
__device__ __forceinline__ TV warp_reduce_scatter(TV (&v)[R], int lane, int &rhs) {
  static_assert(R >= 1 && R <= 32 && (R & (R - 1)) == 0, "R must be a power of two <= 32");
  const unsigned full = 0xffffffffu;
  int base = 0;
#pragma unroll
  for (int h = R / 2, o = 16; h >= 1; h /= 2, o /= 2) {
    const bool up = (lane & o) != 0;
#pragma unroll
    for (int k = 0; k < h; k++) {
      const TV send = up ? v[k] : v[k + h];
      const TV keep = up ? v[k + h] : v[k];
      v[k] = keep + __shfl_xor_sync(full, send, o);
    }
    if (up) base += h;
  }
  TV sum = v[0];
#pragma unroll
  for (int o = 16 / R; o >= 1; o /= 2) sum += __shfl_xor_sync(full, sum, o);
  rhs = base;
  return sum;
}

// Stage a PB6 x R vector (row-major, [c][r]) in shared memory as [r][c], so
// that lanes reading consecutive c hit consecutive banks.
template <typename TV, int R>
__device__ __forceinline__ void stage_panel_vec(TV *sv, const TV *v) {
  for (int k = threadIdx.x; k < PB6 * R; k += blockDim.x) sv[(k % R) * PB6 + k / R] = v[k];
}

// acc[q][r] = sum_c row_q[c] sv[r][c] over this lane's columns (lane + 32 j).
template <typename T, typename TV, int R, int NQ>
__device__ __forceinline__ void panel_rows_dot(const T *const (&rows)[NQ], const TV *sv, int lane,
                                               TV (&acc)[NQ][R]) {
  T m[NQ][6];
#pragma unroll
  for (int q = 0; q < NQ; q++)
#pragma unroll
    for (int j = 0; j < 6; j++) m[q][j] = rows[q] ? rows[q][lane + 32 * j] : T(0);
#pragma unroll
  for (int q = 0; q < NQ; q++)
#pragma unroll
    for (int r = 0; r < R; r++) {
      TV s = 0;
#pragma unroll
      for (int j = 0; j < 6; j++) s += (TV)m[q][j] * sv[r * PB6 + lane + 32 * j];
      acc[q][r] = s;
    }
}

// w = P v, P = PB6 x PB6 row-major, v and w PB6 x R; one warp per row of P.
template <typename T, typename TV, int R>
__global__ void __launch_bounds__(256) k_dense_panel_apply(const T *__restrict__ P, const TV *v,
                                                           TV *__restrict__ w) {
  static_assert(PB6 == 6 * 32, "a panel row is six warp-wide segments");
  __shared__ TV sv[PB6 * R];
  stage_panel_vec<TV, R>(sv, v);
  __syncthreads();
  const int row = blockIdx.x * 8 + (threadIdx.x >> 5), lane = threadIdx.x & 31;
  if (row >= PB6) return;
  const T *rows[1] = {P + (size_t)row * PB6};
  TV acc[1][R];
  panel_rows_dot<T, TV, R, 1>(rows, sv, lane, acc);
  int rhs;
  const TV sum = warp_reduce_scatter<TV, R>(acc[0], lane, rhs);
  if ((lane & (32 / R - 1)) == 0) w[(size_t)row * R + rhs] = sum;
}

// Rows [r0, r0 + nrows) of the dense segment yD: y -= M[rows, c0 : c0 + PB6] w;
// CTA 0 also stores w as the panel's final values (yD rows c0 ..).  Each
// warp takes DENSE_ROWS_PER_WARP rows, two at a time (their twelve loads
// issued together); M is the dense block, leading dimension ld.
constexpr int DENSE_ROWS_PER_WARP = 4;
template <typename T, typename TV, int R>
__global__ void __launch_bounds__(256) k_dense_panel_update(const T *__restrict__ M, int ld,
                                                            int r0, int nrows, int c0,
                                                            const TV *__restrict__ w, TV *yD) {
  __shared__ TV sw[PB6 * R];
  stage_panel_vec<TV, R>(sw, w);
  if (blockIdx.x == 0)
    for (int k = threadIdx.x; k < PB6 * R; k += blockDim.x) yD[(size_t)c0 * R + k] = w[k];
  __syncthreads();
  const int warp = blockIdx.x * 8 + (threadIdx.x >> 5), lane = threadIdx.x & 31;
#pragma unroll 1
  for (int q = 0; q < DENSE_ROWS_PER_WARP; q += 2) {
    const int rr = warp * DENSE_ROWS_PER_WARP + q;
    if (rr >= nrows) break;
    const T *rows[2] = {M + (size_t)(r0 + rr) * ld + c0,
                        rr + 1 < nrows ? M + (size_t)(r0 + rr + 1) * ld + c0 : nullptr};
    TV acc[2][R];
    panel_rows_dot<T, TV, R, 2>(rows, sw, lane, acc);
#pragma unroll
    for (int d = 0; d < 2; d++) {
      int rhs;
      const TV sum = warp_reduce_scatter<TV, R>(acc[d], lane, rhs);
      if (rr + d < nrows && (lane & (32 / R - 1)) == 0)
        yD[(size_t)(r0 + rr + d) * R + rhs] -= sum;
    }
  }
}

// Copy the factor's blocks of the dense block rows into the dense array
// (zeroed beforehand); one warp per block row.
template <typename T>
__global__ void k_dense_scatter(int t0, int nd, const int *__restrict__ frowp,
                                const int *__restrict__ fcols, const T *__restrict__ F,
                                T *__restrict__ M) {
  const int rr = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (rr >= nd) return;
  const int i = t0 + rr, ld = 6 * nd;
  int k0 = frowp[i];
  const int k1 = frowp[i + 1];
  while (k0 < k1 && fcols[k0] < t0) k0++;  // columns are sorted
  const int nb = k1 - k0;
  for (int idx = lane; idx < nb * 36; idx += 32) {
    const int k = k0 + idx / 36, e = idx % 36;
    const int a = e / 6, b = e % 6;
    M[(size_t)(6 * rr + a) * ld + 6 * (fcols[k] - t0) + b] = F[(size_t)k * 36 + e];
  }
}

// Inverse of every diagonal panel, thread (panel, column c).  Lower: the
// unit block-lower L_pp, forward substitution on e_c.  Upper: D + U_pp with
// the stored D_i^{-1}: z_i = D_i^{-1} (e_c - sum_{j > i} U_ij z_j), backward.
template <typename T, bool UPPER>
__global__ void k_dense_panel_inverse(const T *__restrict__ M, int ld, int npanels,
                                      T *__restrict__ Pinv) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  const int p = t / PB6, c = t % PB6;
  if (p >= npanels) return;
  const T *Mp = M + (size_t)p * PB6 * ld + (size_t)p * PB6;
  T *X = Pinv + (size_t)p * PB6 * PB6;
  if (!UPPER) {
    for (int i = 0; i < DENSE_PANEL; i++)
      for (int a = 0; a < 6; a++) {
        const int r = 6 * i + a;
        T v = (r == c) ? T(1) : T(0);
        for (int q = 0; q < 6 * i; q++) v -= Mp[(size_t)r * ld + q] * X[(size_t)q * PB6 + c];
        X[(size_t)r * PB6 + c] = v;
      }
  } else {
    for (int i = DENSE_PANEL - 1; i >= 0; i--) {
      T z[6];
      for (int a = 0; a < 6; a++) {
        const int r = 6 * i + a;
        T v = (r == c) ? T(1) : T(0);
        for (int q = 6 * (i + 1); q < PB6; q++) v -= Mp[(size_t)r * ld + q] * X[(size_t)q * PB6 + c];
        z[a] = v;
      }
      for (int a = 0; a < 6; a++) {
        T v = 0;
        for (int b = 0; b < 6; b++) v += Mp[(size_t)(6 * i + a) * ld + 6 * i + b] * z[b];
        X[(size_t)(6 * i + a) * PB6 + c] = v;
      }
    }
  }
}

template <typename T>
struct DenseBufs;
template <>
struct DenseBufs<double> {
  static double *M(const Factor &f) { return f.dense64.p; }
  static double *L(const Factor &f) { return f.pinvL64.p; }
  static double *U(const Factor &f) { return f.pinvU64.p; }
  static double *W(const Factor &f) { return f.dwork64.p; }
};
template <>
struct DenseBufs<float> {
  static float *M(const Factor &f) { return f.dense32.p; }
  static float *L(const Factor &f) { return f.pinvL32.p; }
  static float *U(const Factor &f) { return f.pinvU32.p; }
  static float *W(const Factor &f) { return f.dwork32.p; }
};

int dense_alloc(Factor &f) {
  if (f.dense_n <= 0) return 0;
  const size_t nd6 = (size_t)6 * f.dense_n, np = (size_t)f.dense_n / DENSE_PANEL;
  int rc;
  if (f.precision == 32) {
    if ((rc = f.dense32.alloc(nd6 * nd6)) || (rc = f.pinvL32.alloc(np * PB6 * PB6)) ||
        (rc = f.pinvU32.alloc(np * PB6 * PB6)) || (rc = f.dwork32.alloc((size_t)PB6 * 16)))
      return rc;
  } else {
    if ((rc = f.dense64.alloc(nd6 * nd6)) || (rc = f.pinvL64.alloc(np * PB6 * PB6)) ||
        (rc = f.pinvU64.alloc(np * PB6 * PB6)) || (rc = f.dwork64.alloc((size_t)PB6 * 16)))
      return rc;
  }
  return 0;
}

template <typename T>
static int dense_build_t(Factor &f, const T *F, cudaStream_t s, long long *launches) {
  const int nd = f.dense_n, ld = 6 * nd, np = nd / DENSE_PANEL;
  T *M = DenseBufs<T>::M(f);
  A2DS_CUDA_TRY(cudaMemsetAsync(M, 0, (size_t)ld * ld * sizeof(T), s));
  k_dense_scatter<T><<<(nd * 32 + 255) / 256, 256, 0, s>>>(f.dense_t0, nd, f.d_frowp.p,
                                                           f.d_fcols.p, F, M);
  k_dense_panel_inverse<T, false><<<(np * PB6 + 127) / 128, 128, 0, s>>>(M, ld, np,
                                                                          DenseBufs<T>::L(f));
  k_dense_panel_inverse<T, true><<<(np * PB6 + 127) / 128, 128, 0, s>>>(M, ld, np,
                                                                         DenseBufs<T>::U(f));
  if (launches) *launches += 3;
  A2DS_CUDA_TRY(cudaGetLastError());
  return 0;
}

int dense_build(Factor &f, const void *F, cudaStream_t s, long long *launches) {
  if (f.dense_n <= 0) return 0;
  if (f.precision == 32) return dense_build_t<float>(f, (const float *)F, s, launches);
  return dense_build_t<double>(f, (const double *)F, s, launches);
}

static int dense_update_grid(int nrows) {
  const int per_cta = 8 * DENSE_ROWS_PER_WARP;
  return std::max(1, (nrows + per_cta - 1) / per_cta);
}

template <typename T, typename TV, int R>
static void dense_solve(const Factor &f, TV *y, cudaStream_t s, long long &nl) {
  const int nd = f.dense_n, ld = 6 * nd, np = nd / DENSE_PANEL;
  const T *M = DenseBufs<T>::M(f);
  TV *w = DenseBufs<TV>::W(f);
  TV *yD = y + (size_t)f.dense_t0 * 6 * R;
  for (int p = 0; p < np; p++) {  // L: forward
    k_dense_panel_apply<T, TV, R><<<PB6 / 8, 256, 0, s>>>(
        DenseBufs<T>::L(f) + (size_t)p * PB6 * PB6, yD + (size_t)p * PB6 * R, w);
    const int r0 = (p + 1) * PB6, nr = ld - r0;
    k_dense_panel_update<T, TV, R><<<dense_update_grid(nr), 256, 0, s>>>(M, ld, r0, nr,
                                                                         p * PB6, w, yD);
    nl += 2;
  }
  for (int p = np - 1; p >= 0; p--) {  // D + U: backward
    k_dense_panel_apply<T, TV, R><<<PB6 / 8, 256, 0, s>>>(
        DenseBufs<T>::U(f) + (size_t)p * PB6 * PB6, yD + (size_t)p * PB6 * R, w);
    const int nr = p * PB6;
    k_dense_panel_update<T, TV, R><<<dense_update_grid(nr), 256, 0, s>>>(M, ld, 0, nr,
                                                                         p * PB6, w, yD);
    nl += 2;
  }
}

// ------------------------------------------------------------ launchers
template <typename T, typename TV, int R>
static int solve_levels_r(const Factor &f, const T *F, const TV *x, TV *y, cudaStream_t s,
                          long long *launches) {
  const LevelSchedule &Lo = f.lower, &Up = f.upper;
  long long nl = 0;
  for (int lv = 0; lv < Lo.nlevels; lv++) {
    const int cnt = Lo.ptr[lv + 1] - Lo.ptr[lv];
    if (f.lower_cta[lv])
      k_tri_block<T, TV, R, false><<<cnt, 256, 0, s>>>(Lo.d_rows.p + Lo.ptr[lv], cnt,
                                                       f.d_frowp.p, f.d_fcols.p, f.d_fdiag.p, F,
                                                       x, y);
    else
      k_lower_warp<T, TV, R><<<(cnt + 7) / 8, 256, 0, s>>>(Lo.d_rows.p + Lo.ptr[lv], cnt,
                                                           f.d_frowp.p, f.d_fcols.p,
                                                           f.d_fdiag.p, F, x, y);
    nl++;
  }
  const int ts = f.tail_s, d = f.n - f.tail_s;
  if (d > 0) {
    k_tail_pull<T, TV, R><<<(d + 7) / 8, 256, 0, s>>>(ts, d, f.d_frowp.p, f.d_fcols.p,
                                                      f.d_lsplit.p, F, x, y);
    nl++;
    for (size_t lv = 0; lv + 1 < f.tl_ptr.size(); lv++) {
      const int e0 = f.tl_ptr[lv], ne = f.tl_ptr[lv + 1] - e0;
      if (ne <= 0) continue;
      k_tail_push<T, TV, R, PUSH_L><<<(ne * R + 255) / 256, 256, 0, s>>>(
          f.d_tl_row.p + e0, f.d_tl_pos.p + e0, f.d_tl_col.p + e0, ne, f.d_fdiag.p, F, y);
      nl++;
    }
    if (f.dense_n > 0) {
      dense_solve<T, TV, R>(f, y, s, nl);
      const int ne = (int)f.td_row.size();
      if (ne > 0) {
        k_tail_push<T, TV, R, PUSH_U_FINAL><<<(ne * R + 255) / 256, 256, 0, s>>>(
            f.d_td_row.p, f.d_td_pos.p, f.d_td_col.p, ne, f.d_fdiag.p, F, y);
        nl++;
      }
    }
    for (size_t lv = 0; lv + 1 < f.tu_ptr.size(); lv++) {
      const int e0 = f.tu_ptr[lv], ne = f.tu_ptr[lv + 1] - e0;
      if (ne <= 0) continue;
      k_tail_push<T, TV, R, PUSH_U><<<(ne * R + 255) / 256, 256, 0, s>>>(
          f.d_tu_row.p + e0, f.d_tu_pos.p + e0, f.d_tu_col.p + e0, ne, f.d_fdiag.p, F, y);
      nl++;
    }
    const int dm = f.dense_t0 - ts;  // middle rows: finalized here (dense rows are final)
    if (dm > 0) {
      k_tail_finalize<T, TV, R><<<(dm * R + 127) / 128, 128, 0, s>>>(ts, dm, f.d_fdiag.p, F, y);
      nl++;
    }
  }
  for (int lv = 0; lv < Up.nlevels; lv++) {
    const int cnt = Up.ptr[lv + 1] - Up.ptr[lv];
    if (f.upper_cta[lv])
      k_tri_block<T, TV, R, true><<<cnt, 256, 0, s>>>(Up.d_rows.p + Up.ptr[lv], cnt,
                                                      f.d_frowp.p, f.d_fcols.p, f.d_fdiag.p, F,
                                                      y, y);
    else
      k_upper_warp<T, TV, R><<<(cnt + 7) / 8, 256, 0, s>>>(Up.d_rows.p + Up.ptr[lv], cnt,
                                                           f.d_frowp.p, f.d_fcols.p,
                                                           f.d_fdiag.p, F, y);
    nl++;
  }
  if (launches) *launches += nl;
  A2DS_CUDA_TRY(cudaGetLastError());
  return 0;
}

template <typename T, typename TV>
int solve_levels(const Factor &f, const T *F, const TV *x, TV *y, int nrhs, cudaStream_t s,
                 long long *launches) {
  switch (nrhs) {
    case 1: return solve_levels_r<T, TV, 1>(f, F, x, y, s, launches);
    case 2: return solve_levels_r<T, TV, 2>(f, F, x, y, s, launches);
    case 4: return solve_levels_r<T, TV, 4>(f, F, x, y, s, launches);
    case 8: return solve_levels_r<T, TV, 8>(f, F, x, y, s, launches);
    case 16: return solve_levels_r<T, TV, 16>(f, F, x, y, s, launches);
    default: return fail(A2DS_ERR_ARG, "solve: nrhs must be 1, 2, 4, 8 or 16");
  }
}

template <typename T, typename TV>
int solve_graph(Factor &f, const T *F, const TV *x, TV *y, int nrhs, cudaStream_t s,
                long long *launches) {
  for (const SolveGraph &g : f.graphs)
    if (g.F == (const void *)F && g.x == (const void *)x && g.y == (void *)y &&
        g.nrhs == nrhs && g.tv_size == (int)sizeof(TV)) {
      A2DS_CUDA_TRY(cudaGraphLaunch(g.exec, s));
      if (launches) *launches += g.nlaunch;
      return 0;
    }
  long long nl = 0;
  cudaGraph_t graph = nullptr;
  A2DS_CUDA_TRY(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
  int rc = solve_levels<T, TV>(f, F, x, y, nrhs, s, &nl);
  cudaError_t e = cudaStreamEndCapture(s, &graph);
  if (rc) {
    if (graph) cudaGraphDestroy(graph);
    return rc;
  }
  if (e != cudaSuccess || !graph)
    return fail(A2DS_ERR_CUDA, std::string("solve graph capture: ") + cudaGetErrorString(e));
  cudaGraphExec_t exec = nullptr;
  e = cudaGraphInstantiate(&exec, graph, 0);
  cudaGraphDestroy(graph);
  if (e != cudaSuccess)
    return fail(A2DS_ERR_CUDA, std::string("solve graph instantiate: ") + cudaGetErrorString(e));
  if (f.graphs.size() >= 8) {
    cudaGraphExecDestroy(f.graphs.front().exec);
    f.graphs.erase(f.graphs.begin());
  }
  f.graphs.push_back(SolveGraph{F, x, y, nrhs, (int)sizeof(TV), exec, nl});
  A2DS_CUDA_TRY(cudaGraphLaunch(exec, s));
  if (launches) *launches += nl;
  return 0;
}

Factor::~Factor() {
  for (SolveGraph &g : graphs)
    if (g.exec) cudaGraphExecDestroy(g.exec);
}

template int solve_levels<double, double>(const Factor &, const double *, const double *, double *,
                                          int, cudaStream_t, long long *);
template int solve_levels<float, float>(const Factor &, const float *, const float *, float *, int,
                                        cudaStream_t, long long *);
template int solve_graph<double, double>(Factor &, const double *, const double *, double *, int,
                                         cudaStream_t, long long *);
template int solve_graph<float, float>(Factor &, const float *, const float *, float *, int,
                                       cudaStream_t, long long *);

}  // namespace a2ds
