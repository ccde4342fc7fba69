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
// to all R vectors.  The rows are cut into chunks of consecutive rows
// (ChunkPlan, ilu.h) scheduled by dependency levels; per level one launch
// pulls, for every row of the level, the sums over its factor blocks outside
// its chunk (a warp per row, or a CTA per row on levels with long rows), and
// one launch applies each chunk's precomputed dense inverse (unit-lower for
// L, D + U for the upper solve) to its rows.  A one-row chunk needs no
// inverse: the pull finishes it (times D_i^{-1} in the upper solve).
// solve_graph() captures the whole launch sequence once per (factor, x, y,
// R) and replays it.
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

// y_i = src_i - sum_{k in [beg_i, end_i)} F_k y_{fcols[k]} for every row of
// a level, one warp per row (five groups of six lanes over the blocks).  In
// the upper solve (UPPER) a row that is its own chunk is finished here:
// y_i = D_i^{-1} (src_i - sum).  Lower: beg = frowp, end = row_lend, src = x;
// upper: beg = row_ustart, end = frowp + 1, src = y.
template <typename T, typename TV, int R, bool UPPER>
__global__ void __launch_bounds__(256) k_pull_warp(const int *__restrict__ rows, int nrows,
                                                   const int *__restrict__ frowp,
                                                   const int *__restrict__ bound,
                                                   const int *__restrict__ single,
                                                   const int *__restrict__ fcols,
                                                   const int *__restrict__ fdiag,
                                                   const T *__restrict__ F, const TV *src, TV *y) {
  __shared__ TV part[8][30][R];
  __shared__ TV z[8][6][R];
  const int wib = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int wr = blockIdx.x * 8 + wib;
  if (wr >= nrows) return;  // whole warp leaves together
  const int i = rows[wr];
  const int g = lane / 6, ii = lane - 6 * g;
  const int kb = UPPER ? bound[i] : frowp[i];
  const int ke = UPPER ? frowp[i + 1] : bound[i];
  TV acc[R];
#pragma unroll
  for (int r = 0; r < R; r++) acc[r] = 0;
  if (lane < 30) row_partial<T, TV, R>(kb, ke, g, 5, ii, fcols, F, y, acc);
  if (lane < 30)
#pragma unroll
    for (int r = 0; r < R; r++) part[wib][lane][r] = acc[r];
  __syncwarp();
  const bool fin = UPPER && single[i];
  for (int o = lane; o < 6 * R; o += 32) {
    const int d = o / R, r = o - R * d;
    const TV v = part[wib][d][r] + part[wib][d + 6][r] + part[wib][d + 12][r] +
                 part[wib][d + 18][r] + part[wib][d + 24][r];
    const size_t idx = ((size_t)i * 6 + d) * R + r;
    if (fin)
      z[wib][d][r] = src[idx] - v;
    else
      y[idx] = src[idx] - v;
  }
  if (!fin) return;
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

// The same for levels with long rows: one 256-thread CTA per row, 42 groups
// of six threads over the row's blocks.  With split > 1 a row's blocks are
// shared by gridDim.y CTAs that subtract their partial sums from y_i with
// atomic adds (y_i already holds src_i; not for rows finished with D_i^{-1}).
template <typename T, typename TV, int R, bool UPPER>
__global__ void __launch_bounds__(256) k_pull_cta(const int *__restrict__ rows, int nrows,
                                                  const int *__restrict__ frowp,
                                                  const int *__restrict__ bound,
                                                  const int *__restrict__ single,
                                                  const int *__restrict__ fcols,
                                                  const int *__restrict__ fdiag,
                                                  const T *__restrict__ F, const TV *src, TV *y) {
  __shared__ TV part[252][R];
  __shared__ TV z[6][R];
  const int rr = blockIdx.x;
  if (rr >= nrows) return;
  const int i = rows[rr];
  const int t = threadIdx.x;
  const int g = t / 6, ii = t - 6 * g;
  int kb = UPPER ? bound[i] : frowp[i];
  int ke = UPPER ? frowp[i + 1] : bound[i];
  const int split = gridDim.y;
  if (split > 1) {
    const int per = (ke - kb + split - 1) / split;
    kb += per * blockIdx.y;
    ke = min(ke, kb + per);
  }
  if (t < 252) {
    TV acc[R];
#pragma unroll
    for (int r = 0; r < R; r++) acc[r] = 0;
    row_partial<T, TV, R>(kb, ke, g, 42, ii, fcols, F, y, acc);
#pragma unroll
    for (int r = 0; r < R; r++) part[t][r] = acc[r];
  }
  __syncthreads();
  const bool fin = UPPER && single[i];
  for (int o = t; o < 6 * R; o += blockDim.x) {
    const int d = o / R, r = o - R * d;
    TV v = 0;
    for (int gg = 0; gg < 42; gg++) v += part[6 * gg + d][r];
    const size_t idx = ((size_t)i * 6 + d) * R + r;
    if (split > 1)
      atomicAdd(&y[idx], -v);
    else if (fin)
      z[d][r] = src[idx] - v;
    else
      y[idx] = src[idx] - v;
  }
  if (!fin || split > 1) return;
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

// y_c <- Inv_c y_c for every chunk c of a level (one CTA per chunk): the
// chunk's rows (6 ns x R values, the pulled sums) are staged in shared
// memory, then each warp takes rows of the inverse (row-major, 6 ns wide;
// lower: only columns up to the row's block, upper: from it on), lanes over
// the columns, and a reduce-scatter over the R right-hand sides.
template <typename T, typename TV, int R, bool UPPER>
__global__ void __launch_bounds__(1024) k_chunk_apply(const int *__restrict__ chunks,
                                                     const int *__restrict__ c0,
                                                     const long long *__restrict__ off,
                                                     const T *__restrict__ inv, TV *y) {
  extern __shared__ unsigned char smem_raw[];
  TV *sv = reinterpret_cast<TV *>(smem_raw);  // [r][col], 6 ns x R
  const int c = chunks[blockIdx.x];
  const int a = c0[c], ns = c0[c + 1] - a, w = 6 * ns;
  const T *Inv = inv + off[c] + (UPPER ? (long long)w * w : 0);
  TV *yc = y + (size_t)a * 6 * R;
  for (int k = threadIdx.x; k < w * R; k += blockDim.x) sv[(k % R) * w + k / R] = yc[k];
  __syncthreads();
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  for (int row = warp; row < w; row += nw) {
    const int blk = row / 6;
    const int cb = UPPER ? 6 * blk : 0, ce = UPPER ? w : 6 * blk + 6;
    const T *Ir = Inv + (size_t)row * w;
    TV acc[R];
#pragma unroll
    for (int r = 0; r < R; r++) acc[r] = 0;
    for (int col = cb + lane; col < ce; col += 32) {
      const TV m = (TV)Ir[col];
#pragma unroll
      for (int r = 0; r < R; r++) acc[r] += m * sv[r * w + col];
    }
    int rhs;
    const TV sum = warp_reduce_scatter<TV, R>(acc, lane, rhs);
    if ((lane & (32 / R - 1)) == 0) yc[(size_t)row * R + rhs] = sum;
  }
}

// Dense FP64 copy of every multi-row chunk's diagonal block out of the factor
// (scratch zeroed beforehand; chunk c's (6 ns)^2 block at off[c] / 2, since
// the inverse storage holds two blocks per chunk), one CTA per chunk, one
// warp per row: the row's blocks inside its chunk are [row_lend, row_ustart).
template <typename TF>
__global__ void __launch_bounds__(256) k_chunk_gather(const int *__restrict__ chunks,
                                                      const int *__restrict__ c0,
                                                      const long long *__restrict__ off,
                                                      const int *__restrict__ fcols,
                                                      const int *__restrict__ row_lend,
                                                      const int *__restrict__ row_ustart,
                                                      const TF *__restrict__ F,
                                                      double *__restrict__ Mall) {
  const int ch = chunks[blockIdx.x];
  const int a = c0[ch], ns = c0[ch + 1] - a, w = 6 * ns;
  double *M = Mall + off[ch] / 2;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  for (int r = warp; r < ns; r += nw) {
    const int i = a + r, k0 = row_lend[i], k1 = row_ustart[i];
    for (int idx = lane; idx < (k1 - k0) * 36; idx += 32) {
      const int k = k0 + idx / 36, e = idx % 36;
      const int ea = e / 6, eb = e % 6;
      M[(size_t)(6 * r + ea) * w + 6 * (fcols[k] - a) + eb] = (double)F[(size_t)k * 36 + e];
    }
  }
}

// Inverses of every multi-row chunk's diagonal block (chunks[] of this
// launch), one CTA per chunk and one thread per column c of the identity.
// Lower: the unit block-lower L, forward substitution; its inverse is
// block-lower, so column c starts at c's block row.  Upper: D + U with the
// stored D_i^{-1}: z_i = D_i^{-1} (e_c - sum_{j > i} U_ij z_j), backward;
// block-upper, so column c ends at c's block row.  The six rows of a block
// row are formed together (one load of X[q][c] for six products).
template <typename T, bool UPPER>
__global__ void k_chunk_inverse(const int *__restrict__ chunks, const int *__restrict__ c0,
                                const long long *__restrict__ off, const T *__restrict__ Mall,
                                T *__restrict__ inv) {
  const int ch = chunks[blockIdx.x];
  const int ns = c0[ch + 1] - c0[ch], w = 6 * ns;
  const T *M = Mall + off[ch] / 2;
  T *X = inv + off[ch] + (UPPER ? (long long)w * w : 0);
  for (int c = threadIdx.x; c < w; c += blockDim.x) {
    const int bc = c / 6;
    if (!UPPER) {
      for (int i = 0; i < ns; i++) {
        T v[6];
#pragma unroll
        for (int a = 0; a < 6; a++) v[a] = (6 * i + a == c) ? T(1) : T(0);
        if (i > bc) {
          for (int q = 6 * bc; q < 6 * i; q++) {
            const T xq = X[(size_t)q * w + c];
#pragma unroll
            for (int a = 0; a < 6; a++) v[a] -= M[(size_t)(6 * i + a) * w + q] * xq;
          }
        }
#pragma unroll
        for (int a = 0; a < 6; a++) X[(size_t)(6 * i + a) * w + c] = v[a];
      }
    } else {
      for (int i = ns - 1; i >= 0; i--) {
        T z[6];
#pragma unroll
        for (int a = 0; a < 6; a++) z[a] = (6 * i + a == c) ? T(1) : T(0);
        if (i <= bc) {
          for (int q = 6 * (i + 1); q < 6 * bc + 6; q++) {
            const T xq = X[(size_t)q * w + c];
#pragma unroll
            for (int a = 0; a < 6; a++) z[a] -= M[(size_t)(6 * i + a) * w + q] * xq;
          }
        }
#pragma unroll
        for (int a = 0; a < 6; a++) {
          const T *Dr = M + (size_t)(6 * i + a) * w + 6 * i;
          T v = 0;
#pragma unroll
          for (int b = 0; b < 6; b++) v += Dr[b] * z[b];
          X[(size_t)(6 * i + a) * w + c] = i <= bc ? v : T(0);
        }
      }
    }
  }
}

// ------------------------------------------------------------ launchers
// Shared memory of k_chunk_apply for the largest chunk: 6 CHUNK_MAX x R
// values, above the default 48 KB for wide blocks of FP64 vectors.
template <typename T, typename TV, int R>
static int chunk_apply_config() {
  const int smem = 6 * CHUNK_MAX * R * (int)sizeof(TV);
  A2DS_CUDA_TRY(cudaFuncSetAttribute(k_chunk_apply<T, TV, R, false>,
                                     cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
  A2DS_CUDA_TRY(cudaFuncSetAttribute(k_chunk_apply<T, TV, R, true>,
                                     cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
  return 0;
}

template <typename T, typename TV>
static int chunk_apply_config_all() {
  int rc;
  if ((rc = chunk_apply_config<T, TV, 1>()) || (rc = chunk_apply_config<T, TV, 2>()) ||
      (rc = chunk_apply_config<T, TV, 4>()) || (rc = chunk_apply_config<T, TV, 8>()) ||
      (rc = chunk_apply_config<T, TV, 16>()))
    return rc;
  return 0;
}

// The inverses are always computed in FP64 (gathered blocks widened); an
// FP32 factor keeps an FP32 copy for its solves.
int chunk_alloc(Factor &f) {
  const ChunkPlan &cp = f.cp;
  int rc;
  // (function attributes are set here, outside any stream capture)
  if ((rc = f.precision == 32 ? chunk_apply_config_all<float, float>()
                              : chunk_apply_config_all<double, double>()))
    return rc;
  if ((rc = f.cinv64.alloc((size_t)cp.inv_size)) || (rc = f.cscr64.alloc((size_t)cp.scr_size)))
    return rc;
  if (f.precision == 32 && (rc = f.cinv32.alloc((size_t)cp.inv_size))) return rc;
  return 0;
}

__global__ void k_narrow(float *__restrict__ y, const double *__restrict__ x, size_t n) {
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x)
    y[i] = (float)x[i];
}

template <typename TF>
static int chunk_build_t(Factor &f, const TF *F, cudaStream_t s, long long *launches) {
  const int nch = (int)f.cp.lo.chunks.size();
  if (nch == 0) return 0;
  double *scr = f.cscr64.p, *inv = f.cinv64.p;
  A2DS_CUDA_TRY(cudaMemsetAsync(scr, 0, (size_t)f.cp.scr_size * sizeof(double), s));
  k_chunk_gather<TF><<<nch, 256, 0, s>>>(f.d_lo_chunks.p, f.d_ck_c0.p, f.d_ck_off.p,
                                         f.d_fcols.p, f.d_row_lend.p, f.d_row_ustart.p, F, scr);
  // small chunks: 64 threads; large ones: a thread per column (6 CHUNK_MAX)
  const int ns_ = (int)f.cp.small.size(), nb_ = (int)f.cp.big.size();
  if (ns_) {
    k_chunk_inverse<double, false><<<ns_, 64, 0, s>>>(f.d_ck_small.p, f.d_ck_c0.p, f.d_ck_off.p,
                                                       scr, inv);
    k_chunk_inverse<double, true><<<ns_, 64, 0, s>>>(f.d_ck_small.p, f.d_ck_c0.p, f.d_ck_off.p,
                                                      scr, inv);
  }
  if (nb_) {
    k_chunk_inverse<double, false><<<nb_, 6 * CHUNK_MAX, 0, s>>>(f.d_ck_big.p, f.d_ck_c0.p,
                                                                 f.d_ck_off.p, scr, inv);
    k_chunk_inverse<double, true><<<nb_, 6 * CHUNK_MAX, 0, s>>>(f.d_ck_big.p, f.d_ck_c0.p,
                                                                f.d_ck_off.p, scr, inv);
  }
  if (launches) *launches += 1 + 2 * (ns_ > 0) + 2 * (nb_ > 0);
  if (f.precision == 32) {
    const size_t n = (size_t)f.cp.inv_size;
    k_narrow<<<(int)std::min<size_t>((n + 255) / 256, 152 * 16), 256, 0, s>>>(f.cinv32.p, inv, n);
    if (launches) *launches += 1;
  }
  A2DS_CUDA_TRY(cudaGetLastError());
  return 0;
}

int chunk_build(Factor &f, const void *F, cudaStream_t s, long long *launches) {
  if (f.precision == 32) return chunk_build_t<float>(f, (const float *)F, s, launches);
  return chunk_build_t<double>(f, (const double *)F, s, launches);
}

template <typename T>
static const T *chunk_inverses(const Factor &f);
template <>
const double *chunk_inverses<double>(const Factor &f) { return f.cinv64.p; }
template <>
const float *chunk_inverses<float>(const Factor &f) { return f.cinv32.p; }

template <typename T, typename TV, int R, bool UPPER>
static void solve_level(const Factor &f, const T *F, const TV *src, TV *y, int l, cudaStream_t s,
                        long long &nl) {
  const ChunkLevels &L = UPPER ? f.cp.up : f.cp.lo;
  const int *rows = (UPPER ? f.d_up_rows.p : f.d_lo_rows.p) + L.row_ptr[l];
  const int nrows = L.row_ptr[l + 1] - L.row_ptr[l];
  const int *bound = UPPER ? f.d_row_ustart.p : f.d_row_lend.p;
  if (L.cta[l])
    k_pull_cta<T, TV, R, UPPER><<<dim3(nrows, L.split[l]), 256, 0, s>>>(
        rows, nrows, f.d_frowp.p, bound, f.d_row_single.p, f.d_fcols.p, f.d_fdiag.p, F, src, y);
  else
    k_pull_warp<T, TV, R, UPPER><<<(nrows + 7) / 8, 256, 0, s>>>(
        rows, nrows, f.d_frowp.p, bound, f.d_row_single.p, f.d_fcols.p, f.d_fdiag.p, F, src, y);
  nl++;
  const int nch = L.ch_ptr[l + 1] - L.ch_ptr[l];
  if (nch > 0) {
    // staging for this level's largest chunk; small chunks take 64 threads
    const int mr = L.max_rows[l];
    const size_t smem = (size_t)6 * mr * R * sizeof(TV);
    k_chunk_apply<T, TV, R, UPPER><<<nch, mr <= 16 ? 64 : (mr <= 48 ? 256 : 1024), smem, s>>>(
        (UPPER ? f.d_up_chunks.p : f.d_lo_chunks.p) + L.ch_ptr[l], f.d_ck_c0.p, f.d_ck_off.p,
        chunk_inverses<T>(f), y);
    nl++;
  }
}

template <typename T, typename TV, int R>
static int solve_levels_r(const Factor &f, const T *F, const TV *x, TV *y, cudaStream_t s,
                          long long *launches) {
  long long nl = 0;
  // the lower pulls subtract from y in place (split rows add atomically)
  if ((const void *)x != (const void *)y)
    A2DS_CUDA_TRY(cudaMemcpyAsync(y, x, (size_t)f.n * 6 * R * sizeof(TV),
                                  cudaMemcpyDeviceToDevice, s));
  for (int l = 0; l < f.cp.lo.nlevels; l++) solve_level<T, TV, R, false>(f, F, y, y, l, s, nl);
  for (int l = 0; l < f.cp.up.nlevels; l++) solve_level<T, TV, R, true>(f, F, y, y, l, s, nl);
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
