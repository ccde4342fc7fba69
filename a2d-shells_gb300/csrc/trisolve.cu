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
// its chunk (a warp per row, or a CTA per row on levels with long rows) into
// a scratch vector t, and one launch applies each chunk's precomputed dense
// inverse (unit-lower for L, D + U for the upper solve) to t's rows of the
// chunk, writing y; the apply of one chunk is spread over many CTAs.  A
// one-row chunk needs no inverse: the pull finishes it in y (times D_i^{-1}
// in the upper solve).
// solve_graph() captures the whole launch sequence once per (factor, x, y,
// R) and replays it.
#include "a2ds_internal.h"
#include "df64.h"
#include "ilu.h"

namespace a2ds {

// Aligned groups of values: a factor block's row ii (six values at
// (36 k + 6 ii), 8-byte aligned in FP32, 16 in FP64) and a vector row's R
// right-hand sides (at a multiple of R values).
template <typename V, int N, int A>
struct alignas(A) Vals {
  V v[N];
};
template <typename T>
using BlockRow = Vals<T, 6, sizeof(T) == 4 ? 8 : 16>;
template <typename TV, int R>
using RhsRow = Vals<TV, R, (R * sizeof(TV) >= 16 ? 16 : R * sizeof(TV))>;

template <typename T, typename TV, int R>
__device__ __forceinline__ void block_row_fma(const BlockRow<T> &a, const TV *yv, TV (&acc)[R]) {
#pragma unroll
  for (int c = 0; c < 6; c++) {
    const RhsRow<TV, R> yr = *reinterpret_cast<const RhsRow<TV, R> *>(yv + c * R);
#pragma unroll
    for (int r = 0; r < R; r++) acc[r] += (TV)a.v[c] * yr.v[r];
  }
}

// Partial sums of sum_k F_k[ii][:] y[fcols[k]] over k = kb + g, kb + g + step,
// ..., four blocks per step so that their index, factor and vector loads are
// in flight together.
template <typename T, typename TV, int R>
__device__ __forceinline__ void row_partial(int kb, int ke, int g, int step, int ii,
                                            const int *__restrict__ fcols,
                                            const T *__restrict__ F, const TV *y, TV (&acc)[R]) {
  int k = kb + g;
  for (; k + 3 * step < ke; k += 4 * step) {
    int j[4];
    BlockRow<T> a[4];
#pragma unroll
    for (int u = 0; u < 4; u++) j[u] = fcols[k + u * step];
#pragma unroll
    for (int u = 0; u < 4; u++)
      a[u] = *reinterpret_cast<const BlockRow<T> *>(F + (size_t)(k + u * step) * 36 + 6 * ii);
#pragma unroll
    for (int u = 0; u < 4; u++) block_row_fma<T, TV, R>(a[u], y + (size_t)j[u] * 6 * R, acc);
  }
  for (; k < ke; k += step) {
    const BlockRow<T> a0 = *reinterpret_cast<const BlockRow<T> *>(F + (size_t)k * 36 + 6 * ii);
    block_row_fma<T, TV, R>(a0, y + (size_t)fcols[k] * 6 * R, acc);
  }
}

// The pull of one level, one warp per segment (a row's external blocks
// [kb, ke), at most SOLVE_SEG of them; five groups of six lanes over the
// blocks): v = sum_k F_k y_{fcols[k]} over the segment, then for the
// segment's row i
//   one segment:  r_i = src_i - v, stored in t_i (rows of multi-row chunks)
//                 or y_i (one-row chunks; upper: y_i = D_i^{-1} r_i);
//   several:      each segment subtracts v atomically from t_i, or from y_i
//                 for a lower one-row chunk; both start as copies of src
//                 (an upper one-row chunk is then finished by the apply
//                 launch: y_i = D_i^{-1} t_i).
// Lower: blocks [frowp, row_lend); upper: [row_ustart, frowp + 1); src = y
// (holding x, then the lower result).
template <typename T, typename TV, int R, bool UPPER>
__global__ void __launch_bounds__(256) k_pull_seg(const int *__restrict__ seg_row,
                                                  const int *__restrict__ seg_kb,
                                                  const int *__restrict__ seg_ke,
                                                  const int *__restrict__ seg_flag, int nseg,
                                                  const int *__restrict__ single,
                                                  const int *__restrict__ fcols,
                                                  const int *__restrict__ fdiag,
                                                  const T *__restrict__ F, const TV *src, TV *y,
                                                  TV *t) {
  __shared__ TV part[8][30][R];
  __shared__ TV z[8][6][R];
  const int wib = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int sg = blockIdx.x * 8 + wib;
  if (sg >= nseg) return;  // whole warp leaves together
  const int i = seg_row[sg];
  const int g = lane / 6, ii = lane - 6 * g;
  TV acc[R];
#pragma unroll
  for (int r = 0; r < R; r++) acc[r] = 0;
  if (lane < 30) row_partial<T, TV, R>(seg_kb[sg], seg_ke[sg], g, 5, ii, fcols, F, y, acc);
  if (lane < 30)
#pragma unroll
    for (int r = 0; r < R; r++) part[wib][lane][r] = acc[r];
  __syncwarp();
  const bool one = single[i], multi = seg_flag[sg] & 1;
  const bool fin = UPPER && one && !multi;
  TV *dst = (one && !(UPPER && multi)) ? y : t;
  for (int o = lane; o < 6 * R; o += 32) {
    const int d = o / R, r = o - R * d;
    const TV v = part[wib][d][r] + part[wib][d + 6][r] + part[wib][d + 12][r] +
                 part[wib][d + 18][r] + part[wib][d + 24][r];
    const size_t idx = ((size_t)i * 6 + d) * R + r;
    if (multi)
      atomicAdd(&dst[idx], -v);
    else if (fin)
      z[wib][d][r] = src[idx] - v;
    else
      dst[idx] = src[idx] - v;
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

template <typename T>
struct Pair;
template <>
struct Pair<float> {
  using type = float2;
};
template <>
struct Pair<double> {
  using type = double2;
};
// The 2 R values of two consecutive vector rows, loaded as one aligned unit.
template <typename TV, int N>
struct alignas(N * sizeof(TV) >= 16 ? 16 : N * sizeof(TV)) Pack {
  TV v[N];
};

// Rows of the inverse formed together by one warp: all six rows of a block
// row share its column range, so the vector values loaded for a column are
// used ROWS times (fewer for wide R to bound the accumulators).  Levels with
// only a few large chunks use one row per warp instead, for more warps.
template <int R>
struct ApplyRows {
  static constexpr int value = R <= 4 ? 6 : (R == 8 ? 3 : 1);
};

// One warp's share of y_c = Inv_c t_c: rows 6 blk + q0 .. + ROWS - 1 of the
// inverse (row-major, w = 6 ns wide; lower: columns up to the block's end,
// upper: from its start on), lanes over column pairs (one 8/16-byte load of
// the inverse per row, one load of the two columns' R values from the
// staged vector sv), then a reduce-scatter over the R right-hand sides per
// row.  Every column range starts at an even column and the inverse's
// offsets are even, so the paired loads are aligned.  The inverse is read
// with the streaming hint: it is used once per solve and must not evict
// the staged vectors' lines.
template <typename T, typename TV, int R, bool UPPER, int ROWS>
__device__ __forceinline__ void apply_rows(const T *__restrict__ Inv, int w, int blk, int q0,
                                           const TV *sv, TV *yc, int lane) {
  using T2 = typename Pair<T>::type;
  const int cb = UPPER ? 6 * blk : 0, ce = UPPER ? w : 6 * blk + 6;
  const T *I0 = Inv + (size_t)(6 * blk + q0) * w;
  TV acc[ROWS][R];
#pragma unroll
  for (int q = 0; q < ROWS; q++)
#pragma unroll
    for (int r = 0; r < R; r++) acc[q][r] = 0;
  constexpr int UNR = ROWS == 1 ? 4 : 1;  // loads in flight per lane
#pragma unroll UNR
  for (int col = cb + 2 * lane; col < ce; col += 64) {
    const Pack<TV, 2 * R> tv = *reinterpret_cast<const Pack<TV, 2 * R> *>(sv + (size_t)col * R);
#pragma unroll
    for (int q = 0; q < ROWS; q++) {
      const T2 m = __ldcs(reinterpret_cast<const T2 *>(I0 + (size_t)q * w + col));
#pragma unroll
      for (int r = 0; r < R; r++) acc[q][r] += (TV)m.x * tv.v[r] + (TV)m.y * tv.v[R + r];
    }
  }
#pragma unroll
  for (int q = 0; q < ROWS; q++) {
    int rhs;
    const TV sum = warp_reduce_scatter<TV, R>(acc[q], lane, rhs);
    if ((lane & (32 / R - 1)) == 0) yc[(size_t)(6 * blk + q0 + q) * R + rhs] = sum;
  }
}

// y_c = Inv_c t_c for every chunk c of a level, in one launch of 256-thread
// CTAs.  The level's nbig chunks of more than APPLY_WARP_ROWS rows come
// first, each spread over S CTAs (blocks [0, nbig S)): the CTA stages t_c
// (6 ns x R values, layout as in t) in shared memory, then its warps take
// units of ROWS rows of one block row, unit u = split + S (warp + 8 k)
// (interleaved, so the short and long block rows of the triangular inverse
// spread evenly).  The small chunks follow, one warp per chunk and eight
// per CTA, each warp staging its own chunk; then the upper solve's one-row
// chunks whose pulls were segmented (fin), one warp each.
template <typename T, typename TV, int R, bool UPPER, int ROWS>
__global__ void __launch_bounds__(256, sizeof(TV) == 4 ? 4 : 2)
    k_chunk_apply(const int *__restrict__ chunks, int nch, int nbig, int S,
                  const int *__restrict__ c0, const long long *__restrict__ off,
                  const T *__restrict__ inv, const TV *__restrict__ t, TV *__restrict__ y,
                  const int *__restrict__ fin, int nfin, const int *__restrict__ fdiag,
                  const T *__restrict__ F) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  constexpr int PER = 6 / ROWS;  // units per block row
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int nsmall = (nch - nbig + 7) / 8;
  const int b = blockIdx.x;
  if (b >= nbig * S + nsmall) {
    // one-row chunks of the upper solve with segmented pulls: y_i = D_i^{-1} t_i
    const int fi = (b - nbig * S - nsmall) * 8 + warp;
    if (fi >= nfin) return;
    const int i = fin[fi];
    const T *Dinv = F + (size_t)fdiag[i] * 36;
    for (int o = lane; o < 6 * R; o += 32) {
      const int d = o / R, r = o - R * d;
      TV v = 0;
#pragma unroll
      for (int c = 0; c < 6; c++) v += (TV)Dinv[6 * d + c] * t[((size_t)i * 6 + c) * R + r];
      y[((size_t)i * 6 + d) * R + r] = v;
    }
    return;
  }
  if (b < nbig * S) {
    TV *sv = reinterpret_cast<TV *>(smem_raw);
    const int c = chunks[b / S], split = b % S;
    const int a = c0[c], ns = c0[c + 1] - a, w = 6 * ns;
    const T *Inv = inv + off[c] + (UPPER ? (long long)w * w : 0);
    const TV *tc = t + (size_t)a * 6 * R;
    for (int k = threadIdx.x; k < w * R; k += blockDim.x) sv[k] = tc[k];
    __syncthreads();
    TV *yc = y + (size_t)a * 6 * R;
    for (int u = split + S * warp; u < ns * PER; u += S * 8)
      apply_rows<T, TV, R, UPPER, ROWS>(Inv, w, u / PER, (u % PER) * ROWS, sv, yc, lane);
    return;
  }
  const int ci = nbig + (b - nbig * S) * 8 + warp;
  if (ci >= nch) return;  // whole warp leaves together
  TV *sv = reinterpret_cast<TV *>(smem_raw) + (size_t)warp * 6 * APPLY_WARP_ROWS * R;
  const int c = chunks[ci];
  const int a = c0[c], ns = c0[c + 1] - a, w = 6 * ns;
  const T *Inv = inv + off[c] + (UPPER ? (long long)w * w : 0);
  const TV *tc = t + (size_t)a * 6 * R;
  for (int k = lane; k < w * R; k += 32) sv[k] = tc[k];
  __syncwarp();
  TV *yc = y + (size_t)a * 6 * R;
  for (int u = 0; u < ns * PER; u++)
    apply_rows<T, TV, R, UPPER, ROWS>(Inv, w, u / PER, (u % PER) * ROWS, sv, yc, lane);
}

// Dense copy (FP64; FP32 for FP32 factors) of every multi-row chunk's
// diagonal block out of the factor (scratch zeroed beforehand; chunk c's
// (6 ns)^2 block at off[c] / 2, since
// the inverse storage holds two blocks per chunk), one CTA per chunk, one
// warp per row: the row's blocks inside its chunk are [row_lend, row_ustart).
template <typename TF, typename TS>
__global__ void __launch_bounds__(256) k_chunk_gather(const int *__restrict__ chunks,
                                                      const int *__restrict__ c0,
                                                      const long long *__restrict__ off,
                                                      const int *__restrict__ fcols,
                                                      const int *__restrict__ row_lend,
                                                      const int *__restrict__ row_ustart,
                                                      const TF *__restrict__ F,
                                                      TS *__restrict__ Mall) {
  const int ch = chunks[blockIdx.x];
  const int a = c0[ch], ns = c0[ch + 1] - a, w = 6 * ns;
  TS *M = Mall + off[ch] / 2;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  for (int r = warp; r < ns; r += nw) {
    const int i = a + r, k0 = row_lend[i], k1 = row_ustart[i];
    for (int idx = lane; idx < (k1 - k0) * 36; idx += 32) {
      const int k = k0 + idx / 36, e = idx % 36;
      const int ea = e / 6, eb = e % 6;
      M[(size_t)(6 * r + ea) * w + 6 * (fcols[k] - a) + eb] = (TS)F[(size_t)k * 36 + e];
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

// The same inverses for FP32 factors on the FP32 pipe: the gathered FP32
// blocks are exact in double-float, the substitution accumulates in
// double-float (~48-bit significand, so the FP32 rounding of the result is
// that of an FP64 computation up to ties) and X (double-float, in the FP64
// inverse storage) is rounded to FP32 afterwards.  ~9 FP32 operations per
// multiply-subtract instead of one FP64 FMA at 1/60 of the FP32 rate.
__device__ __forceinline__ void df_sub_prod_f(float &hi, float &lo, float m, df64 x) {
  const float ph = __fmul_rn(m, x.hi);
  float pe = fmaf(m, x.hi, -ph);
  pe = fmaf(m, x.lo, pe);
  const float s = __fsub_rn(hi, ph);
  const float bb = __fsub_rn(s, hi);
  const float err = __fadd_rn(__fsub_rn(hi, __fsub_rn(s, bb)), __fsub_rn(-ph, bb));
  hi = s;
  lo = __fadd_rn(lo, __fsub_rn(err, pe));
}

template <bool UPPER>
__global__ void k_chunk_inverse_df(const int *__restrict__ chunks, const int *__restrict__ c0,
                                   const long long *__restrict__ off,
                                   const float *__restrict__ Mall, df64 *__restrict__ inv) {
  const int ch = chunks[blockIdx.x];
  const int ns = c0[ch + 1] - c0[ch], w = 6 * ns;
  const float *M = Mall + off[ch] / 2;
  df64 *X = inv + off[ch] + (UPPER ? (long long)w * w : 0);
  for (int c = threadIdx.x; c < w; c += blockDim.x) {
    const int bc = c / 6;
    if (!UPPER) {
      for (int i = 0; i < ns; i++) {
        float vh[6], vl[6];
#pragma unroll
        for (int a = 0; a < 6; a++) {
          vh[a] = (6 * i + a == c) ? 1.0f : 0.0f;
          vl[a] = 0.0f;
        }
        if (i > bc) {
          for (int q = 6 * bc; q < 6 * i; q++) {
            const df64 xq = X[(size_t)q * w + c];
#pragma unroll
            for (int a = 0; a < 6; a++)
              df_sub_prod_f(vh[a], vl[a], M[(size_t)(6 * i + a) * w + q], xq);
          }
        }
#pragma unroll
        for (int a = 0; a < 6; a++) X[(size_t)(6 * i + a) * w + c] = df_norm(vh[a], vl[a]);
      }
    } else {
      for (int i = ns - 1; i >= 0; i--) {
        float zh[6], zl[6];
#pragma unroll
        for (int a = 0; a < 6; a++) {
          zh[a] = (6 * i + a == c) ? 1.0f : 0.0f;
          zl[a] = 0.0f;
        }
        if (i <= bc) {
          for (int q = 6 * (i + 1); q < 6 * bc + 6; q++) {
            const df64 xq = X[(size_t)q * w + c];
#pragma unroll
            for (int a = 0; a < 6; a++)
              df_sub_prod_f(zh[a], zl[a], M[(size_t)(6 * i + a) * w + q], xq);
          }
        }
        df64 z[6];
#pragma unroll
        for (int a = 0; a < 6; a++) z[a] = df_norm(zh[a], zl[a]);
#pragma unroll
        for (int a = 0; a < 6; a++) {
          const float *Dr = M + (size_t)(6 * i + a) * w + 6 * i;
          float h = 0.0f, l = 0.0f;
#pragma unroll
          for (int b = 0; b < 6; b++) df_sub_prod_f(h, l, -Dr[b], z[b]);
          X[(size_t)(6 * i + a) * w + c] = i <= bc ? df_norm(h, l) : df64{0.0f, 0.0f};
        }
      }
    }
  }
}

__global__ void k_narrow_df(float *__restrict__ y, const df64 *__restrict__ x, size_t n) {
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x)
    y[i] = __fadd_rn(x[i].hi, x[i].lo);
}

// ------------------------------------------------------------ launchers
// Dynamic shared memory of the apply kernel at its largest (one chunk of
// CHUNK_MAX rows, or eight of APPLY_WARP_ROWS rows), above the default 48 KB
// for wide blocks of FP64 vectors.  Set outside any stream capture.
template <typename T, typename TV, int R>
static int chunk_apply_config() {
  const int smem = std::max(CHUNK_MAX, 8 * APPLY_WARP_ROWS) * 6 * R * (int)sizeof(TV);
  constexpr int RW = ApplyRows<R>::value;
  A2DS_CUDA_TRY(cudaFuncSetAttribute(k_chunk_apply<T, TV, R, false, RW>,
                                     cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
  A2DS_CUDA_TRY(cudaFuncSetAttribute(k_chunk_apply<T, TV, R, true, RW>,
                                     cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
  A2DS_CUDA_TRY(cudaFuncSetAttribute(k_chunk_apply<T, TV, R, false, 1>,
                                     cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
  A2DS_CUDA_TRY(cudaFuncSetAttribute(k_chunk_apply<T, TV, R, true, 1>,
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
  if ((rc = f.precision == 32 ? chunk_apply_config_all<float, float>()
                              : chunk_apply_config_all<double, double>()))
    return rc;
  if ((rc = f.cinv64.alloc((size_t)cp.inv_size)) || (rc = f.cscr64.alloc((size_t)cp.scr_size)))
    return rc;
  if (f.precision == 32 && (rc = f.cinv32.alloc((size_t)cp.inv_size))) return rc;
  return 0;
}


template <typename TF>
static int chunk_build_t(Factor &f, const TF *F, cudaStream_t s, long long *launches) {
  const int nch = (int)f.cp.lo.chunks.size();
  if (nch == 0) return 0;
  const int ns_ = (int)f.cp.small.size(), nb_ = (int)f.cp.big.size();
  if (f.precision == 32) {
    // FP32 factor: gathered blocks as FP32 (in the scratch), inverses in
    // double-float (in the FP64 inverse storage), then rounded to FP32
    float *scr = reinterpret_cast<float *>(f.cscr64.p);
    df64 *inv = reinterpret_cast<df64 *>(f.cinv64.p);
    A2DS_CUDA_TRY(cudaMemsetAsync(scr, 0, (size_t)f.cp.scr_size * sizeof(float), s));
    k_chunk_gather<TF, float><<<nch, 256, 0, s>>>(f.d_lo_chunks.p, f.d_ck_c0.p, f.d_ck_off.p,
                                                  f.d_fcols.p, f.d_row_lend.p, f.d_row_ustart.p,
                                                  F, scr);
    if (ns_) {
      k_chunk_inverse_df<false><<<ns_, 64, 0, s>>>(f.d_ck_small.p, f.d_ck_c0.p, f.d_ck_off.p,
                                                   scr, inv);
      k_chunk_inverse_df<true><<<ns_, 64, 0, s>>>(f.d_ck_small.p, f.d_ck_c0.p, f.d_ck_off.p,
                                                  scr, inv);
    }
    if (nb_) {
      k_chunk_inverse_df<false><<<nb_, 6 * CHUNK_MAX, 0, s>>>(f.d_ck_big.p, f.d_ck_c0.p,
                                                              f.d_ck_off.p, scr, inv);
      k_chunk_inverse_df<true><<<nb_, 6 * CHUNK_MAX, 0, s>>>(f.d_ck_big.p, f.d_ck_c0.p,
                                                             f.d_ck_off.p, scr, inv);
    }
    const size_t n = (size_t)f.cp.inv_size;
    k_narrow_df<<<(int)std::min<size_t>((n + 255) / 256, 152 * 16), 256, 0, s>>>(f.cinv32.p,
                                                                              inv, n);
    if (launches) *launches += 2 + 2 * (ns_ > 0) + 2 * (nb_ > 0);
    A2DS_CUDA_TRY(cudaGetLastError());
    return 0;
  }
  double *scr = f.cscr64.p, *inv = f.cinv64.p;
  A2DS_CUDA_TRY(cudaMemsetAsync(scr, 0, (size_t)f.cp.scr_size * sizeof(double), s));
  k_chunk_gather<TF, double><<<nch, 256, 0, s>>>(f.d_lo_chunks.p, f.d_ck_c0.p, f.d_ck_off.p,
                                                 f.d_fcols.p, f.d_row_lend.p, f.d_row_ustart.p,
                                                 F, scr);
  // small chunks: 64 threads; large ones: a thread per column (6 CHUNK_MAX)
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

// CTAs per big chunk of a level with nbig big chunks of at most mr rows
// (units = block rows x 6 / ROWS): about 4 x 152 CTAs for the big chunks,
// at least one unit per warp.
static int chunk_apply_split(int nbig, int mr, int per) {
  return std::max(1, std::min((4 * 152 + nbig - 1) / nbig, mr * per / 8));
}

template <typename T, typename TV, int R, bool UPPER>
static void solve_level(const Factor &f, const T *F, TV *y, TV *t, int l, cudaStream_t s,
                        long long &nl) {
  const ChunkLevels &L = UPPER ? f.cp.up : f.cp.lo;
  const int s0 = L.seg_ptr[l], nseg = L.seg_ptr[l + 1] - s0;
  if (nseg > 0) {
    k_pull_seg<T, TV, R, UPPER><<<(nseg + 7) / 8, 256, 0, s>>>(
        (UPPER ? f.d_up_seg_row.p : f.d_lo_seg_row.p) + s0,
        (UPPER ? f.d_up_seg_kb.p : f.d_lo_seg_kb.p) + s0,
        (UPPER ? f.d_up_seg_ke.p : f.d_lo_seg_ke.p) + s0,
        (UPPER ? f.d_up_seg_flag.p : f.d_lo_seg_flag.p) + s0, nseg, f.d_row_single.p,
        f.d_fcols.p, f.d_fdiag.p, F, y, y, t);
    nl++;
  }
  const int nch = L.ch_ptr[l + 1] - L.ch_ptr[l];
  const int f0 = UPPER ? L.fin_ptr[l] : 0, nfin = UPPER ? L.fin_ptr[l + 1] - f0 : 0;
  if (nch > 0 || nfin > 0) {
    const int *chunks = (UPPER ? f.d_up_chunks.p : f.d_lo_chunks.p) + L.ch_ptr[l];
    const int nbig = L.nbig[l], mr = L.max_rows[l];
    constexpr int RW = ApplyRows<R>::value;
    // few large chunks: one row per warp (six times the warps)
    const bool few = (long long)nbig * mr * (6 / RW) < 8LL * 4 * 152;
    const int S = nbig ? chunk_apply_split(nbig, mr, few ? 6 : 6 / RW) : 1;
    const int blocks = nbig * S + (nch - nbig + 7) / 8 + (nfin + 7) / 8;
    const size_t smem =
        (size_t)(nbig ? std::max(mr, 8 * APPLY_WARP_ROWS) : 8 * APPLY_WARP_ROWS) * 6 * R *
        sizeof(TV);
    if (few)
      k_chunk_apply<T, TV, R, UPPER, 1><<<blocks, 256, smem, s>>>(
          chunks, nch, nbig, S, f.d_ck_c0.p, f.d_ck_off.p, chunk_inverses<T>(f), t, y,
          UPPER ? f.d_up_fin.p + f0 : nullptr, nfin, f.d_fdiag.p, F);
    else
      k_chunk_apply<T, TV, R, UPPER, RW><<<blocks, 256, smem, s>>>(
          chunks, nch, nbig, S, f.d_ck_c0.p, f.d_ck_off.p, chunk_inverses<T>(f), t, y,
          UPPER ? f.d_up_fin.p + f0 : nullptr, nfin, f.d_fdiag.p, F);
    nl++;
  }
}

// The scratch vector t of the solves (n x 6 x R values of TV), grown on
// demand; growing it drops the captured solve graphs that refer to the old
// buffer (never called while s is capturing).
static int solve_scratch(Factor &f, size_t bytes) {
  if (f.tvec.n >= bytes) return 0;
  for (SolveGraph &g : f.graphs)
    if (g.exec) cudaGraphExecDestroy(g.exec);
  f.graphs.clear();
  return f.tvec.alloc(bytes);
}

template <typename T, typename TV, int R>
static int solve_levels_r(Factor &f, const T *F, const TV *x, TV *y, cudaStream_t s,
                          long long *launches) {
  long long nl = 0;
  const size_t vb = (size_t)f.n * 6 * R * sizeof(TV);
  int rc;
  if ((rc = solve_scratch(f, vb))) return rc;
  TV *t = reinterpret_cast<TV *>(f.tvec.p);
  // the pulls subtract from y_i (one-row chunks) or t_i in place (split rows
  // add atomically), so both start from x, then t from the lower result
  if ((const void *)x != (const void *)y)
    A2DS_CUDA_TRY(cudaMemcpyAsync(y, x, vb, cudaMemcpyDeviceToDevice, s));
  A2DS_CUDA_TRY(cudaMemcpyAsync(t, y, vb, cudaMemcpyDeviceToDevice, s));
  for (int l = 0; l < f.cp.lo.nlevels; l++) solve_level<T, TV, R, false>(f, F, y, t, l, s, nl);
  A2DS_CUDA_TRY(cudaMemcpyAsync(t, y, vb, cudaMemcpyDeviceToDevice, s));
  for (int l = 0; l < f.cp.up.nlevels; l++) solve_level<T, TV, R, true>(f, F, y, t, l, s, nl);
  if (launches) *launches += nl;
  A2DS_CUDA_TRY(cudaGetLastError());
  return 0;
}

template <typename T, typename TV>
int solve_levels(Factor &f, const T *F, const TV *x, TV *y, int nrhs, cudaStream_t s,
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
  int rc0;
  if ((rc0 = solve_scratch(f, (size_t)f.n * 6 * nrhs * sizeof(TV)))) return rc0;
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

template int solve_levels<double, double>(Factor &, const double *, const double *, double *,
                                          int, cudaStream_t, long long *);
template int solve_levels<float, float>(Factor &, const float *, const float *, float *, int,
                                        cudaStream_t, long long *);
template int solve_graph<double, double>(Factor &, const double *, const double *, double *, int,
                                         cudaStream_t, long long *);
template int solve_graph<float, float>(Factor &, const float *, const float *, float *, int,
                                       cudaStream_t, long long *);

}  // namespace a2ds
