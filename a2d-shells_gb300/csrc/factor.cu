// Numeric block LU / ILU(k) factorization of 6x6-block CSR matrices on the
// GPU, level-scheduled and right-looking, in FP64, FP32 or "df64"
// (double-float: an unevaluated sum of two FP32 numbers, ~48-bit mantissa,
// computed on the FP32 pipe).
//
// Numerics follow BCSRMatFactor6 (src/bpmat/BCSRMatFact6.cpp:946-1330):
// every L block becomes L_ij = A_ij D_j^{-1}, the row is updated with
// -L_ij U_jk on the factor pattern, and each diagonal block is replaced by
// its inverse (partial pivoting, as BMatComputeInverse,
// src/bpmat/BCSRMatMult.cpp:308).
//
// Why df64: on GB300 the FP64 pipe runs at ~1/58 of FP32 (about 1.75 DFMA
// per clock per SM), and the factorization is bound by it.  A df64
// multiply-subtract costs ~12 FP32 instructions, so the update runs several
// times faster on the FP32 pipe, with a rounding unit of ~2^-48 instead of
// 2^-53; the factor is converted to FP64 afterwards and every solve that
// uses it is FP64 with FP64 iterative refinement.
//
// Schedule: rows are grouped by dependency level.  For level l,
// (1) k_factor_pivot inverts the diagonal blocks of the level's rows (final
// once every lower level has been applied), (2) the update kernels process
// one task per target row i with L entries in level-l columns: form each
// L_ij = A_ij D_j^{-1} (j in level l) and apply -L_ij U_j* to row i.
// Pivots of one level never update each other's rows or L entries, and one
// task owns its target row, so no atomics are needed.  Six threads share
// each 6x6 block update (one output column each), except where noted: three
// (two columns each) for double-float long rows and panels, one (the whole
// block) for FP32 panels.  Long rows: one CTA per task (or several CTAs per
// single-pivot task when a level has few, with k_factor_lcol forming the L
// blocks first).  Short rows: a group of 6, 12 or 30 lanes per task within a
// warp, sized to the level's U-row lengths.  Runs of narrow levels are
// grouped into panels (k_update_panel).
#include <type_traits>

#include "a2ds_internal.h"
#include "df64.h"
#include "ilu.h"

namespace a2ds {

// ------------------------------------------------------------ value types
template <typename T>
struct Traits;
template <>
struct Traits<double> {
  using C = double;  // type of the pivot inverse arithmetic
};
template <>
struct Traits<float> {
  using C = float;
};
template <>
struct Traits<df64> {
  using C = double;
};

__device__ __forceinline__ double to_c(double v) { return v; }
__device__ __forceinline__ float to_c(float v) { return v; }
__device__ __forceinline__ double to_c(df64 v) { return (double)v.hi + (double)v.lo; }

template <typename T>
__device__ __forceinline__ T from_f64(double v);
template <>
__device__ __forceinline__ double from_f64<double>(double v) {
  return v;
}
template <>
__device__ __forceinline__ float from_f64<float>(double v) {
  return (float)v;
}
template <>
__device__ __forceinline__ df64 from_f64<df64>(double v) {
  return df_split(v);
}
__device__ __forceinline__ double from_c(double v, double *) { return v; }
__device__ __forceinline__ float from_c(float v, float *) { return v; }
__device__ __forceinline__ df64 from_c(double v, df64 *) { return from_f64<df64>(v); }

// ------------------------------------------------------- 6x6 block kernels
// Entry e = 6 a + b of A B (L_ij = A_ij D_j^{-1}).
__device__ __forceinline__ double blk_mul_entry(const double *A, const double *B, int e) {
  const int a = e / 6, b = e - 6 * (e / 6);
  double s = 0.0;
#pragma unroll
  for (int k = 0; k < 6; k++) s += A[6 * a + k] * B[6 * k + b];
  return s;
}
__device__ __forceinline__ float blk_mul_entry(const float *A, const float *B, int e) {
  const int a = e / 6, b = e - 6 * (e / 6);
  float s = 0.0f;
#pragma unroll
  for (int k = 0; k < 6; k++) s += A[6 * a + k] * B[6 * k + b];
  return s;
}
__device__ __forceinline__ df64 blk_mul_entry(const df64 *A, const df64 *B, int e) {
  const int a = e / 6, b = e - 6 * (e / 6);
  float hi = 0.0f, lo = 0.0f;
#pragma unroll
  for (int k = 0; k < 6; k++) {
    const df64 x = A[6 * a + k];
    df_sub_prod(hi, lo, df64{-x.hi, -x.lo}, B[6 * k + b]);
  }
  return df_norm(hi, lo);
}

// ------------------------------------------------------------- scatter
// F <- pattern-embedded copy of A (+ alpha2 A2), zero elsewhere; one warp per row.
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
  for (int idx = lane; idx < (fe - fs) * 36; idx += 32) F[(size_t)fs * 36 + idx] = from_f64<T>(0.0);
  __syncwarp();
  const int s = rowp[i], e = rowp[i + 1];
  for (int jp = s; jp < e; jp++) {
    const int c = cols[jp];
    int lo = fs, hi = fe - 1;
    while (lo < hi) {
      const int mid = (lo + hi) >> 1;
      if (fcols[mid] < c)
        lo = mid + 1;
      else
        hi = mid;
    }
    for (int k = lane; k < 36; k += 32) {
      double v = A[(size_t)jp * 36 + k];
      if (A2) v += alpha2 * A2[(size_t)jp * 36 + k];
      F[(size_t)lo * 36 + k] = from_f64<T>(v);
    }
  }
}

// ------------------------------------------------------------- pivots
// Invert the diagonal blocks of one level in place (6x6 Gauss-Jordan with
// partial pivoting, first maximum wins, as BMatComputeInverse).  Six lanes
// per block, one row of M and of the inverse each; pivot search, row swap
// and the pivot-row broadcast go through warp shuffles, so every value stays
// in registers and a level's blocks spread over many SMs.  Arithmetic in
// FP64 for FP64 and df64 factors, FP32 for FP32 factors.
template <typename T>
__global__ void __launch_bounds__(128) k_factor_pivot(const int *__restrict__ rows, int nrows,
                                                      const int *__restrict__ fdiag,
                                                      T *__restrict__ F, int *__restrict__ status) {
  using C = typename Traits<T>::C;
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
  C m[6], v[6];
#pragma unroll
  for (int k = 0; k < 6; k++) {
    m[k] = live ? to_c(D[6 * r + k]) : C(0);
    v[k] = (k == r) ? C(1) : C(0);
  }
  int fail = 0;
#pragma unroll
  for (int c = 0; c < 6; c++) {
    C bv = C(-1);
    int bp = c;
#pragma unroll
    for (int q = 0; q < 6; q++) {
      const C vq = __shfl_sync(full, fabs(m[c]), base + q);
      if (q >= c && vq > bv) {
        bv = vq;
        bp = q;
      }
    }
    if (bv == C(0) && !fail) fail = c + 1;  // singular; result unused
#pragma unroll
    for (int k = 0; k < 6; k++) {
      const C mc = __shfl_sync(full, m[k], base + c), mp = __shfl_sync(full, m[k], base + bp);
      const C vc = __shfl_sync(full, v[k], base + c), vp = __shfl_sync(full, v[k], base + bp);
      if (r == c) {
        m[k] = mp;
        v[k] = vp;
      } else if (r == bp) {
        m[k] = mc;
        v[k] = vc;
      }
    }
    const C piv = __shfl_sync(full, m[c], base + c);
    const C inv = piv != C(0) ? C(1) / piv : C(0);
    if (r == c) {
#pragma unroll
      for (int k = 0; k < 6; k++) {
        m[k] *= inv;
        v[k] *= inv;
      }
    }
    C pm[6], pv[6];
#pragma unroll
    for (int k = 0; k < 6; k++) {
      pm[k] = __shfl_sync(full, m[k], base + c);
      pv[k] = __shfl_sync(full, v[k], base + c);
    }
    if (r != c) {
      const C f = m[c];
#pragma unroll
      for (int k = 0; k < 6; k++) {
        m[k] -= f * pm[k];
        v[k] -= f * pv[k];
      }
    }
  }
  if (live) {
#pragma unroll
    for (int k = 0; k < 6; k++) D[6 * r + k] = from_c(v[k], (T *)nullptr);
    if (fail && r == 0) atomicMax(status, j + 1);
  }
}

// Double-float version for df64 factors: the same Gauss-Jordan steps and
// lane layout with every operation on the FP32 pipe (the FP64 version's
// ~30 FP64 instructions per column run at ~1/64 rate and set a latency
// floor of several microseconds per level).  The pivot search compares the
// leading parts; 1/pivot is the FP32 reciprocal refined by one Newton step,
// x1 = x0 + x0 (1 - p x0), in double-float (~48 bits).
__device__ __forceinline__ df64 df_mul(df64 a, df64 b) {
  const float ph = __fmul_rn(a.hi, b.hi);
  float pe = fmaf(a.hi, b.hi, -ph);
  pe = fmaf(a.hi, b.lo, pe);
  pe = fmaf(a.lo, b.hi, pe);
  return df_norm(ph, pe);
}
__device__ __forceinline__ df64 df_recip(df64 p) {
  const float q = __frcp_rn(p.hi);
  float hi = 1.0f, lo = 0.0f;
  df_sub_prod(hi, lo, p, df64{q, 0.0f});  // e = 1 - p q
  const float qe = __fmul_rn(q, __fadd_rn(hi, lo));
  return df_norm(q, qe);
}
__device__ __forceinline__ df64 df_shfl(unsigned mask, df64 v, int src) {
  return df64{__shfl_sync(mask, v.hi, src), __shfl_sync(mask, v.lo, src)};
}
__global__ void __launch_bounds__(128) k_factor_pivot_df(const int *__restrict__ rows, int nrows,
                                                         const int *__restrict__ fdiag,
                                                         df64 *__restrict__ F,
                                                         int *__restrict__ status) {
  const unsigned full = 0xffffffffu;
  const int lane = threadIdx.x & 31;
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (warp * 5 >= nrows) return;  // whole warp
  const int sub = lane / 6, r = lane - 6 * (lane / 6);
  const int idx = warp * 5 + sub;
  const bool live = sub < 5 && idx < nrows;
  const int base = sub < 5 ? 6 * sub : 0;
  const int j = live ? rows[idx] : 0;
  df64 *D = F + (size_t)(live ? fdiag[j] : 0) * 36;
  df64 m[6], v[6];
#pragma unroll
  for (int k = 0; k < 6; k++) {
    m[k] = live ? D[6 * r + k] : df64{0.0f, 0.0f};
    v[k] = df64{(k == r) ? 1.0f : 0.0f, 0.0f};
  }
  int fail = 0;
#pragma unroll
  for (int c = 0; c < 6; c++) {
    float bv = -1.0f;
    int bp = c;
#pragma unroll
    for (int q = 0; q < 6; q++) {
      const float vq = __shfl_sync(full, fabsf(m[c].hi), base + q);
      if (q >= c && vq > bv) {
        bv = vq;
        bp = q;
      }
    }
    if (bv == 0.0f && !fail) fail = c + 1;  // singular; result unused
#pragma unroll
    for (int k = 0; k < 6; k++) {
      const df64 mc = df_shfl(full, m[k], base + c), mp = df_shfl(full, m[k], base + bp);
      const df64 vc = df_shfl(full, v[k], base + c), vp = df_shfl(full, v[k], base + bp);
      if (r == c) {
        m[k] = mp;
        v[k] = vp;
      } else if (r == bp) {
        m[k] = mc;
        v[k] = vc;
      }
    }
    const df64 piv = df_shfl(full, m[c], base + c);
    const df64 inv = piv.hi != 0.0f ? df_recip(piv) : df64{0.0f, 0.0f};
    if (r == c) {
#pragma unroll
      for (int k = 0; k < 6; k++) {
        m[k] = df_mul(m[k], inv);
        v[k] = df_mul(v[k], inv);
      }
    }
    df64 pm[6], pv[6];
#pragma unroll
    for (int k = 0; k < 6; k++) {
      pm[k] = df_shfl(full, m[k], base + c);
      pv[k] = df_shfl(full, v[k], base + c);
    }
    if (r != c) {
      const df64 f = m[c];
#pragma unroll
      for (int k = 0; k < 6; k++) {
        float mh = m[k].hi, ml = m[k].lo, vh = v[k].hi, vl = v[k].lo;
        df_sub_prod(mh, ml, f, pm[k]);
        df_sub_prod(vh, vl, f, pv[k]);
        m[k] = df_norm(mh, ml);
        v[k] = df_norm(vh, vl);
      }
    }
  }
  if (live) {
#pragma unroll
    for (int k = 0; k < 6; k++) D[6 * r + k] = v[k];
    if (fail && r == 0) atomicMax(status, j + 1);
  }
}

// ------------------------------------------------------------- updates
// Position of column c in cols[lo, hi) (sorted), or -1.
__device__ __forceinline__ int find_col(const int *cols, int lo, int hi, int c) {
  int h = hi - 1;
  while (lo < h) {
    const int mid = (lo + h) >> 1;
    if (cols[mid] < c)
      lo = mid + 1;
    else
      h = mid;
  }
  return (lo < hi && cols[lo] == c) ? lo : -1;
}

// Galloping search for c in the sorted cols[lo, hi): probes lo, lo + 2,
// lo + 5, ... until a column >= c, then a binary search in the last gap.
// A slot's successive U columns land at increasing target positions close
// to the previous one, so starting from there costs a few probes of nearby
// (cached) addresses instead of a search of the whole remaining row.
__device__ __forceinline__ int find_col_from(const int *cols, int lo, int hi, int c) {
  int step = 1, b = lo;
  while (b < hi && cols[b] < c) {
    lo = b + 1;
    b = lo + step;
    step <<= 1;
  }
  return find_col(cols, lo, min(b + 1, hi), c);
}

// L_ij = A_ij D_j^{-1} for every L entry of one level, in place; a CTA of
// 288 threads handles 8 entries, thread (entry q, element e).  D_j^{-1} is
// final (the level's pivot kernel ran), A_ij is final (every pivot that
// updates it lies in a lower level), and the level's updates read the L
// blocks only after this kernel.  All 36 threads of an entry are in one CTA,
// so a barrier separates the reads of A_ij from the in-place writes.
template <typename T>
__global__ void __launch_bounds__(288) k_factor_lcol(const int *__restrict__ jps, int nq,
                                                     const int *__restrict__ fcols,
                                                     const int *__restrict__ fdiag,
                                                     T *__restrict__ F) {
  const int q = blockIdx.x * 8 + threadIdx.x / 36, e = threadIdx.x % 36;
  const bool live = q < nq;
  T v{};
  size_t pos = 0;
  if (live) {
    const int jp = jps[q];
    pos = (size_t)jp * 36;
    v = blk_mul_entry(F + pos, F + (size_t)fdiag[fcols[jp]] * 36, e);
  }
  __syncthreads();
  if (live) F[pos + e] = v;
}

// Column b of the target block: C[:, b] -= L U[:, b] (L in shared memory).
// Six threads share one block update, thread b owning column b: the six
// threads read each 48-byte row of U and C together (coalesced), and a
// thread holds only 18 values, so many warps fit on an SM to hide the
// memory latency of the scattered U and target blocks.  blk_col_sub is the
// register form (c = C[:, b], u = U[:, b]) shared by both update paths.
__device__ __forceinline__ void blk_col_sub(double (&c)[6], const double *L, const double (&u)[6]) {
#pragma unroll
  for (int a = 0; a < 6; a++) {
    double s = 0.0;
#pragma unroll
    for (int k = 0; k < 6; k++) s += L[6 * a + k] * u[k];
    c[a] = c[a] - s;
  }
}
__device__ __forceinline__ void blk_col_sub(float (&c)[6], const float *L, const float (&u)[6]) {
#pragma unroll
  for (int a = 0; a < 6; a++) {
    float s = 0.0f;
#pragma unroll
    for (int k = 0; k < 6; k++) s += L[6 * a + k] * u[k];
    c[a] = c[a] - s;
  }
}
__device__ __forceinline__ void blk_col_sub(df64 (&c)[6], const df64 *L, const df64 (&u)[6]) {
#pragma unroll
  for (int a = 0; a < 6; a++) {
    float hi = c[a].hi, lo = c[a].lo;
#pragma unroll
    for (int k = 0; k < 6; k++) df_sub_prod(hi, lo, L[6 * a + k], u[k]);
    c[a] = df_norm(hi, lo);
  }
}
template <typename T>
__device__ __forceinline__ void blk_col_load(T (&v)[6], const T *B, int b) {
#pragma unroll
  for (int k = 0; k < 6; k++) v[k] = B[6 * k + b];
}
template <typename T>
__device__ __forceinline__ void blk_col_update(T *C, const T *L, const T *U, int b) {
  T u[6], c[6];
  blk_col_load(u, U, b);
  blk_col_load(c, C, b);
  blk_col_sub(c, L, u);
#pragma unroll
  for (int a = 0; a < 6; a++) C[6 * a + b] = c[a];
}

// Columns 2h and 2h + 1 of C -= L U (double-float): 16-byte loads of C, U
// and the L rows (L 16-byte aligned), the same operation sequence per value
// as blk_col_sub.
__device__ __forceinline__ void blk_update_pair(df64 *C, const df64 *L, const df64 *U, int h) {
  float4 *C4 = reinterpret_cast<float4 *>(C + 2 * h);
  const float4 *U4 = reinterpret_cast<const float4 *>(U + 2 * h);
  df64 u0[6], u1[6];
#pragma unroll
  for (int q = 0; q < 6; q++) {
    const float4 v = U4[3 * q];
    u0[q] = df64{v.x, v.y};
    u1[q] = df64{v.z, v.w};
  }
  const float4 *L4 = reinterpret_cast<const float4 *>(L);
#pragma unroll
  for (int a = 0; a < 6; a++) {
    const float4 cv = C4[3 * a];
    float h0 = cv.x, l0 = cv.y, h1 = cv.z, l1 = cv.w;
    df64 l[6];
#pragma unroll
    for (int q = 0; q < 3; q++) {
      const float4 v = L4[3 * a + q];
      l[2 * q] = df64{v.x, v.y};
      l[2 * q + 1] = df64{v.z, v.w};
    }
#pragma unroll
    for (int q = 0; q < 6; q++) {
      df_sub_prod(h0, l0, l[q], u0[q]);
      df_sub_prod(h1, l1, l[q], u1[q]);
    }
    const df64 r0 = df_norm(h0, l0), r1 = df_norm(h1, l1);
    C4[3 * a] = make_float4(r0.hi, r0.lo, r1.hi, r1.lo);
  }
}

// Threads per block update in the long-row kernel: three for double-float
// (two columns each), six for FP64 and FP32 (one column each; one thread
// per whole FP32 block needs ~140 registers, and the fewer resident warps
// made the leaf levels' long tasks slower).
template <typename T>
struct UpdateLanes {
  static constexpr int n = 6;
};
template <>
struct UpdateLanes<df64> {
  static constexpr int n = 3;
};

// Long target rows: one CTA per task (64 or 32 block updates at a time,
// six threads each in FP64 and FP32, three in double-float); every pivot's
// U blocks are strided over the update units (a pivot's U columns are
// distinct, so no two units touch one target block), one barrier between
// pivots.  The row's column indices are staged
// in shared memory.  With nsplit == 1 the CTA also forms its L blocks
// L_ij = A_ij D_j^{-1} (it owns them: no other task reads them in this
// level).  With nsplit > 1 (levels whose tasks have one pivot each) nsplit
// CTAs share a task, each taking every nsplit-th stride of the pivot's U
// blocks, and k_factor_lcol has formed the L blocks beforehand.
template <typename T>
__global__ void __launch_bounds__(384, 2) k_update_long(const int *__restrict__ task_row,
                                                        const int *__restrict__ task_ptr,
                                                        const int *__restrict__ task_jp,
                                                        int ntasks, int nsplit, int cap,
                                                        const int *__restrict__ frowp,
                                                        const int *__restrict__ fcols,
                                                        const int *__restrict__ fdiag,
                                                        T *__restrict__ F) {
  extern __shared__ int s_cols[];
  __shared__ __align__(16) T s_L[36];
  const int t = blockIdx.x / nsplit, sidx = blockIdx.x - nsplit * t;
  if (t >= ntasks) return;
  const int tid = threadIdx.x;
  constexpr int NL = UpdateLanes<T>::n;
  const int slot = tid / NL, b = tid - NL * (tid / NL);
  const int nslots = blockDim.x / NL;
  const int i = task_row[t];
  const int rs = frowp[i], len = frowp[i + 1] - rs;
  const bool staged = len <= cap;
  if (staged)
    for (int k = tid; k < len; k += blockDim.x) s_cols[k] = fcols[rs + k];
  const int *cols = staged ? s_cols : fcols + rs;
  for (int q = task_ptr[t]; q < task_ptr[t + 1]; q++) {
    const int jp = task_jp[q];
    const int j = fcols[jp];
    if (nsplit == 1) {
      T v{};
      if (tid < 36) {
        v = blk_mul_entry(F + (size_t)jp * 36, F + (size_t)fdiag[j] * 36, tid);
        s_L[tid] = v;
      }
      __syncthreads();  // s_L (and, first time, s_cols) ready; every read of A_ij done
      // in place, after every read of A_ij; no update of this pivot touches
      // position jp (they search from jp + 1)
      if (tid < 36) F[(size_t)jp * 36 + tid] = v;
    } else {
      if (tid < 36) s_L[tid] = F[(size_t)jp * 36 + tid];
      __syncthreads();  // s_L (and, first time, s_cols) ready
    }
    const int ue = frowp[j + 1], lo0 = jp + 1 - rs;
    const int stride = nslots * nsplit;
#pragma unroll 1
    for (int pu = fdiag[j] + 1 + sidx * nslots + slot; slot < nslots && pu < ue; pu += stride) {
      // re-read s_L each block (cheap) rather than pinning 36 values in
      // registers for the whole loop, which would halve the resident warps
      asm volatile("" ::: "memory");
      const int pos = find_col(cols, lo0, len, fcols[pu]);
      if (pos < 0) continue;
      T *C = F + (size_t)(rs + pos) * 36;
      if constexpr (std::is_same<T, df64>::value)
        blk_update_pair(C, s_L, F + (size_t)pu * 36, b);
      else
        blk_col_update(C, s_L, F + (size_t)pu * 36, b);
    }
    __syncthreads();  // this pivot's updates done before the next pivot's
  }
}

// Short target rows: a group of 6 S lanes per task inside one warp (S block
// updates at a time; S = 1, 2 or 5 gives 5, 2 or 1 groups per warp, chosen
// per level from the mean U-row length of its pivots); the task's pivots
// are applied in order, each pivot's U blocks strided over the S slots.  The
// group first forms each L block L_ij = A_ij D_j^{-1} in place (the task
// owns it).
template <typename T, int S>
__global__ void __launch_bounds__(256) k_update_group(const int *__restrict__ task_row,
                                                      const int *__restrict__ task_ptr,
                                                      const int *__restrict__ task_jp,
                                                      int ntasks, const int *__restrict__ frowp,
                                                      const int *__restrict__ fcols,
                                                      const int *__restrict__ fdiag,
                                                      T *__restrict__ F) {
  constexpr int G = 6 * S, GW = 32 / G, NE = (36 + G - 1) / G;
  __shared__ T s_L[8][GW][36];
  const int wib = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int gw = lane / G, gl = lane - G * (lane / G);
  const int t = (blockIdx.x * 8 + wib) * GW + gw;
  if (gw >= GW || t >= ntasks) return;  // spare lanes; whole groups past the end
  const unsigned gmask = (G == 32) ? 0xffffffffu : (((1u << G) - 1u) << (gw * G));
  const int slot = gl / 6, b = gl - 6 * (gl / 6);
  const int i = task_row[t];
  const int rs = frowp[i], len = frowp[i + 1] - rs;
  const int *cols = fcols + rs;
  T *L = s_L[wib][gw];
  for (int q = task_ptr[t]; q < task_ptr[t + 1]; q++) {
    const int jp = task_jp[q];
    const int j = fcols[jp];
    T v[NE];
#pragma unroll
    for (int d = 0; d < NE; d++)
      if (gl + d * G < 36)
        v[d] = blk_mul_entry(F + (size_t)jp * 36, F + (size_t)fdiag[j] * 36, gl + d * G);
    __syncwarp(gmask);  // every read of A_ij done before the in-place write
#pragma unroll
    for (int d = 0; d < NE; d++)
      if (gl + d * G < 36) {
        L[gl + d * G] = v[d];
        F[(size_t)jp * 36 + gl + d * G] = v[d];
      }
    __syncwarp(gmask);
    const int ue = frowp[j + 1];
    int hint = jp + 1 - rs;  // the U columns of pivot j lie after column j in row i
#pragma unroll 1
    for (int pu = fdiag[j] + 1 + slot; pu < ue; pu += S) {
      const int pos = find_col_from(cols, hint, len, fcols[pu]);
      if (pos >= 0) {
        blk_col_update(F + (size_t)(rs + pos) * 36, L, F + (size_t)pu * 36, b);
        hint = pos + 1;
      }
    }
    __syncwarp(gmask);
  }
}

// Phase 2 of a panel (runs of narrow levels whose pivot rows P are
// factored together): one CTA per target row i outside P.
// (a) Row i's L blocks in P's columns, in pivot order: L_ik = A_ik D_k^{-1}
// (A_ik is final once the earlier pivots of P have been applied to it), kept
// in shared memory, written back, and applied to row i's later P columns.
// (b) Every other block of row i that a U row of P reaches (its column is in
// uc, the union of P's U columns outside P) is held in registers while all
// of row i's pivots in P are applied to it in pivot order, so the trailing
// blocks are read and written once per panel instead of once per level.
// FP32: one thread per target block (its 36 values in registers, the U
// block read as nine 16-byte vectors, 216 multiply-adds per U block read);
// double-float: three threads per target block, two columns each (16-byte
// loads of C, U and the L rows); FP64: six threads per target block, one
// column each.  tab[k nuc + u] / tp[k PM + k2] are the U positions of pivot
// k at column uc[u] / at P's column k2 (-1: none); task_jpk holds row i's L
// positions in P's columns (-1: none).  Dynamic shared memory: row i's
// columns (FACTOR_CTA_COLS ints) and uc (PANEL_UC_SMEM ints), each read
// from global memory instead when longer.  FP32 and double-float factor
// values must be 16-byte aligned (checked by the launcher).
template <typename T>
struct PanelLaunch {
  static constexpr int threads = 384, min_blocks = 3;
};
template <>
struct PanelLaunch<float> {
  static constexpr int threads = 256, min_blocks = 2;
};
template <>
struct PanelLaunch<df64> {
  static constexpr int threads = 384, min_blocks = 2;
};
template <typename T>
__global__ void __launch_bounds__(PanelLaunch<T>::threads, PanelLaunch<T>::min_blocks)
    k_update_panel(
    const int *__restrict__ task_row, const int *__restrict__ task_jpk, int ntasks,
    const int *__restrict__ prow, int np, const int *__restrict__ uc, int nuc, int cols_cap,
    int uc_cap,
    const int *__restrict__ tab, const int *__restrict__ tp, const int *__restrict__ frowp,
    const int *__restrict__ fcols, const int *__restrict__ fdiag, T *__restrict__ F) {
  constexpr int PM = PANEL_MAX_ROWS;
  extern __shared__ int s_dyn[];
  __shared__ __align__(16) T s_L[PM][36];
  __shared__ int s_jp[PM], s_kk[PM], s_nk;
  const int t = blockIdx.x;
  if (t >= ntasks) return;
  const int tid = threadIdx.x;
  const int slot = tid / 6, b = tid - 6 * (tid / 6);
  const int nslots = blockDim.x / 6;
  const int i = task_row[t];
  const int rs = frowp[i], len = frowp[i + 1] - rs;
  int *s_cols = s_dyn, *s_uc = s_dyn + cols_cap;
  const bool staged = len <= cols_cap, uc_staged = nuc <= uc_cap;
  if (staged)
    for (int k = tid; k < len; k += blockDim.x) s_cols[k] = fcols[rs + k];
  if (uc_staged)
    for (int k = tid; k < nuc; k += blockDim.x) s_uc[k] = uc[k];
  if (tid < PM) s_jp[tid] = task_jpk[(size_t)t * PM + tid];
  __syncthreads();
  if (tid == 0) {  // row i's pivots in P, in pivot order
    int nk = 0;
    for (int k = 0; k < np; k++)
      if (s_jp[k] >= 0) s_kk[nk++] = k;
    s_nk = nk;
  }
  const int *cols = staged ? s_cols : fcols + rs;
  const int *ucs = uc_staged ? s_uc : uc;
  __syncthreads();
  const int nk = s_nk;
  // (a) L blocks in P's columns
  for (int kk = 0; kk < nk; kk++) {
    const int k = s_kk[kk], jp = s_jp[k];
    T v{};
    if (tid < 36) {
      v = blk_mul_entry(F + (size_t)jp * 36, F + (size_t)fdiag[prow[k]] * 36, tid);
      s_L[k][tid] = v;
    }
    __syncthreads();  // s_L[k] ready; every read of A_ik done
    // in place, after every read of A_ik; the updates below write only the
    // blocks of row i's later pivots in P
    if (tid < 36) F[(size_t)jp * 36 + tid] = v;
    if (slot < nslots)
      for (int q = kk + 1 + slot; q < nk; q += nslots) {
        const int k2 = s_kk[q];
        const int pu = tp[k * PM + k2];
        if (pu >= 0)
          blk_col_update(F + (size_t)s_jp[k2] * 36, &s_L[k][0], F + (size_t)pu * 36, b);
      }
    __syncthreads();  // before the next pivot reads its (updated) A_ik
  }
  // (b) the other blocks: positions after row i's first L block in P (the
  // pivot order of P is its level order, not its column order)
  int lo0 = len;
  for (int kk = 0; kk < nk; kk++) lo0 = min(lo0, s_jp[s_kk[kk]] - rs + 1);
  if constexpr (std::is_same<T, float>::value) {
    // one thread per target block; the U position of the next pivot is
    // loaded while the current one is applied (nk >= 1 whenever lo0 < len)
#pragma unroll 1
    for (int pos = lo0 + tid; pos < len; pos += blockDim.x) {
      const int u = find_col(ucs, 0, nuc, cols[pos]);
      if (u < 0) continue;  // no U row of P reaches this block
      float4 *C4 = reinterpret_cast<float4 *>(F + (size_t)(rs + pos) * 36);
      float c[36];
#pragma unroll
      for (int q = 0; q < 9; q++) {
        const float4 v = C4[q];
        c[4 * q] = v.x;
        c[4 * q + 1] = v.y;
        c[4 * q + 2] = v.z;
        c[4 * q + 3] = v.w;
      }
      int pu_next = tab[(size_t)s_kk[0] * nuc + u];
#pragma unroll 1
      for (int kk = 0; kk < nk; kk++) {
        const int k = s_kk[kk], pu = pu_next;
        if (kk + 1 < nk) pu_next = tab[(size_t)s_kk[kk + 1] * nuc + u];
        if (pu < 0) continue;
        const float4 *U4 = reinterpret_cast<const float4 *>(F + (size_t)pu * 36);
        float U[36];
#pragma unroll
        for (int q = 0; q < 9; q++) {
          const float4 v = __ldg(U4 + q);  // U rows of P: read-only in this launch
          U[4 * q] = v.x;
          U[4 * q + 1] = v.y;
          U[4 * q + 2] = v.z;
          U[4 * q + 3] = v.w;
        }
        const float2 *L2 = reinterpret_cast<const float2 *>(&s_L[k][0]);
#pragma unroll
        for (int a = 0; a < 6; a++) {
          const float2 l0 = L2[3 * a], l1 = L2[3 * a + 1], l2 = L2[3 * a + 2];
          const float l[6] = {l0.x, l0.y, l1.x, l1.y, l2.x, l2.y};
#pragma unroll
          for (int bb = 0; bb < 6; bb++) {
            float sacc = 0.0f;
#pragma unroll
            for (int q = 0; q < 6; q++) sacc += l[q] * U[6 * q + bb];
            c[6 * a + bb] = c[6 * a + bb] - sacc;
          }
        }
      }
#pragma unroll
      for (int q = 0; q < 9; q++)
        C4[q] = make_float4(c[4 * q], c[4 * q + 1], c[4 * q + 2], c[4 * q + 3]);
    }
    return;
  }
  if constexpr (std::is_same<T, df64>::value) {
    // three threads per target block, thread h owning columns 2h and 2h + 1
    // (16-byte loads of C, U and the L rows; the same operation sequence per
    // value as blk_col_sub)
    const int nsl = blockDim.x / 3, sl = tid / 3, h = tid - 3 * (tid / 3);
    if (sl >= nsl) return;
#pragma unroll 1
    for (int pos = lo0 + sl; pos < len; pos += nsl) {
      const int u = find_col(ucs, 0, nuc, cols[pos]);
      if (u < 0) continue;  // no U row of P reaches this block
      float4 *C4 = reinterpret_cast<float4 *>(F + (size_t)(rs + pos) * 36 + 2 * h);
      float ch[12], cl[12];
#pragma unroll
      for (int a = 0; a < 6; a++) {
        const float4 v = C4[3 * a];  // row a: 6 values of 8 bytes, 3 float4
        ch[2 * a] = v.x;
        cl[2 * a] = v.y;
        ch[2 * a + 1] = v.z;
        cl[2 * a + 1] = v.w;
      }
      int pu_next = tab[(size_t)s_kk[0] * nuc + u];
#pragma unroll 1
      for (int kk = 0; kk < nk; kk++) {
        const int k = s_kk[kk], pu = pu_next;
        if (kk + 1 < nk) pu_next = tab[(size_t)s_kk[kk + 1] * nuc + u];
        if (pu < 0) continue;
        const float4 *U4 = reinterpret_cast<const float4 *>(F + (size_t)pu * 36 + 2 * h);
        df64 U0[6], U1[6];
#pragma unroll
        for (int q = 0; q < 6; q++) {
          const float4 v = __ldg(U4 + 3 * q);  // U rows of P: read-only in this launch
          U0[q] = df64{v.x, v.y};
          U1[q] = df64{v.z, v.w};
        }
        const float4 *L4 = reinterpret_cast<const float4 *>(&s_L[k][0]);
#pragma unroll
        for (int a = 0; a < 6; a++) {
          df64 l[6];
#pragma unroll
          for (int q = 0; q < 3; q++) {
            const float4 v = L4[3 * a + q];
            l[2 * q] = df64{v.x, v.y};
            l[2 * q + 1] = df64{v.z, v.w};
          }
          float h0 = ch[2 * a], l0 = cl[2 * a], h1 = ch[2 * a + 1], l1 = cl[2 * a + 1];
#pragma unroll
          for (int q = 0; q < 6; q++) {
            df_sub_prod(h0, l0, l[q], U0[q]);
            df_sub_prod(h1, l1, l[q], U1[q]);
          }
          const df64 r0 = df_norm(h0, l0), r1 = df_norm(h1, l1);
          ch[2 * a] = r0.hi;
          cl[2 * a] = r0.lo;
          ch[2 * a + 1] = r1.hi;
          cl[2 * a + 1] = r1.lo;
        }
      }
#pragma unroll
      for (int a = 0; a < 6; a++)
        C4[3 * a] = make_float4(ch[2 * a], cl[2 * a], ch[2 * a + 1], cl[2 * a + 1]);
    }
    return;
  }
#pragma unroll 1
  for (int pos = lo0 + slot; pos < len; pos += nslots) {
    const int u = find_col(ucs, 0, nuc, cols[pos]);
    if (u < 0) continue;  // no U row of P reaches this block
    T *C = F + (size_t)(rs + pos) * 36;
    T c[6];
    blk_col_load(c, C, b);
    // pivots four at a time: their U positions loaded together
#pragma unroll 1
    for (int k0 = 0; k0 < nk; k0 += 4) {
      int pus[4], ks[4];
#pragma unroll
      for (int d = 0; d < 4; d++) {
        ks[d] = k0 + d < nk ? s_kk[k0 + d] : 0;
        pus[d] = k0 + d < nk ? tab[(size_t)ks[d] * nuc + u] : -1;
      }
#pragma unroll
      for (int d = 0; d < 4; d++)
        if (pus[d] >= 0) {
          T uu[6];
          blk_col_load(uu, F + (size_t)pus[d] * 36, b);
          blk_col_sub(c, &s_L[ks[d]][0], uu);
        }
    }
#pragma unroll
    for (int a = 0; a < 6; a++) C[6 * a + b] = c[a];
  }
}

// df64 factor values -> FP64, in place (same 8 bytes per value).
__global__ void k_df64_to_f64(double *F, size_t n) {
  df64 *D = reinterpret_cast<df64 *>(F);
  for (size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x; k < n;
       k += (size_t)gridDim.x * blockDim.x) {
    const df64 v = D[k];
    F[k] = (double)v.hi + (double)v.lo;
  }
}

// ------------------------------------------------------------ launchers
template <typename T>
static int scatter_t(int n, const int *rowp, const int *cols, const double *A, const double *A2,
                     double alpha2, const int *frowp, const int *fcols, T *F, cudaStream_t s) {
  k_scatter_into_factor<T><<<(n * 32 + 255) / 256, 256, 0, s>>>(n, rowp, cols, A, A2, alpha2,
                                                               frowp, fcols, F);
  A2DS_CUDA_TRY(cudaGetLastError());
  return 0;
}

template <typename T>
static int levels_t(const Factor &f, T *F, int *status, cudaStream_t s, long long *launches) {
  const LevelSchedule &L = f.flv;
  static bool configured = false;
  const int smem = FACTOR_CTA_COLS * (int)sizeof(int);
  const int psmem = (FACTOR_CTA_COLS + PANEL_UC_SMEM) * (int)sizeof(int);
  if (!configured) {
    A2DS_CUDA_TRY(cudaFuncSetAttribute(k_update_long<T>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
    A2DS_CUDA_TRY(cudaFuncSetAttribute(k_update_panel<T>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, psmem));
    configured = true;
  }
  static int num_sms = 0;
  if (!num_sms) {
    int dev = 0;
    A2DS_CUDA_TRY(cudaGetDevice(&dev));
    A2DS_CUDA_TRY(cudaDeviceGetAttribute(&num_sms, cudaDevAttrMultiProcessorCount, dev));
  }
  if (!std::is_same<T, double>::value && (reinterpret_cast<uintptr_t>(F) & 15))
    return fail(A2DS_ERR_ARG, "FP32 and double-float factor values must be 16-byte aligned");
  long long nl = 0;
  const PanelSchedule &pn = f.pn;
  constexpr int PM = PANEL_MAX_ROWS;
  for (int lv = 0; lv < L.nlevels; lv++) {
    const int cnt = L.ptr[lv + 1] - L.ptr[lv];
    if constexpr (std::is_same<T, df64>::value)
      k_factor_pivot_df<<<(cnt + 19) / 20, 128, 0, s>>>(L.d_rows.p + L.ptr[lv], cnt, f.d_fdiag.p, F,
                                                       status);
    else
      k_factor_pivot<T><<<(cnt + 19) / 20, 128, 0, s>>>(L.d_rows.p + L.ptr[lv], cnt, f.d_fdiag.p,
                                                        F, status);
    nl++;
    const int pk = pn.level_panel[lv];
    const int t0 = f.task_level_ptr[lv];
    // panel levels: only the tasks with targets in the panel (phase 1)
    const int nt = pk >= 0 ? pn.task_np[lv] : f.task_level_ptr[lv + 1] - t0;
    const int nlong = pk >= 0 ? nt : f.task_nlong[lv], ns = nt - nlong;
    if (nlong > 0) {
      // few single-pivot long tasks: several CTAs per task
      const int q0 = f.task_ptr[t0], nq = f.task_ptr[t0 + nlong] - q0;
      const int nsplit = (nq == nlong && nlong < 2 * num_sms)
                             ? std::min(FACTOR_MAX_SPLIT, (2 * num_sms + nlong - 1) / nlong)
                             : 1;
      if (nsplit > 1) {
        k_factor_lcol<T><<<(nq + 7) / 8, 288, 0, s>>>(f.d_task_jp.p + q0, nq, f.d_fcols.p,
                                                      f.d_fdiag.p, F);
        nl++;
      }
      // single CTAs per task: 192 threads (32 block updates at a time; the
      // leaf levels' long tasks apply few short U rows per pivot) and the
      // column staging sized to the level's longest row, so more tasks are
      // in flight per SM; split tasks (long U rows) keep 384 threads
      const int cap = pk >= 0 ? FACTOR_CTA_COLS
                              : std::min(FACTOR_CTA_COLS, std::max(1, f.task_long_cols[lv]));
      k_update_long<T><<<nlong * nsplit, nsplit > 1 ? 384 : 192, cap * (int)sizeof(int), s>>>(
          f.d_task_row.p + t0, f.d_task_ptr.p + t0, f.d_task_jp.p, nlong, nsplit, cap,
          f.d_frowp.p, f.d_fcols.p, f.d_fdiag.p, F);
      nl++;
    }
    if (ns > 0) {
      const int S = f.task_group[lv], GW = 32 / (6 * S);
      const int grid = (ns + 8 * GW - 1) / (8 * GW);
      const int *tr = f.d_task_row.p + t0 + nlong, *tp = f.d_task_ptr.p + t0 + nlong;
      if (S == 1)
        k_update_group<T, 1><<<grid, 256, 0, s>>>(tr, tp, f.d_task_jp.p, ns, f.d_frowp.p,
                                                  f.d_fcols.p, f.d_fdiag.p, F);
      else if (S == 2)
        k_update_group<T, 2><<<grid, 256, 0, s>>>(tr, tp, f.d_task_jp.p, ns, f.d_frowp.p,
                                                  f.d_fcols.p, f.d_fdiag.p, F);
      else
        k_update_group<T, 5><<<grid, 256, 0, s>>>(tr, tp, f.d_task_jp.p, ns, f.d_frowp.p,
                                                  f.d_fcols.p, f.d_fdiag.p, F);
      nl++;
    }
    if (pk >= 0 && lv + 1 == pn.l1[pk]) {  // phase 2 of the panel
      const int a = pn.task_ptr[pk], ntk = pn.task_ptr[pk + 1] - a;
      const int u0 = pn.uc_ptr[pk], nuc = pn.uc_ptr[pk + 1] - u0;
      if (ntk > 0) {
        // shared staging sized to this panel (longest target row, union of
        // U columns), so more CTAs fit on an SM
        const int cols_cap = std::min(FACTOR_CTA_COLS, std::max(1, pn.task_maxlen[pk]));
        const int uc_cap = std::min(PANEL_UC_SMEM, std::max(1, nuc));
        k_update_panel<T><<<ntk, PanelLaunch<T>::threads, (cols_cap + uc_cap) * (int)sizeof(int),
                            s>>>(
            f.d_pn_task_row.p + a, f.d_pn_task_jpk.p + (size_t)a * PM, ntk,
            f.d_pn_prow.p + (size_t)pk * PM, pn.np[pk], f.d_pn_uc.p + u0, nuc, cols_cap, uc_cap,
            f.d_pn_tab.p + pn.tab_off[pk], f.d_pn_tp.p + (size_t)pk * PM * PM, f.d_frowp.p,
            f.d_fcols.p, f.d_fdiag.p, F);
        nl++;
      }
    }
  }
  if (launches) *launches += nl;
  A2DS_CUDA_TRY(cudaGetLastError());
  return 0;
}

int factor_scatter(const Factor &f, int n, const int *rowp, const int *cols, const double *A,
                   const double *A2, double alpha2, void *F, cudaStream_t s) {
  switch (f.precision) {
    case 64:
      return scatter_t<double>(n, rowp, cols, A, A2, alpha2, f.d_frowp.p, f.d_fcols.p,
                               (double *)F, s);
    case 48:
      return scatter_t<df64>(n, rowp, cols, A, A2, alpha2, f.d_frowp.p, f.d_fcols.p, (df64 *)F, s);
    case 32:
      return scatter_t<float>(n, rowp, cols, A, A2, alpha2, f.d_frowp.p, f.d_fcols.p, (float *)F,
                              s);
    default:
      return fail(A2DS_ERR_ARG, "factor precision must be 64, 48 or 32");
  }
}

__global__ void k_df64_to_f32(float *__restrict__ out, const df64 *__restrict__ F, size_t n) {
  for (size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x; k < n;
       k += (size_t)gridDim.x * blockDim.x) {
    const df64 v = F[k];
    out[k] = __fadd_rn(v.hi, v.lo);  // the nearest FP32 value of hi + lo
  }
}

int factor_df_to_f32(const Factor &f, int n, const int *rowp, const int *cols, const double *A,
                     const double *A2, double alpha2, void *work, float *F32, int *status,
                     cudaStream_t s, long long *launches) {
  df64 *Fd = (df64 *)work;
  int rc;
  if ((rc = scatter_t<df64>(n, rowp, cols, A, A2, alpha2, f.d_frowp.p, f.d_fcols.p, Fd, s)) ||
      (rc = levels_t<df64>(f, Fd, status, s, launches)))
    return rc;
  const size_t nv = (size_t)f.nnzb() * 36;
  k_df64_to_f32<<<(int)std::min<size_t>((nv + 255) / 256, 152 * 32), 256, 0, s>>>(F32, Fd, nv);
  if (launches) *launches += 2;
  A2DS_CUDA_TRY(cudaGetLastError());
  return 0;
}

int factor_levels(const Factor &f, void *F, int *status, cudaStream_t s, long long *launches) {
  switch (f.precision) {
    case 64:
      return levels_t<double>(f, (double *)F, status, s, launches);
    case 48: {
      int rc = levels_t<df64>(f, (df64 *)F, status, s, launches);
      if (rc) return rc;
      const size_t n = (size_t)f.nnzb() * 36;
      k_df64_to_f64<<<(int)std::min<size_t>((n + 255) / 256, 152 * 32), 256, 0, s>>>((double *)F,
                                                                                     n);
      if (launches) (*launches)++;
      A2DS_CUDA_TRY(cudaGetLastError());
      return 0;
    }
    case 32:
      return levels_t<float>(f, (float *)F, status, s, launches);
    default:
      return fail(A2DS_ERR_ARG, "factor precision must be 64, 48 or 32");
  }
}

}  // namespace a2ds
