// Host-side schedules of the block ILU(k) / LU factorization and of the
// triangular solves: dependency levels, right-looking update tasks and the
// head / dense-tail split of the solves.  The kernels are in factor.cu and
// trisolve.cu.
#include "a2ds_internal.h"
#include "ilu.h"

namespace a2ds {


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
// the L entries by column level; within a level, the tasks of long target
// rows (more than FACTOR_WARP_COLS blocks, one CTA each) come first, then
// the short ones (one warp each), both in row order.
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
  f.task_nlong.assign(nl, 0);
  f.task_group.clear();
  f.task_row.clear();
  f.task_ptr.assign(1, 0);
  f.task_jp.clear();
  f.task_jp.reserve(bucket_jp.size());
  for (int l = 0; l < nl; l++) {
    // tasks of this level: runs of equal rows in [cnt[l], cnt[l+1])
    for (int pass = 0; pass < 2; pass++) {  // 0: long rows, 1: short rows
      for (long long p = cnt[l]; p < cnt[l + 1];) {
        long long e = p;
        while (e < cnt[l + 1] && bucket_row[e] == bucket_row[p]) e++;
        const int i = bucket_row[p];
        const bool is_long = f.frowp[i + 1] - f.frowp[i] > FACTOR_WARP_COLS;
        if (is_long == (pass == 0)) {
          f.task_row.push_back(i);
          for (long long q = p; q < e; q++) f.task_jp.push_back(bucket_jp[q]);
          f.task_ptr.push_back((int)f.task_jp.size());
          if (pass == 0) f.task_nlong[l]++;
        }
        p = e;
      }
    }
    f.task_level_ptr[l + 1] = (int)f.task_row.size();
    // block updates in flight per short task (6 lanes each): from the
    // level's mean U-row length per pivot entry
    double ublocks = 0.0, entries = 0.0;
    for (int t = f.task_level_ptr[l] + f.task_nlong[l]; t < f.task_level_ptr[l + 1]; t++)
      for (int q = f.task_ptr[t]; q < f.task_ptr[t + 1]; q++) {
        const int j = f.fcols[f.task_jp[q]];
        ublocks += f.frowp[j + 1] - f.fdiag[j] - 1;
        entries += 1.0;
      }
    const double mean = entries > 0 ? ublocks / entries : 0.0;
    f.task_group.push_back(mean <= 2.0 ? 1 : mean <= 8.0 ? 2 : 5);
  }
}

// Rows are split at s = the smallest row index among rows of the first
// narrow factor level (fewer than `narrow` rows); rows [s, n) are the tail,
// whose last rows [t0, n) (when dense enough) are solved as one dense block.
// Head solves are row-oriented by levels; the tail pulls its head couplings
// once, the middle rows [s, t0) push columns level by level (lower), the
// dense block is solved panel by panel, its values are pushed into the
// middle rows, the middle pushes D^{-1}-scaled columns in reverse level order
// (upper), and the head upper solve pulls the final tail values.
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
  // kernel choice per head level (see SOLVE_LONG_ROW)
  auto choose = [&](const LevelSchedule &L, bool upper, std::vector<char> &cta) {
    cta.assign(L.nlevels, 0);
    for (int l = 0; l < L.nlevels; l++) {
      int maxlen = 0;
      for (int k = L.ptr[l]; k < L.ptr[l + 1]; k++) {
        const int i = L.rows[k];
        const int len = upper ? f.frowp[i + 1] - f.fdiag[i] - 1 : f.fdiag[i] - f.frowp[i];
        maxlen = std::max(maxlen, len);
      }
      cta[l] = (L.ptr[l + 1] - L.ptr[l] < SOLVE_NARROW_ROWS || maxlen > SOLVE_LONG_ROW) ? 1 : 0;
    }
  };
  choose(f.lower, false, f.lower_cta);
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
  choose(f.upper, true, f.upper_cta);
  f.lsplit.assign(d, 0);
  f.tl_ptr.assign(1, 0);
  f.tu_ptr.assign(1, 0);
  f.tl_row.clear();
  f.tl_pos.clear();
  f.tl_col.clear();
  f.tu_row.clear();
  f.tu_pos.clear();
  f.tu_col.clear();
  f.td_row.clear();
  f.td_pos.clear();
  f.td_col.clear();
  f.dense_t0 = n;
  f.dense_n = 0;
  if (d == 0) return;
  // Dense trailing block [t0, n): the largest multiple of DENSE_PANEL block
  // rows, at most DENSE_MAX and inside the tail, whose factor blocks fill at
  // least DENSE_MIN_FILL of it.  nnz_from[t] = factor blocks (i, c) with
  // min(i, c) >= t.
  {
    std::vector<long long> nnz_from(n + 1, 0);
    for (int i = 0; i < n; i++)
      for (int k = f.frowp[i]; k < f.frowp[i + 1]; k++) nnz_from[std::min(i, f.fcols[k])]++;
    for (int t = n - 1; t >= 0; t--) nnz_from[t] += nnz_from[t + 1];
    for (int nd = std::min(DENSE_MAX, d) / DENSE_PANEL * DENSE_PANEL; nd >= DENSE_MIN; nd -= DENSE_PANEL) {
      const double fill = (double)nnz_from[n - nd] / ((double)nd * nd);
      if (fill >= DENSE_MIN_FILL) {
        f.dense_t0 = n - nd;
        f.dense_n = nd;
        break;
      }
    }
  }
  const int t0 = f.dense_t0;
  // lower tail: pivot columns in [s, t0) push into every later row; levels
  // over the middle columns, push lists grouped by pivot level
  std::vector<int> tl(d, 0);
  int maxl = 0;
  for (int i = s; i < n; i++) {
    int k = f.frowp[i];
    while (k < f.fdiag[i] && f.fcols[k] < s) k++;
    f.lsplit[i - s] = k;
    if (i >= t0) continue;
    int l = 0;
    for (; k < f.fdiag[i]; k++) l = std::max(l, tl[f.fcols[k] - s] + 1);
    tl[i - s] = l;
    maxl = std::max(maxl, l);
  }
  if (t0 > s) {
    std::vector<long long> cnt(maxl + 2, 0);
    for (int i = s; i < n; i++)
      for (int k = f.lsplit[i - s]; k < f.fdiag[i] && f.fcols[k] < t0; k++)
        cnt[tl[f.fcols[k] - s] + 1]++;
    for (int l = 0; l <= maxl; l++) cnt[l + 1] += cnt[l];
    const long long tot = cnt[maxl + 1];
    f.tl_row.resize(tot);
    f.tl_pos.resize(tot);
    f.tl_col.resize(tot);
    std::vector<long long> fill(cnt.begin(), cnt.end() - 1);
    for (int i = s; i < n; i++)
      for (int k = f.lsplit[i - s]; k < f.fdiag[i] && f.fcols[k] < t0; k++) {
        long long p = fill[tl[f.fcols[k] - s]]++;
        f.tl_row[p] = i;
        f.tl_pos[p] = k;
        f.tl_col[p] = f.fcols[k];
      }
    f.tl_ptr.resize(maxl + 2);
    for (int l = 0; l <= maxl + 1; l++) f.tl_ptr[l] = (int)cnt[l];
  }
  // upper tail, middle rows [s, t0) only (the dense block is solved whole):
  // (a) couplings to dense columns, all final after the dense solve: one list;
  // (b) middle columns in reverse level order
  for (int i = s; i < t0; i++)
    for (int k = f.fdiag[i] + 1; k < f.frowp[i + 1]; k++)
      if (f.fcols[k] >= t0) {
        f.td_row.push_back(i);
        f.td_pos.push_back(k);
        f.td_col.push_back(f.fcols[k]);
      }
  std::vector<int> tu(d, 0);
  maxl = 0;
  for (int i = t0 - 1; i >= s; i--) {
    int l = 0;
    for (int k = f.fdiag[i] + 1; k < f.frowp[i + 1] && f.fcols[k] < t0; k++)
      l = std::max(l, tu[f.fcols[k] - s] + 1);
    tu[i - s] = l;
    maxl = std::max(maxl, l);
  }
  if (t0 > s) {
    std::vector<long long> cnt(maxl + 2, 0);
    for (int i = s; i < t0; i++)
      for (int k = f.fdiag[i] + 1; k < f.frowp[i + 1] && f.fcols[k] < t0; k++)
        cnt[tu[f.fcols[k] - s] + 1]++;
    for (int l = 0; l <= maxl; l++) cnt[l + 1] += cnt[l];
    const long long tot = cnt[maxl + 1];
    f.tu_row.resize(tot);
    f.tu_pos.resize(tot);
    f.tu_col.resize(tot);
    std::vector<long long> fill(cnt.begin(), cnt.end() - 1);
    for (int i = s; i < t0; i++)
      for (int k = f.fdiag[i] + 1; k < f.frowp[i + 1] && f.fcols[k] < t0; k++) {
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
  if ((rc = f.d_td_row.upload(f.td_row.data(), f.td_row.size(), s))) return rc;
  if ((rc = f.d_td_pos.upload(f.td_pos.data(), f.td_pos.size(), s))) return rc;
  if ((rc = f.d_td_col.upload(f.td_col.data(), f.td_col.size(), s))) return rc;
  return 0;
}

}  // namespace a2ds
