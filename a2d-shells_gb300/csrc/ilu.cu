// Host-side schedules of the block ILU(k) / LU factorization and of the
// triangular solves: dependency levels, right-looking update tasks and the
// head / dense-tail split of the solves.  The kernels are in factor.cu and
// trisolve.cu.
#include <algorithm>

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
  // Panels: runs of consecutive narrow levels (at most PANEL_LEVEL_ROWS rows
  // each, PANEL_MAX_ROWS rows together, at least two levels).  A panel's
  // own rows P are factored level by level (phase 1, tasks with targets in
  // P); every other target row receives all the panel's pivots in one task
  // (phase 2), so its trailing blocks are read and written once per panel
  // instead of once per level.
  PanelSchedule &pn = f.pn;
  pn = PanelSchedule();
  pn.level_panel.assign(nl, -1);
  {
    // the tables hold at most PANEL_MAX_ROWS entries per U block of P; their
    // total stays below PANEL_TABLE_MAX (int32 offsets, bounded memory)
    long long tab_bound = 0;
    int l = 0;
    while (l < nl) {
      int l1 = l, rows = 0, minrow = n;
      long long ublocks = 0;
      while (l1 < nl) {
        const int r = f.flv.ptr[l1 + 1] - f.flv.ptr[l1];
        if (r > PANEL_LEVEL_ROWS || rows + r > PANEL_MAX_ROWS) break;
        for (int k = f.flv.ptr[l1]; k < f.flv.ptr[l1 + 1]; k++) {
          const int j = f.flv.rows[k];
          ublocks += f.frowp[j + 1] - f.fdiag[j] - 1;
          minrow = std::min(minrow, j);
        }
        rows += r;
        l1++;
      }
      // table entries: np x (union of P's U columns), the union bounded by
      // the U blocks of P and by the columns after P's first row
      const long long est = (long long)rows * std::min<long long>(ublocks, n - minrow);
      if (l1 - l >= 2 && tab_bound + est < PANEL_TABLE_MAX) {
        tab_bound += est;
        for (int k = l; k < l1; k++) pn.level_panel[k] = (int)pn.l0.size();
        pn.l0.push_back(l);
        pn.l1.push_back(l1);
        pn.np.push_back(rows);
        l = l1;
      } else {
        l++;
      }
    }
  }
  std::vector<char> in_panel_rows(n, 0);
  pn.task_np.assign(nl, 0);
  for (int l = 0; l < nl; l++) {
    // tasks of this level: runs of equal rows in [cnt[l], cnt[l+1])
    const int pk = pn.level_panel[l];
    if (pk >= 0 && l == pn.l0[pk]) {  // mark the panel's rows
      for (int k = f.flv.ptr[l]; k < f.flv.ptr[pn.l1[pk]]; k++) in_panel_rows[f.flv.rows[k]] = 1;
    }
    // panel levels: 0 = targets in the panel (phase 1), 1 = the others (phase 2);
    // other levels: 0 = long rows, 1 = short rows
    for (int pass = 0; pass < 2; pass++) {
      for (long long p = cnt[l]; p < cnt[l + 1];) {
        long long e = p;
        while (e < cnt[l + 1] && bucket_row[e] == bucket_row[p]) e++;
        const int i = bucket_row[p];
        const bool first = pk >= 0 ? in_panel_rows[i] != 0
                                   : f.frowp[i + 1] - f.frowp[i] > FACTOR_WARP_COLS;
        if (first == (pass == 0)) {
          f.task_row.push_back(i);
          for (long long q = p; q < e; q++) f.task_jp.push_back(bucket_jp[q]);
          f.task_ptr.push_back((int)f.task_jp.size());
          if (pass == 0) {
            if (pk >= 0)
              pn.task_np[l]++;
            else
              f.task_nlong[l]++;
          }
        }
        p = e;
      }
    }
    if (pk >= 0 && l + 1 == pn.l1[pk]) {  // unmark
      for (int k = f.flv.ptr[pn.l0[pk]]; k < f.flv.ptr[l + 1]; k++) in_panel_rows[f.flv.rows[k]] = 0;
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
  // phase-2 tables and tasks of every panel
  const int PM = PANEL_MAX_ROWS;
  pn.uc_ptr.assign(1, 0);
  pn.tab_off.assign(1, 0);
  pn.task_ptr.assign(1, 0);
  std::vector<int> kof(n, -1), slot(n, -1), mark(n, -1);
  for (int pk = 0; pk < (int)pn.l0.size(); pk++) {
    const int r0 = f.flv.ptr[pn.l0[pk]], np = pn.np[pk];
    for (int k = 0; k < PM; k++) pn.prow.push_back(k < np ? f.flv.rows[r0 + k] : -1);
    const int *prow = pn.prow.data() + (size_t)pk * PM;
    for (int k = 0; k < np; k++) kof[prow[k]] = k;
    // union of the U columns outside P, and both U position tables
    std::vector<int> uc;
    for (int k = 0; k < np; k++) {
      const int j = prow[k];
      for (int q = f.fdiag[j] + 1; q < f.frowp[j + 1]; q++) {
        const int c = f.fcols[q];
        if (kof[c] < 0 && mark[c] != pk) {
          mark[c] = pk;
          uc.push_back(c);
        }
      }
    }
    std::sort(uc.begin(), uc.end());
    const int nuc = (int)uc.size();
    for (int u = 0; u < nuc; u++) slot[uc[u]] = u;
    const size_t t0 = pn.tab.size();
    pn.tab.resize(t0 + (size_t)np * nuc, -1);
    const size_t p0 = pn.tp.size();
    pn.tp.resize(p0 + (size_t)PM * PM, -1);
    for (int k = 0; k < np; k++) {
      const int j = prow[k];
      for (int q = f.fdiag[j] + 1; q < f.frowp[j + 1]; q++) {
        const int c = f.fcols[q];
        if (kof[c] >= 0)
          pn.tp[p0 + (size_t)k * PM + kof[c]] = q;
        else
          pn.tab[t0 + (size_t)k * nuc + slot[c]] = q;
      }
    }
    pn.uc.insert(pn.uc.end(), uc.begin(), uc.end());
    pn.uc_ptr.push_back((int)pn.uc.size());
    pn.tab_off.push_back((int)pn.tab.size());
    // target rows outside P with L entries in P's columns
    std::vector<int> rows;
    for (int l = pn.l0[pk]; l < pn.l1[pk]; l++)
      for (int t = f.task_level_ptr[l] + pn.task_np[l]; t < f.task_level_ptr[l + 1]; t++)
        rows.push_back(f.task_row[t]);
    std::sort(rows.begin(), rows.end());
    rows.erase(std::unique(rows.begin(), rows.end()), rows.end());
    for (int i : rows) {
      pn.task_row.push_back(i);
      const size_t b0 = pn.task_jpk.size();
      pn.task_jpk.resize(b0 + PM, -1);
      for (int q = f.frowp[i]; q < f.fdiag[i]; q++)
        if (kof[f.fcols[q]] >= 0) pn.task_jpk[b0 + kof[f.fcols[q]]] = q;
    }
    pn.task_ptr.push_back((int)pn.task_row.size());
    for (int k = 0; k < np; k++) kof[prow[k]] = -1;
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
  const PanelSchedule &pn = f.pn;
  if ((rc = f.d_pn_prow.upload(pn.prow.data(), pn.prow.size(), s))) return rc;
  if ((rc = f.d_pn_uc.upload(pn.uc.data(), pn.uc.size(), s))) return rc;
  if ((rc = f.d_pn_tab.upload(pn.tab.data(), pn.tab.size(), s))) return rc;
  if ((rc = f.d_pn_tp.upload(pn.tp.data(), pn.tp.size(), s))) return rc;
  if ((rc = f.d_pn_task_row.upload(pn.task_row.data(), pn.task_row.size(), s))) return rc;
  if ((rc = f.d_pn_task_jpk.upload(pn.task_jpk.data(), pn.task_jpk.size(), s))) return rc;
  return 0;
}

}  // namespace a2ds
