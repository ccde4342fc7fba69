// Host-side schedules of the block ILU(k) / LU factorization and of the
// triangular solves: dependency levels, right-looking update tasks and the
// chunk plan of the solves.  The kernels are in factor.cu and trisolve.cu.
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
  f.task_long_cols.assign(nl, 0);
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
        // a long target row takes a CTA only when its task has enough block
        // updates to fill one; small tasks on long rows (the leaf levels'
        // updates of the top separators' rows) go to the warp-group kernel,
        // which searches the row's columns in global memory
        long long work = 0;
        if (pk < 0 && f.frowp[i + 1] - f.frowp[i] > FACTOR_WARP_COLS)
          for (long long q = p; q < e; q++) {
            const int j = f.fcols[bucket_jp[q]];
            work += f.frowp[j + 1] - f.fdiag[j] - 1;
          }
        const bool first = pk >= 0 ? in_panel_rows[i] != 0
                                   : (f.frowp[i + 1] - f.frowp[i] > FACTOR_WARP_COLS &&
                                      work >= FACTOR_LONG_WORK);
        if (first == (pass == 0)) {
          f.task_row.push_back(i);
          for (long long q = p; q < e; q++) f.task_jp.push_back(bucket_jp[q]);
          f.task_ptr.push_back((int)f.task_jp.size());
          if (pass == 0) {
            if (pk >= 0) {
              pn.task_np[l]++;
            } else {
              f.task_nlong[l]++;
              f.task_long_cols[l] = std::max(f.task_long_cols[l], f.frowp[i + 1] - f.frowp[i]);
            }
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
    int maxlen = 0;
    for (int i : rows) {
      maxlen = std::max(maxlen, f.frowp[i + 1] - f.frowp[i]);
      pn.task_row.push_back(i);
      const size_t b0 = pn.task_jpk.size();
      pn.task_jpk.resize(b0 + PM, -1);
      for (int q = f.frowp[i]; q < f.fdiag[i]; q++)
        if (kof[f.fcols[q]] >= 0) pn.task_jpk[b0 + kof[f.fcols[q]]] = q;
    }
    pn.task_ptr.push_back((int)pn.task_row.size());
    pn.task_maxlen.push_back(maxlen);
    for (int k = 0; k < np; k++) kof[prow[k]] = -1;
  }
}

// The chunk plan (ChunkPlan): chunk boundaries, each row's pull ranges,
// chunk levels of the lower solve (from the first row on) and of the upper
// solve (from the last row back), and the inverse storage offsets.
void build_solve_schedule(Factor &f) {
  const int n = f.n;
  ChunkPlan &cp = f.cp;
  cp = ChunkPlan();
  // chunks: a new one where row i has no L block in column i - 1, or at
  // CHUNK_MAX rows
  cp.c0.clear();
  std::vector<int> chunk_of(n);
  int cur = 0;
  for (int i = 0; i < n; i++) {
    const int d = f.fdiag[i];
    const bool chained = i > 0 && d > f.frowp[i] && f.fcols[d - 1] == i - 1;
    if (!chained || cur >= CHUNK_MAX) {
      cp.c0.push_back(i);
      cur = 0;
    }
    cur++;
    chunk_of[i] = (int)cp.c0.size() - 1;
  }
  cp.c0.push_back(n);
  const int nc = (int)cp.c0.size() - 1;
  cp.off.assign(nc, -1);
  cp.row_lend.resize(n);
  cp.row_ustart.resize(n);
  cp.row_single.resize(n);
  long long off = 0, scr = 0;
  for (int c = 0; c < nc; c++) {
    const int a = cp.c0[c], b = cp.c0[c + 1], ns = b - a;
    cp.max_rows = std::max(cp.max_rows, ns);
    if (ns >= 2) {
      const long long sq = (long long)(6 * ns) * (6 * ns);
      cp.off[c] = off;
      off += 2 * sq;
      scr += sq;
    }
    for (int i = a; i < b; i++) {
      int k = f.frowp[i];
      while (k < f.fdiag[i] && f.fcols[k] < a) k++;
      cp.row_lend[i] = k;
      k = f.fdiag[i] + 1;
      while (k < f.frowp[i + 1] && f.fcols[k] < b) k++;
      cp.row_ustart[i] = k;
      cp.row_single[i] = ns == 1;
    }
  }
  cp.inv_size = off;
  cp.scr_size = scr;
  // lower levels: 1 + the deepest chunk among the external L columns
  std::vector<int> lv(nc, 0), uv(nc, 0);
  int maxl = 0, maxu = 0;
  for (int c = 0; c < nc; c++) {
    int l = 0;
    for (int i = cp.c0[c]; i < cp.c0[c + 1]; i++)
      for (int k = f.frowp[i]; k < cp.row_lend[i]; k++) l = std::max(l, lv[chunk_of[f.fcols[k]]] + 1);
    lv[c] = l;
    maxl = std::max(maxl, l);
  }
  // upper levels, from the last chunk back: 1 + the deepest chunk among the
  // external U columns
  for (int c = nc - 1; c >= 0; c--) {
    int l = 0;
    for (int i = cp.c0[c]; i < cp.c0[c + 1]; i++)
      for (int k = cp.row_ustart[i]; k < f.frowp[i + 1]; k++)
        l = std::max(l, uv[chunk_of[f.fcols[k]]] + 1);
    uv[c] = l;
    maxu = std::max(maxu, l);
  }
  auto fill_levels = [&](const std::vector<int> &lev, int nl, bool upper, ChunkLevels &L) {
    L.nlevels = n ? nl + 1 : 0;
    L.row_ptr.assign(L.nlevels + 1, 0);
    L.ch_ptr.assign(L.nlevels + 1, 0);
    for (int c = 0; c < nc; c++) {
      const int ns = cp.c0[c + 1] - cp.c0[c];
      L.row_ptr[lev[c] + 1] += ns;
      if (ns >= 2) L.ch_ptr[lev[c] + 1]++;
    }
    for (int l = 0; l < L.nlevels; l++) {
      L.row_ptr[l + 1] += L.row_ptr[l];
      L.ch_ptr[l + 1] += L.ch_ptr[l];
    }
    L.rows.resize(n);
    L.chunks.resize(L.ch_ptr[L.nlevels]);
    std::vector<int> fr(L.row_ptr.begin(), L.row_ptr.end() - 1);
    std::vector<int> fc(L.ch_ptr.begin(), L.ch_ptr.end() - 1);
    // big chunks (more than APPLY_WARP_ROWS rows) first within each level
    L.nbig.assign(L.nlevels, 0);
    for (int c = 0; c < nc; c++)
      if (cp.c0[c + 1] - cp.c0[c] > APPLY_WARP_ROWS) L.nbig[lev[c]]++;
    std::vector<int> fb(fc), fs(L.nlevels);
    for (int l = 0; l < L.nlevels; l++) fs[l] = fc[l] + L.nbig[l];
    for (int c = 0; c < nc; c++) {
      const int ns = cp.c0[c + 1] - cp.c0[c];
      for (int i = cp.c0[c]; i < cp.c0[c + 1]; i++) L.rows[fr[lev[c]]++] = i;
      if (ns > APPLY_WARP_ROWS)
        L.chunks[fb[lev[c]]++] = c;
      else if (ns >= 2)
        L.chunks[fs[lev[c]]++] = c;
    }
    L.max_rows.assign(L.nlevels, 1);
    for (int c = 0; c < nc; c++)
      L.max_rows[lev[c]] = std::max(L.max_rows[lev[c]], cp.c0[c + 1] - cp.c0[c]);
    // pull segments, level by level in row order
    L.seg_ptr.assign(1, 0);
    L.seg_row.clear();
    L.seg_kb.clear();
    L.seg_ke.clear();
    L.seg_flag.clear();
    L.fin_ptr.assign(1, 0);
    L.fin_rows.clear();
    for (int l = 0; l < L.nlevels; l++) {
      for (int k = L.row_ptr[l]; k < L.row_ptr[l + 1]; k++) {
        const int i = L.rows[k];
        const int kb = upper ? cp.row_ustart[i] : f.frowp[i];
        const int ke = upper ? f.frowp[i + 1] : cp.row_lend[i];
        const int len = ke - kb;
        const int nseg = std::max(1, (len + SOLVE_SEG - 1) / SOLVE_SEG);
        for (int q = 0; q < nseg; q++) {
          L.seg_row.push_back(i);
          L.seg_kb.push_back(kb + q * SOLVE_SEG);
          L.seg_ke.push_back(std::min(ke, kb + (q + 1) * SOLVE_SEG));
          L.seg_flag.push_back(nseg > 1 ? 1 : 0);
        }
        if (upper && nseg > 1 && cp.row_single[i]) L.fin_rows.push_back(i);
      }
      L.seg_ptr.push_back((int)L.seg_row.size());
      L.fin_ptr.push_back((int)L.fin_rows.size());
    }
  };
  fill_levels(lv, maxl, false, cp.lo);
  fill_levels(uv, maxu, true, cp.up);
  for (int c = 0; c < nc; c++) {
    const int ns = cp.c0[c + 1] - cp.c0[c];
    if (ns >= 2) (ns <= 10 ? cp.small : cp.big).push_back(c);
  }
}

int upload_schedules(Factor &f, cudaStream_t s) {
  int rc;
  if ((rc = f.flv.d_rows.upload(f.flv.rows.data(), f.flv.rows.size(), s))) return rc;
  if ((rc = f.d_task_row.upload(f.task_row.data(), f.task_row.size(), s))) return rc;
  if ((rc = f.d_task_ptr.upload(f.task_ptr.data(), f.task_ptr.size(), s))) return rc;
  if ((rc = f.d_task_jp.upload(f.task_jp.data(), f.task_jp.size(), s))) return rc;
  const ChunkPlan &cp = f.cp;
  if ((rc = f.d_ck_c0.upload(cp.c0.data(), cp.c0.size(), s))) return rc;
  if ((rc = f.d_ck_off.upload(cp.off.data(), cp.off.size(), s))) return rc;
  if ((rc = f.d_row_lend.upload(cp.row_lend.data(), cp.row_lend.size(), s))) return rc;
  if ((rc = f.d_row_ustart.upload(cp.row_ustart.data(), cp.row_ustart.size(), s))) return rc;
  if ((rc = f.d_row_single.upload(cp.row_single.data(), cp.row_single.size(), s))) return rc;
  if ((rc = f.d_lo_chunks.upload(cp.lo.chunks.data(), cp.lo.chunks.size(), s))) return rc;
  if ((rc = f.d_up_chunks.upload(cp.up.chunks.data(), cp.up.chunks.size(), s))) return rc;
  if ((rc = f.d_lo_seg_row.upload(cp.lo.seg_row.data(), cp.lo.seg_row.size(), s)) ||
      (rc = f.d_lo_seg_kb.upload(cp.lo.seg_kb.data(), cp.lo.seg_kb.size(), s)) ||
      (rc = f.d_lo_seg_ke.upload(cp.lo.seg_ke.data(), cp.lo.seg_ke.size(), s)) ||
      (rc = f.d_lo_seg_flag.upload(cp.lo.seg_flag.data(), cp.lo.seg_flag.size(), s)) ||
      (rc = f.d_up_seg_row.upload(cp.up.seg_row.data(), cp.up.seg_row.size(), s)) ||
      (rc = f.d_up_seg_kb.upload(cp.up.seg_kb.data(), cp.up.seg_kb.size(), s)) ||
      (rc = f.d_up_seg_ke.upload(cp.up.seg_ke.data(), cp.up.seg_ke.size(), s)) ||
      (rc = f.d_up_seg_flag.upload(cp.up.seg_flag.data(), cp.up.seg_flag.size(), s)) ||
      (rc = f.d_up_fin.upload(cp.up.fin_rows.data(), cp.up.fin_rows.size(), s)))
    return rc;
  if ((rc = f.d_ck_small.upload(cp.small.data(), cp.small.size(), s))) return rc;
  if ((rc = f.d_ck_big.upload(cp.big.data(), cp.big.size(), s))) return rc;
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
