// Host-side integer graph work (see host_graph.h).
#include "host_graph.h"

#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <set>
#include <utility>
#include <vector>

namespace a2ds {

void node_csr(int nn, int ne, int npe, const int *conn, int nodiag, std::vector<int> &rowp,
              std::vector<int> &cols) {
  // node -> elements
  std::vector<int> nptr(nn + 1, 0), nel((size_t)ne * npe);
  for (size_t k = 0; k < (size_t)ne * npe; k++) nptr[conn[k] + 1]++;
  for (int i = 0; i < nn; i++) nptr[i + 1] += nptr[i];
  {
    std::vector<int> fill(nptr.begin(), nptr.end() - 1);
    for (int e = 0; e < ne; e++)
      for (int a = 0; a < npe; a++) nel[fill[conn[(size_t)e * npe + a]]++] = e;
  }
  rowp.assign(nn + 1, 0);
  cols.clear();
  std::vector<int> buf;
  for (int i = 0; i < nn; i++) {
    buf.clear();
    for (int p = nptr[i]; p < nptr[i + 1]; p++) {
      const int *en = &conn[(size_t)nel[p] * npe];
      for (int a = 0; a < npe; a++)
        if (!(nodiag && en[a] == i)) buf.push_back(en[a]);
    }
    std::sort(buf.begin(), buf.end());
    buf.erase(std::unique(buf.begin(), buf.end()), buf.end());
    cols.insert(cols.end(), buf.begin(), buf.end());
    rowp[i + 1] = (int)cols.size();
  }
}

void greedy_element_colors(int nn, int ne, int npe, const int *conn, std::vector<int> &color_ptr,
                           std::vector<int> &color_elems) {
  // node -> elements, then first-fit colouring in element order
  std::vector<int> nptr(nn + 1, 0), nel((size_t)ne * npe);
  for (size_t k = 0; k < (size_t)ne * npe; k++) nptr[conn[k] + 1]++;
  for (int i = 0; i < nn; i++) nptr[i + 1] += nptr[i];
  {
    std::vector<int> fill(nptr.begin(), nptr.end() - 1);
    for (int e = 0; e < ne; e++)
      for (int a = 0; a < npe; a++) nel[fill[conn[(size_t)e * npe + a]]++] = e;
  }
  std::vector<int> color(ne, -1), mark;
  int ncolors = 0;
  for (int e = 0; e < ne; e++) {
    mark.assign(ncolors + 1, 0);
    for (int a = 0; a < npe; a++) {
      int n = conn[(size_t)e * npe + a];
      for (int p = nptr[n]; p < nptr[n + 1]; p++) {
        int c = color[nel[p]];
        if (c >= 0) mark[c] = 1;
      }
    }
    int c = 0;
    while (mark[c]) c++;
    color[e] = c;
    if (c == ncolors) ncolors++;
  }
  color_ptr.assign(ncolors + 1, 0);
  for (int e = 0; e < ne; e++) color_ptr[color[e] + 1]++;
  for (int c = 0; c < ncolors; c++) color_ptr[c + 1] += color_ptr[c];
  color_elems.resize(ne);
  std::vector<int> fill(color_ptr.begin(), color_ptr.end() - 1);
  for (int e = 0; e < ne; e++) color_elems[fill[color[e]]++] = e;
}

// ------------------------------------------------------------------ ILU(k)
// Complete fill (levFill >= n - 1: no fill entry has a higher level) of a
// structurally symmetric pattern.  computeILUk then produces the filled
// graph of symmetric elimination in this order, which is computed here
// column by column along the elimination tree: the upper structure of
// column j is its own upper entries and those of its children (the columns
// whose first upper entry is j), O(fill) instead of O(block updates).  The
// lower part of row i is the transpose.  Returns false (nothing written)
// when the pattern is not symmetric.
static bool complete_fill_symbolic(int n, const std::vector<int> &rowp,
                                   const std::vector<int> &cols, std::vector<int> &frowp,
                                   std::vector<int> &fcols, std::vector<int> &fdiag) {
  for (int i = 0; i < n; i++)
    for (int q = rowp[i]; q < rowp[i + 1]; q++) {
      const int c = cols[q];
      if (c < 0 || c >= n ||
          !std::binary_search(cols.begin() + rowp[c], cols.begin() + rowp[c + 1], i))
        return false;
    }
  std::vector<std::vector<int>> U(n);
  std::vector<int> mark(n, -1), child_head(n, -1), child_next(n, -1);
  for (int j = 0; j < n; j++) {
    std::vector<int> &u = U[j];
    mark[j] = j;
    for (int q = rowp[j]; q < rowp[j + 1]; q++) {
      const int c = cols[q];
      if (c > j && mark[c] != j) {
        mark[c] = j;
        u.push_back(c);
      }
    }
    for (int ch = child_head[j]; ch >= 0; ch = child_next[ch])
      for (int c : U[ch])
        if (mark[c] != j) {  // every entry of a child's column is >= j
          mark[c] = j;
          u.push_back(c);
        }
    std::sort(u.begin(), u.end());
    if (!u.empty()) {
      child_next[j] = child_head[u[0]];
      child_head[u[0]] = j;
    }
  }
  std::vector<int> lcount(n, 0);
  for (int k = 0; k < n; k++)
    for (int c : U[k]) lcount[c]++;
  frowp.assign(n + 1, 0);
  for (int i = 0; i < n; i++) frowp[i + 1] = frowp[i] + lcount[i] + 1 + (int)U[i].size();
  fcols.assign(frowp[n], 0);
  fdiag.assign(n, 0);
  std::vector<int> pos(frowp.begin(), frowp.end() - 1);
  for (int k = 0; k < n; k++)
    for (int c : U[k]) fcols[pos[c]++] = k;  // ascending k: sorted lower parts
  for (int i = 0; i < n; i++) {
    fdiag[i] = frowp[i] + lcount[i];
    fcols[fdiag[i]] = i;
    std::copy(U[i].begin(), U[i].end(), fcols.begin() + fdiag[i] + 1);
  }
  return true;
}

// Row-by-row level-of-fill symbolic factorization: lev(i, j) is the minimum
// over eliminated k < i of lev(i, k) + lev(k, j) + 1 (original entries have
// level 0); entries with lev <= lev_fill are kept.  The working row is a
// sorted singly linked list over column indices so fill can be merged in
// while the row is being eliminated left to right.  Complete fill of a
// symmetric pattern takes the elimination-tree path above (same pattern).
int ilu_symbolic(int n, const std::vector<int> &rowp, const std::vector<int> &cols, int lev_fill,
                 std::vector<int> &frowp, std::vector<int> &fcols, std::vector<int> &fdiag) {
  if (lev_fill >= n - 1 && complete_fill_symbolic(n, rowp, cols, frowp, fcols, fdiag)) return 0;
  frowp.assign(n + 1, 0);
  fcols.clear();
  fdiag.assign(n, 0);
  std::vector<int> flev;  // level per stored entry
  std::vector<int> next(n + 1, -1), lev(n, 0);
  const int HEAD = n;
  for (int i = 0; i < n; i++) {
    // build the linked list of the original row (plus the diagonal)
    int prev = HEAD;
    bool has_diag = false;
    std::vector<int> rc(cols.begin() + rowp[i], cols.begin() + rowp[i + 1]);
    for (int c : rc) has_diag |= (c == i);
    if (!has_diag) {
      rc.push_back(i);
      std::sort(rc.begin(), rc.end());
    }
    for (int c : rc) {
      next[prev] = c;
      lev[c] = 0;
      prev = c;
    }
    next[prev] = -1;
    // eliminate with the already-factored rows k < i in increasing order
    for (int k = next[HEAD]; k >= 0 && k < i; k = next[k]) {
      const int lk = lev[k];
      int p = k;  // insertion cursor: list position before candidate columns
      for (int q = fdiag[k] + 1; q < frowp[k + 1]; q++) {
        const int c = fcols[q];
        const int l = lk + flev[q] + 1;
        while (next[p] >= 0 && next[p] < c) p = next[p];
        if (next[p] == c) {
          if (lev[c] > l) lev[c] = l;
        } else if (l <= lev_fill) {
          next[c] = next[p];
          next[p] = c;
          lev[c] = l;
        }
      }
    }
    int cnt = 0;
    for (int c = next[HEAD]; c >= 0; c = next[c]) {
      if (c == i) fdiag[i] = (int)fcols.size();
      fcols.push_back(c);
      flev.push_back(lev[c]);
      cnt++;
    }
    frowp[i + 1] = frowp[i] + cnt;
  }
  return 0;
}

// -------------------------------------------------------------------- AMD
// Approximate minimum degree on the quotient graph, following the steps of
// the reference's amd_order_interface (src/bpmat/AMDInterface.cpp) for the
// single-rank case (no interface nodes, no dependent nodes, approximate
// degrees).  The packed row storage, its compaction rules and the order of
// every scan are kept identical because the permutation must match the
// reference's bit for bit; the only change is the pivot search, which uses
// an ordered set keyed (degree, index) instead of a linear scan and selects
// the same pivot (smallest degree, then smallest index).
namespace {

struct AmdState {
  int n;
  std::vector<int> &rowp, &cols;
  std::vector<int> alen, elen, slen, degree, edeg, Lp, state, touched;
  std::set<std::pair<int, int>> cand;  // (degree, index) of live variables

  AmdState(int n_, std::vector<int> &r, std::vector<int> &c) : n(n_), rowp(r), cols(c) {}

  void set_degree(int v, int d) {
    if (state[v] == 1) cand.erase({degree[v], v});
    degree[v] = d;
    if (state[v] == 1) cand.insert({degree[v], v});
  }
  void set_state(int v, int s) {
    if (state[v] == 1) cand.erase({degree[v], v});
    state[v] = s;
    if (state[v] == 1) cand.insert({degree[v], v});
  }

  // sort Lp[0:len), drop duplicates and negative entries
  int unique_sorted(int len) {
    std::sort(Lp.begin(), Lp.begin() + len);
    int i = 0, j = 0;
    while (i < len && Lp[i] < 0) i++;
    for (; i < len; i++, j++) {
      while (i < len - 1 && Lp[i] == Lp[i + 1]) i++;
      if (i != j) Lp[j] = Lp[i];
    }
    return j;
  }

  // make room for `need` more entries in row r by compacting neighbouring
  // rows (first those before r, then those after)
  void add_space(int r, int need) {
    int got = 0;
    if (r > 0) {
      int s = r - 1;
      for (; got < need && s >= 0; s--) got += (rowp[s + 1] - rowp[s]) - alen[s];
      s++;
      int dst = rowp[s] + alen[s];
      for (int i = s + 1; i <= r; i++) {
        int src = rowp[i], nr = dst, end = src + alen[i];
        for (; src < end; src++, dst++) cols[dst] = cols[src];
        rowp[i] = nr;
      }
    }
    if (got < need) {
      int s = r + 1;
      for (; got < need && s < n; s++) got += (rowp[s + 1] - rowp[s]) - alen[s];
      s--;
      if (s >= n) s = n - 1;
      int dst = rowp[s + 1] - 1;
      for (int i = s; i > r; i--) {
        int lo = rowp[i];
        for (int src = lo + alen[i] - 1; src >= lo; src--, dst--) cols[dst] = cols[src];
        rowp[i] = rowp[i + 1] - alen[i];
      }
    }
  }

  bool same_adjacency(int i, int j) const {
    if (i == j || alen[i] != alen[j] || elen[i] != elen[j]) return false;
    int ip = rowp[i], iend = ip + alen[i], jp = rowp[j], jend = jp + alen[j];
    for (int k = 0; k < alen[i]; k++, jp++, ip++) {
      if (cols[ip] == j) ip++;
      if (cols[jp] == i) jp++;
      if (cols[ip] != cols[jp]) break;
    }
    return ip == iend && jp == jend;
  }

  void remove_variable(int v) {
    int i = rowp[v];
    for (; i < rowp[v] + elen[v]; i++) {
      int e = cols[i];
      int j = rowp[e], jend = rowp[e] + alen[e] - 1;
      for (; j < jend; j++)
        if (cols[j] == v) break;
      for (; j < jend; j++) cols[j] = cols[j + 1];
      alen[e]--;
    }
    for (; i < rowp[v] + alen[v]; i++) {
      int w = cols[i];
      int j = rowp[w] + elen[w], jend = rowp[w] + alen[w] - 1;
      for (; j < jend; j++)
        if (cols[j] == v) break;
      for (; j < jend; j++) cols[j] = cols[j + 1];
      alen[w]--;
    }
    elen[v] = 0;
    alen[v] = 0;
  }
};

}  // namespace

int amd_order(int n, std::vector<int> &rowp, std::vector<int> &cols, std::vector<int> &perm) {
  AmdState S(n, rowp, cols);
  perm.assign(n, 0);
  S.alen.resize(n);
  S.elen.assign(n, 0);
  S.slen.assign(n, 1);
  S.degree.resize(n);
  S.edeg.assign(n, -1);
  S.Lp.resize(n);
  S.state.assign(n, 1);
  for (int i = 0; i < n; i++) {
    perm[i] = i;
    S.degree[i] = rowp[i + 1] - rowp[i];
    S.alen[i] = rowp[i + 1] - rowp[i];
    S.cand.insert({S.degree[i], i});
  }
  std::vector<int> &Lp = S.Lp;
  int nsv = 0;
  for (int i = 0; i < n; nsv++) {
    if (S.cand.empty()) return 1;
    const int piv = S.cand.begin()->second;
    perm[nsv] = piv;
    S.set_state(piv, 0);

    // Lp = piv + variables of piv + variables of piv's elements
    int len = 0;
    Lp[len++] = piv;
    for (int j = rowp[piv] + S.elen[piv]; j < rowp[piv] + S.alen[piv]; j++)
      if (cols[j] != piv) Lp[len++] = cols[j];
    for (int j = rowp[piv]; j < rowp[piv] + S.elen[piv]; j++) {
      int e = cols[j];
      for (int k = rowp[e] + S.elen[e]; k < rowp[e] + S.alen[e]; k++) {
        if (len >= n) len = S.unique_sorted(len);
        if (cols[k] != piv) Lp[len++] = cols[k];
      }
    }
    len = S.unique_sorted(len);

    // remove absorbed elements and Lp variables from every row in Lp
    for (int j = 0; j < len; j++) {
      int lj = Lp[j];
      if (lj == piv) continue;
      int nre = 0, end = rowp[piv] + S.elen[piv];
      for (int k = rowp[piv], ck = rowp[lj]; k < end && ck < rowp[lj] + S.elen[lj]; ck++) {
        while (k < end && cols[k] < cols[ck]) k++;
        if (k < end && cols[k] == cols[ck]) {
          cols[ck] = -1;
          nre++;
        }
      }
      int nrv = 0;
      for (int k = 0, ck = rowp[lj] + S.elen[lj]; k < len && ck < rowp[lj] + S.alen[lj]; ck++) {
        while (k < len && Lp[k] < cols[ck]) k++;
        if (k < len && cols[ck] == Lp[k]) {
          cols[ck] = -1;
          nrv++;
        }
      }
      if (nre > 0 || nrv > 0) {
        int e2 = rowp[lj] + S.alen[lj];
        int k = rowp[lj], nk = k;
        for (; k < e2; k++, nk++) {
          while (k < e2 && cols[k] == -1) k++;
          if (k < e2) cols[nk] = cols[k];
        }
        S.elen[lj] -= nre;
        S.alen[lj] -= nre + nrv;
      }
    }
    // add the new element piv to every row in Lp (sorted among elements)
    for (int j = 0; j < len; j++) {
      int lj = Lp[j];
      if (lj == piv) continue;
      if (S.alen[lj] == rowp[lj + 1] - rowp[lj]) S.add_space(lj, 1);
      int k = rowp[lj], end = k + S.elen[lj];
      while (k < end && cols[k] < piv) k++;
      if (cols[k] != piv) {
        for (int p = rowp[lj] + S.alen[lj] - 1; p >= k; p--) cols[p + 1] = cols[p];
        cols[k] = piv;
        S.alen[lj]++;
        S.elen[lj]++;
      }
    }
    // elements adjacent to piv are absorbed
    for (int j = rowp[piv]; j < rowp[piv] + S.elen[piv]; j++) {
      int e = cols[j];
      S.alen[e] = 0;
      S.elen[e] = 0;
      S.set_state(e, -1);
    }
    // piv's row becomes the element Lp \ {piv}
    int rsize = rowp[piv + 1] - rowp[piv];
    if (len - 1 > rsize) S.add_space(piv, len - 1 - (rowp[piv + 1] - rowp[piv]));
    S.elen[piv] = 0;
    S.alen[piv] = len - 1;
    for (int j = rowp[piv], k = 0; k < len; k++, j++) {
      if (Lp[k] == piv) {
        k++;
        if (k == len) break;
      }
      cols[j] = Lp[k];
    }
    // approximate degrees of the variables in Lp (edeg entries are -1
    // outside this step; only the ones touched here are reset afterwards)
    std::vector<int> &touched = S.touched;
    touched.clear();
    for (int j = 0; j < len; j++) {
      int lj = Lp[j];
      for (int k = rowp[lj]; k < rowp[lj] + S.elen[lj]; k++) {
        int e = cols[k];
        if (S.edeg[e] < 0) {
          S.edeg[e] = 0;
          touched.push_back(e);
          for (int p = rowp[e]; p < rowp[e] + S.alen[e]; p++) S.edeg[e] += S.slen[cols[p]];
        }
        S.edeg[e] -= S.slen[lj];
      }
    }
    int degLp = 0;
    for (int j = 0; j < len; j++)
      if (Lp[j] != piv) degLp += S.slen[Lp[j]];
    for (int j = 0; j < len; j++) {
      int lj = Lp[j];
      if (lj == piv) continue;
      int d = degLp;
      for (int k = rowp[lj] + S.elen[lj]; k < rowp[lj] + S.alen[lj]; k++) d += S.slen[cols[k]];
      int start = rowp[lj] + S.elen[lj], vl = S.alen[lj] - S.elen[lj];
      if (vl > 0 && std::binary_search(&cols[start], &cols[start] + vl, lj)) d -= S.slen[lj];
      if (std::binary_search(Lp.begin(), Lp.begin() + len, lj)) d -= S.slen[lj];
      for (int k = rowp[lj]; k < rowp[lj] + S.elen[lj]; k++) {
        int e = cols[k];
        if (e == piv) continue;
        if (S.edeg[e] < 0) {
          S.edeg[e] = 0;
          touched.push_back(e);
          for (int p = rowp[e]; p < rowp[e] + S.alen[e]; p++) S.edeg[e] += S.slen[cols[p]];
        }
        d += S.edeg[e];
      }
      d = std::min(d, n - i);
      S.set_degree(lj, std::min(d, S.degree[lj] + degLp));
    }
    for (int e : touched) S.edeg[e] = -1;
    // indistinguishable variables become supervariables
    for (int j = 0; j < len; j++) {
      int lj = Lp[j];
      if (lj == piv || S.slen[lj] < 0) continue;
      for (int k = j + 1; k < len; k++) {
        int lk = Lp[k];
        if (lk == piv || S.slen[lk] < 0) continue;
        if (S.same_adjacency(lj, lk)) {
          S.slen[lj] += S.slen[lk];
          S.set_degree(lj, S.degree[lj] - S.slen[lk]);
          S.slen[lk] = -(lj + 1);
          S.set_state(lk, -1);
          S.remove_variable(lk);
        }
      }
    }
    i += S.slen[piv];
  }
  // expand supervariables into the final permutation
  int end = n;
  for (int j = nsv - 1; j >= 0; j--) {
    int sv = perm[j];
    end -= S.slen[sv];
    perm[end] = sv;
    S.state[sv] = end + 1;
  }
  for (int k = 0; k < n; k++) {
    if (S.slen[k] < 0) {
      int j = k;
      while (S.slen[j] < 0) j = -(S.slen[j] + 1);
      perm[S.state[j]] = k;
      S.state[j]++;
    }
  }
  return 0;
}

// ------------------------------------------------------------------ RCM
static int rcm_pass(int nn, const std::vector<int> &rowp, const std::vector<int> &cols, int root,
                    std::vector<int> &order, std::vector<int> &num) {
  num.assign(nn, -1);
  order.assign(nn, 0);
  int head = 0, tail = 0, count = 0;
  while (count < nn) {
    if (head == tail) {
      // next component: the root first, then the lowest unnumbered node
      if (num[root] >= 0) {
        int i = 0;
        while (i < nn && num[i] >= 0) i++;
        if (i == nn) return count;
        root = i;
      }
      order[tail++] = root;
      num[root] = count++;
    }
    while (head < tail) {
      const int level_end = tail;
      for (; head < level_end; head++) {
        const int v = order[head];
        for (int k = rowp[v]; k < rowp[v + 1]; k++) {
          const int w = cols[k];
          if (num[w] < 0) {
            num[w] = count++;
            order[tail++] = w;
          }
        }
      }
    }
  }
  for (int i = 0; i < count; i++) num[order[i]] = count - 1 - i;
  return count;
}

int rcm_order(int nn, const std::vector<int> &rowp, const std::vector<int> &cols, int root,
              int passes, std::vector<int> &new_vars) {
  std::vector<int> order;
  int got = 0;
  for (int p = 0; p < std::max(passes, 1); p++) {
    got = rcm_pass(nn, rowp, cols, root, order, new_vars);
    if (got != nn) return got;
    root = new_vars[0];
  }
  return got;
}

// -------------------------------------------------------- multicolouring
int multicolor_order(int nn, const std::vector<int> &rowp, const std::vector<int> &cols,
                     std::vector<int> &colors, std::vector<int> &new_vars) {
  colors.assign(nn, -1);
  std::vector<int> seen(nn + 1, -1);  // seen[c] == i: colour c used next to node i
  int ncolors = 0;
  for (int i = 0; i < nn; i++) {
    for (int k = rowp[i]; k < rowp[i + 1]; k++)
      if (colors[cols[k]] >= 0) seen[colors[cols[k]]] = i;
    int c = 0;
    while (c < ncolors && seen[c] == i) c++;
    if (c == ncolors) ncolors++;
    colors[i] = c;
  }
  std::vector<int> start(ncolors + 1, 0);
  for (int i = 0; i < nn; i++) start[colors[i] + 1]++;
  for (int c = 0; c < ncolors; c++) start[c + 1] += start[c];
  new_vars.resize(nn);
  for (int i = 0; i < nn; i++) new_vars[i] = start[colors[i]]++;
  return ncolors;
}

}  // namespace a2ds
