/*
  Multi-threaded CPU pieces of the buckling solve, for the timed CPU
  baseline (TEST INFRASTRUCTURE ONLY -- bench.py's cpu_baseline and
  reference arm; nothing shipped links it).

  The numerics are the reference's, restated for OpenMP threads:
    BCSRMatFactor6 (IKJ block LU, inverted diagonal)  src/bpmat/BCSRMatFact6.cpp:946-1330
      -- every row is eliminated in the reference's order (L_ij = A_ij D_j^-1
         left to right, A_ik -= L_ij U_jk), so the values equal the serial
         restatement orc_factor bit for bit; rows of one dependency level run
         on different threads (the role of the reference's pthread variant
         BCSRMatFactor6_thread, BCSRMatFact6.cpp:28), and the long rows of
         narrow levels split each pivot's U row over the threads;
    BCSRMatApplyLower6 / Upper6                         src/bpmat/BCSRMatMult6.cpp:319-416
      -- level-scheduled over rows, p right-hand sides at once (row-major
         (row, dof, rhs) layout).
  The fill-reducing ordering is a geometric nested dissection of the node
  graph (median cuts along the widest coordinate axis, separator = the
  lower side's nodes that touch the upper side), and the complete-LU
  pattern comes from the elimination tree: both are host set-up of the CPU
  run, outside its timed region (the reference's own TACS-AMD ordering and
  symbolic phase are set-up too).  The 6x6 inverse is orc_factor's.
*/
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include <omp.h>

/* ------------------------------------------------- nested dissection */
typedef struct {
  const int *rowp, *cols;
  const double *X;
  int *perm, *side, *tmp;
  int next, leaf;
} nd_ctx;

static int cmp_key_axis;
static const double *cmp_key_X;
static int cmp_nodes(const void *a, const void *b) {
  const double xa = cmp_key_X[3 * *(const int *)a + cmp_key_axis];
  const double xb = cmp_key_X[3 * *(const int *)b + cmp_key_axis];
  if (xa < xb) return -1;
  if (xa > xb) return 1;
  return *(const int *)a - *(const int *)b;
}

/* Orders the nodes of `set` (count m, modified) into perm[next ...]. */
static void nd_recurse(nd_ctx *c, int *set, int m) {
  if (m <= c->leaf) {
    for (int k = 0; k < m; k++) c->perm[c->next++] = set[k];
    return;
  }
  int axis = 0;
  double best = -1.0;
  for (int a = 0; a < 3; a++) {
    double lo = 1e300, hi = -1e300;
    for (int k = 0; k < m; k++) {
      const double v = c->X[3 * set[k] + a];
      lo = v < lo ? v : lo;
      hi = v > hi ? v : hi;
    }
    if (hi - lo > best) {
      best = hi - lo;
      axis = a;
    }
  }
  cmp_key_axis = axis;
  cmp_key_X = c->X;
  qsort(set, (size_t)m, sizeof(int), cmp_nodes);
  const int h = m / 2;
  /* side: 1 lower half, 2 upper half (of this set); 0 elsewhere */
  for (int k = 0; k < m; k++) c->side[set[k]] = k < h ? 1 : 2;
  int na = 0, ns = 0;
  int *A = c->tmp, *S = c->tmp + m;
  for (int k = 0; k < h; k++) {
    const int v = set[k];
    int touch = 0;
    for (int p = c->rowp[v]; p < c->rowp[v + 1] && !touch; p++) touch = c->side[c->cols[p]] == 2;
    if (touch)
      S[ns++] = v;
    else
      A[na++] = v;
  }
  for (int k = 0; k < m; k++) c->side[set[k]] = 0;
  /* set <- [A | B | S]; recurse on A and B, separator last */
  int *B = set + na;
  memmove(B, set + h, sizeof(int) * (size_t)(m - h));
  memcpy(set, A, sizeof(int) * (size_t)na);
  memcpy(set + m - ns, S, sizeof(int) * (size_t)ns);
  const int nb = m - h;
  int *Sk = (int *)malloc(sizeof(int) * (size_t)(ns ? ns : 1));
  memcpy(Sk, set + m - ns, sizeof(int) * (size_t)ns);
  nd_recurse(c, set, na);
  nd_recurse(c, B, nb);
  for (int k = 0; k < ns; k++) c->perm[c->next++] = Sk[k];
  free(Sk);
}

/* perm[k] = node of matrix row k.  rowp/cols: node graph (the diagonal may
   be present).  leaf: largest set ordered as is. */
void orc_nd_order(int n, const int *rowp, const int *cols, const double *X, int leaf, int *perm) {
  nd_ctx c;
  c.rowp = rowp;
  c.cols = cols;
  c.X = X;
  c.perm = perm;
  c.side = (int *)calloc((size_t)n, sizeof(int));
  c.tmp = (int *)malloc(sizeof(int) * 2 * (size_t)n);
  c.next = 0;
  c.leaf = leaf < 1 ? 1 : leaf;
  int *set = (int *)malloc(sizeof(int) * (size_t)n);
  for (int i = 0; i < n; i++) set[i] = i;
  nd_recurse(&c, set, n);
  free(set);
  free(c.tmp);
  free(c.side);
}

/* ------------------------------------------------ symbolic complete LU */
/* Pattern (rows in the matrix ordering, symmetric, sorted, with diagonal):
   L row structures from the elimination tree (Liu's algorithm with path
   compression, then the row subtrees).  Pass frowp = NULL to get the
   number of factor blocks; then frowp[n+1] and fcols are filled (sorted). */
long long orc_symbolic_lu(int n, const int *rowp, const int *cols, int *frowp, int *fcols) {
  int *parent = (int *)malloc(sizeof(int) * (size_t)n);
  int *anc = (int *)malloc(sizeof(int) * (size_t)n);
  int *mark = (int *)malloc(sizeof(int) * (size_t)n);
  for (int i = 0; i < n; i++) {
    parent[i] = -1;
    anc[i] = -1;
    for (int p = rowp[i]; p < rowp[i + 1]; p++) {
      int r = cols[p];
      if (r >= i) continue;
      while (anc[r] != -1 && anc[r] != i) {
        const int t = anc[r];
        anc[r] = i;
        r = t;
      }
      if (anc[r] == -1) {
        anc[r] = i;
        parent[r] = i;
      }
    }
  }
  /* L row counts (row subtree sizes), then the structures */
  long long *lcnt = (long long *)calloc((size_t)n + 1, sizeof(long long));
  int *ucnt = (int *)calloc((size_t)n, sizeof(int));
  for (int i = 0; i < n; i++) mark[i] = -1;
  for (int i = 0; i < n; i++) {
    mark[i] = i;
    for (int p = rowp[i]; p < rowp[i + 1]; p++) {
      int j = cols[p];
      if (j >= i) continue;
      while (mark[j] != i) {
        mark[j] = i;
        lcnt[i + 1]++;
        ucnt[j]++;
        j = parent[j];
      }
    }
  }
  long long tot = 0;
  for (int i = 0; i < n; i++) tot += lcnt[i + 1] + 1 + ucnt[i];
  if (!frowp) {
    free(parent);
    free(anc);
    free(mark);
    free(lcnt);
    free(ucnt);
    return tot;
  }
  frowp[0] = 0;
  for (int i = 0; i < n; i++) frowp[i + 1] = (int)(frowp[i] + lcnt[i + 1] + 1 + ucnt[i]);
  /* fill: L part of row i sorted, diagonal, then U part (entries (j, i) of
     L appended to row j in increasing i) */
  int *upos = (int *)malloc(sizeof(int) * (size_t)n);
  for (int i = 0; i < n; i++) {
    upos[i] = frowp[i] + (int)lcnt[i + 1] + 1;
    mark[i] = -1;
  }
  int *buf = (int *)malloc(sizeof(int) * (size_t)n);
  for (int i = 0; i < n; i++) {
    mark[i] = i;
    int nb = 0;
    for (int p = rowp[i]; p < rowp[i + 1]; p++) {
      int j = cols[p];
      if (j >= i) continue;
      while (mark[j] != i) {
        mark[j] = i;
        buf[nb++] = j;
        j = parent[j];
      }
    }
    /* sort the row's L columns */
    for (int a = 1; a < nb; a++) {
      const int v = buf[a];
      int b = a - 1;
      while (b >= 0 && buf[b] > v) {
        buf[b + 1] = buf[b];
        b--;
      }
      buf[b + 1] = v;
    }
    int *row = fcols + frowp[i];
    for (int a = 0; a < nb; a++) row[a] = buf[a];
    row[nb] = i;
    for (int a = 0; a < nb; a++) fcols[upos[buf[a]]++] = i;
  }
  free(buf);
  free(upos);
  free(parent);
  free(anc);
  free(mark);
  free(lcnt);
  free(ucnt);
  return tot;
}

/* ------------------------------------------------------ numeric factor */
int orc_inv6(const double *A, double *Ainv); /* solver_oracle.c */

static inline void mul66(const double *a, const double *b, double *d) {
  for (int r = 0; r < 6; r++)
    for (int c = 0; c < 6; c++) {
      double s = 0.0;
      for (int k = 0; k < 6; k++) s += a[6 * r + k] * b[6 * k + c];
      d[6 * r + c] = s;
    }
}
static inline void sub_mul66(const double *d, const double *u, double *t) {
  for (int r = 0; r < 6; r++)
    for (int c = 0; c < 6; c++) {
      double s = 0.0;
      for (int q = 0; q < 6; q++) s += d[6 * r + q] * u[6 * q + c];
      t[6 * r + c] -= s;
    }
}

/* Dependency levels of the rows: level[i] = 1 + max over L columns j.
   Returns the number of levels; lev_ptr[nlev+1], lev_rows[n]. */
int orc_factor_levels(int n, const int *frowp, const int *fcols, const int *fdiag, int upper,
                      int *lev_ptr, int *lev_rows) {
  int *lev = (int *)malloc(sizeof(int) * (size_t)n);
  int nl = 0;
  if (!upper) {
    for (int i = 0; i < n; i++) {
      int l = 0;
      for (int k = frowp[i]; k < fdiag[i]; k++) {
        const int v = lev[fcols[k]] + 1;
        l = v > l ? v : l;
      }
      lev[i] = l;
      nl = l + 1 > nl ? l + 1 : nl;
    }
  } else {
    for (int i = n - 1; i >= 0; i--) {
      int l = 0;
      for (int k = fdiag[i] + 1; k < frowp[i + 1]; k++) {
        const int v = lev[fcols[k]] + 1;
        l = v > l ? v : l;
      }
      lev[i] = l;
      nl = l + 1 > nl ? l + 1 : nl;
    }
  }
  if (lev_ptr) {
    memset(lev_ptr, 0, sizeof(int) * (size_t)(nl + 1));
    for (int i = 0; i < n; i++) lev_ptr[lev[i] + 1]++;
    for (int l = 0; l < nl; l++) lev_ptr[l + 1] += lev_ptr[l];
    int *fill = (int *)malloc(sizeof(int) * (size_t)(nl + 1));
    memcpy(fill, lev_ptr, sizeof(int) * (size_t)(nl + 1));
    for (int i = 0; i < n; i++) lev_rows[fill[lev[i]]++] = i;
    free(fill);
  }
  free(lev);
  return nl;
}

/* In-place IKJ factorization of F (pattern frowp/fcols/fdiag) over the
   dependency levels; returns 0 or 1 + the row of a singular pivot. */
int orc_factor_par(int n, const int *frowp, const int *fcols, const int *fdiag, int nlev,
                   const int *lev_ptr, const int *lev_rows, double *F) {
  const int nt = omp_get_max_threads();
  int *posmap = (int *)malloc(sizeof(int) * (size_t)n * (size_t)nt);
  for (size_t k = 0; k < (size_t)n * nt; k++) posmap[k] = -1;
  int bad = 0;
  for (int l = 0; l < nlev && !bad; l++) {
    const int r0 = lev_ptr[l], r1 = lev_ptr[l + 1];
    if (r1 - r0 >= 2 * nt) {
      /* many rows: one row per thread at a time */
#pragma omp parallel for schedule(dynamic, 1)
      for (int q = r0; q < r1; q++) {
        const int i = lev_rows[q];
        int *pm = posmap + (size_t)omp_get_thread_num() * n;
        for (int k = frowp[i]; k < frowp[i + 1]; k++) pm[fcols[k]] = k;
        for (int j = frowp[i]; j < fdiag[i]; j++) {
          const int cj = fcols[j];
          double d[36];
          mul66(F + (size_t)j * 36, F + (size_t)fdiag[cj] * 36, d);
          memcpy(F + (size_t)j * 36, d, sizeof(d));
          for (int p = fdiag[cj] + 1; p < frowp[cj + 1]; p++) {
            const int k = pm[fcols[p]];
            if (k >= 0) sub_mul66(d, F + (size_t)p * 36, F + (size_t)k * 36);
          }
        }
        double inv[36];
        if (orc_inv6(F + (size_t)fdiag[i] * 36, inv)) {
#pragma omp atomic write
          bad = i + 1;
        } else {
          memcpy(F + (size_t)fdiag[i] * 36, inv, sizeof(inv));
        }
        for (int k = frowp[i]; k < frowp[i + 1]; k++) pm[fcols[k]] = -1;
      }
    } else {
      /* few (long) rows: each pivot's U row split over the threads */
      for (int q = r0; q < r1 && !bad; q++) {
        const int i = lev_rows[q];
        int *pm = posmap;
        for (int k = frowp[i]; k < frowp[i + 1]; k++) pm[fcols[k]] = k;
        double d[36];
#pragma omp parallel
        for (int j = frowp[i]; j < fdiag[i]; j++) {
          const int cj = fcols[j];
#pragma omp single
          {
            mul66(F + (size_t)j * 36, F + (size_t)fdiag[cj] * 36, d);
            memcpy(F + (size_t)j * 36, d, sizeof(d));
          }
#pragma omp for schedule(static)
          for (int p = fdiag[cj] + 1; p < frowp[cj + 1]; p++) {
            const int k = pm[fcols[p]];
            if (k >= 0) sub_mul66(d, F + (size_t)p * 36, F + (size_t)k * 36);
          }
        }
        double inv[36];
        if (orc_inv6(F + (size_t)fdiag[i] * 36, inv))
          bad = i + 1;
        else
          memcpy(F + (size_t)fdiag[i] * 36, inv, sizeof(inv));
        for (int k = frowp[i]; k < frowp[i + 1]; k++) pm[fcols[k]] = -1;
      }
    }
  }
  free(posmap);
  return bad;
}

/* ---------------------------------------------------- triangular solves */
/* y = (LU)^-1 x for p right-hand sides ((row, dof, rhs) layout), over the
   lower and upper dependency levels; y may alias x. */
void orc_apply_factor_par(int n, const int *frowp, const int *fcols, const int *fdiag,
                          const double *F, int nlo, const int *lo_ptr, const int *lo_rows,
                          int nup, const int *up_ptr, const int *up_rows, int p, const double *x,
                          double *y) {
  const int w = 6 * p;
  const int nt = omp_get_max_threads();
  double *part = (double *)malloc(sizeof(double) * (size_t)w * nt);
  for (int pass = 0; pass < 2; pass++) {
    const int upper = pass == 1;
    const int nl = upper ? nup : nlo;
    const int *ptr = upper ? up_ptr : lo_ptr, *rows = upper ? up_rows : lo_rows;
    for (int l = 0; l < nl; l++) {
      const int r0 = ptr[l], r1 = ptr[l + 1];
      if (r1 - r0 >= 2 * nt) {
#pragma omp parallel for schedule(dynamic, 16)
        for (int q = r0; q < r1; q++) {
          const int i = rows[q];
          double z[96];
          const double *src = upper ? y : x;
          for (int e = 0; e < w; e++) z[e] = src[(size_t)i * w + e];
          const int kb = upper ? fdiag[i] + 1 : frowp[i], ke = upper ? frowp[i + 1] : fdiag[i];
          for (int k = kb; k < ke; k++) {
            const double *a = F + (size_t)k * 36, *yy = y + (size_t)fcols[k] * w;
            for (int r = 0; r < 6; r++)
              for (int c = 0; c < 6; c++) {
                const double m = a[6 * r + c];
                for (int h = 0; h < p; h++) z[r * p + h] -= m * yy[c * p + h];
              }
          }
          if (upper) {
            const double *dinv = F + (size_t)fdiag[i] * 36;
            for (int r = 0; r < 6; r++)
              for (int h = 0; h < p; h++) {
                double s = 0.0;
                for (int c = 0; c < 6; c++) s += dinv[6 * r + c] * z[c * p + h];
                y[(size_t)i * w + r * p + h] = s;
              }
          } else {
            for (int e = 0; e < w; e++) y[(size_t)i * w + e] = z[e];
          }
        }
      } else {
        for (int q = r0; q < r1; q++) {
          const int i = rows[q];
          const int kb = upper ? fdiag[i] + 1 : frowp[i], ke = upper ? frowp[i + 1] : fdiag[i];
#pragma omp parallel
          {
            double *zt = part + (size_t)omp_get_thread_num() * w;
            for (int e = 0; e < w; e++) zt[e] = 0.0;
#pragma omp for schedule(static)
            for (int k = kb; k < ke; k++) {
              const double *a = F + (size_t)k * 36, *yy = y + (size_t)fcols[k] * w;
              for (int r = 0; r < 6; r++)
                for (int c = 0; c < 6; c++) {
                  const double m = a[6 * r + c];
                  for (int h = 0; h < p; h++) zt[r * p + h] += m * yy[c * p + h];
                }
            }
          }
          double z[96];
          const double *src = upper ? y : x;
          for (int e = 0; e < w; e++) {
            double s = 0.0;
            for (int t = 0; t < nt; t++) s += part[(size_t)t * w + e];
            z[e] = src[(size_t)i * w + e] - s;
          }
          if (upper) {
            const double *dinv = F + (size_t)fdiag[i] * 36;
            for (int r = 0; r < 6; r++)
              for (int h = 0; h < p; h++) {
                double s = 0.0;
                for (int c = 0; c < 6; c++) s += dinv[6 * r + c] * z[c * p + h];
                y[(size_t)i * w + r * p + h] = s;
              }
          } else {
            for (int e = 0; e < w; e++) y[(size_t)i * w + e] = z[e];
          }
        }
      }
    }
  }
  free(part);
}

/* Y = A X (B == NULL) or Y = B - A X for p right-hand sides. */
void orc_spmm(int n, const int *rowp, const int *cols, const double *A, int p, const double *X,
              const double *B, double *Y) {
  const int w = 6 * p;
#pragma omp parallel for schedule(static)
  for (int i = 0; i < n; i++) {
    double z[96];
    for (int e = 0; e < w; e++) z[e] = 0.0;
    for (int k = rowp[i]; k < rowp[i + 1]; k++) {
      const double *a = A + (size_t)k * 36, *xx = X + (size_t)cols[k] * w;
      for (int r = 0; r < 6; r++)
        for (int c = 0; c < 6; c++) {
          const double m = a[6 * r + c];
          for (int h = 0; h < p; h++) z[r * p + h] += m * xx[c * p + h];
        }
    }
    for (int e = 0; e < w; e++) Y[(size_t)i * w + e] = B ? B[(size_t)i * w + e] - z[e] : z[e];
  }
}
