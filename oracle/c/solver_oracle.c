/*
  CPU restatement of the reference's assembly and buckling-solve path
  (TEST INFRASTRUCTURE ONLY -- the checker and the timed CPU baseline).

  Follows:
    TACSAssembler::assembleMatType   src/TACSAssembler.cpp:4186-4257
      (element loop, scatter by binary search: TACSSchurMat::addValues
       src/bpmat/TACSSchurMat.cpp:453, BCSRMat::addRowValues
       src/bpmat/BCSRMat.cpp:1778)
    BCSRMat::zeroRow (row-only Dirichlet)          src/bpmat/BCSRMat.cpp:2005
    BCSRMatFactor6 (IKJ block LU, inverted diag)   src/bpmat/BCSRMatFact6.cpp:946
    BCSRMatApplyLower6 / Upper6                    src/bpmat/BCSRMatMult6.cpp:319-416
    BCSRMatVecMult6                                src/bpmat/BCSRMatMult6.cpp:82
    GMRES::solve (right preconditioned, MGS)       src/bpmat/KSM.cpp:785-970
    TACSLinearBuckling::solve                      src/TACSBuckling.cpp:197-278
    SEP::solve (FULL orthogonalisation)            src/bpmat/GSEP.cpp:485-596
    EPBucklingShiftInvert (mult/dot/convert)       src/bpmat/GSEP.cpp:224-244

  The element routines are in shell_element.c.  The BCSR pattern (rows in
  the matrix ordering), the permutation and the factor pattern are inputs.
*/
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "shell_oracle.h"

/* ------------------------------------------------------------- assembly */
static int find_block(const int *rowp, const int *cols, int row, int col) {
  int lo = rowp[row], hi = rowp[row + 1] - 1;
  while (lo <= hi) {
    int mid = (lo + hi) / 2;
    if (cols[mid] == col) return mid;
    if (cols[mid] < col)
      lo = mid + 1;
    else
      hi = mid - 1;
  }
  return -1;
}

/* conn_rows: element connectivity mapped to matrix rows; X_nodes/vars in
   the caller's node numbering via conn_nodes.  vals (36 per block) is
   zeroed here.  kind: ORC_STIFFNESS or ORC_GEOMETRIC. */
void orc_assemble(int order, int nl, int kind, const orc_material *mat0, int nrows, int ne,
                  const int *conn_nodes, const int *conn_rows, const double *X, const double *vars,
                  const double *tvals, const int *tgroup, const int *rowp, const int *cols,
                  double *vals) {
  const int nn = order * order, nv = 6 * nn;
  memset(vals, 0, sizeof(double) * 36 * (size_t)rowp[nrows]);
#pragma omp parallel
  {
    double Xe[27], ve[54], Ke[54 * 54];
#pragma omp for schedule(dynamic, 64)
    for (int e = 0; e < ne; e++) {
      orc_material m = *mat0;
      m.t = tvals[tgroup ? tgroup[e] : 0];
      for (int a = 0; a < nn; a++) {
        int node = conn_nodes[e * nn + a];
        for (int c = 0; c < 3; c++) Xe[3 * a + c] = X[3 * node + c];
        for (int c = 0; c < 6; c++) ve[6 * a + c] = vars ? vars[6 * node + c] : 0.0;
      }
      orc_get_mat_type(order, nl, kind, &m, Xe, ve, Ke);
      for (int a = 0; a < nn; a++) {
        int r = conn_rows[e * nn + a];
        for (int b = 0; b < nn; b++) {
          int c = conn_rows[e * nn + b];
          int p = find_block(rowp, cols, r, c);
          double *blk = vals + (size_t)p * 36;
          for (int ii = 0; ii < 6; ii++)
            for (int jj = 0; jj < 6; jj++) {
#pragma omp atomic
              blk[6 * ii + jj] += Ke[(6 * a + ii) * nv + 6 * b + jj];
            }
        }
      }
    }
  }
}

void orc_apply_bcs(const int *rowp, const int *cols, double *vals, int nbc, const int *bc_rows,
                   const int *bc_masks) {
  for (int b = 0; b < nbc; b++) {
    int row = bc_rows[b];
    for (int j = rowp[row]; j < rowp[row + 1]; j++) {
      double *a = vals + (size_t)j * 36;
      for (int ii = 0; ii < 6; ii++)
        if (bc_masks[b] & (1 << ii)) {
          for (int jj = 0; jj < 6; jj++) a[6 * ii + jj] = 0.0;
          if (cols[j] == row) a[7 * ii] = 1.0;
        }
    }
  }
}

/* ----------------------------------------------------------- BCSR algebra */
void orc_spmv(int n, const int *rowp, const int *cols, const double *A, const double *x,
              double *y) {
#pragma omp parallel for schedule(static)
  for (int i = 0; i < n; i++) {
    double s[6] = {0, 0, 0, 0, 0, 0};
    for (int j = rowp[i]; j < rowp[i + 1]; j++) {
      const double *a = A + (size_t)j * 36, *xx = x + 6 * (size_t)cols[j];
      for (int r = 0; r < 6; r++)
        s[r] += a[6 * r] * xx[0] + a[6 * r + 1] * xx[1] + a[6 * r + 2] * xx[2] +
                a[6 * r + 3] * xx[3] + a[6 * r + 4] * xx[4] + a[6 * r + 5] * xx[5];
    }
    for (int r = 0; r < 6; r++) y[6 * (size_t)i + r] = s[r];
  }
}

/* 6x6 inverse with partial pivoting (as BMatComputeInverse's result) */
static int inv6(const double *A, double *Ainv) {
  double M[36], I[36];
  for (int k = 0; k < 36; k++) {
    M[k] = A[k];
    I[k] = (k % 7 == 0) ? 1.0 : 0.0;
  }
  for (int c = 0; c < 6; c++) {
    int p = c;
    double best = fabs(M[7 * c]);
    for (int r = c + 1; r < 6; r++)
      if (fabs(M[6 * r + c]) > best) {
        best = fabs(M[6 * r + c]);
        p = r;
      }
    if (best == 0.0) return c + 1;
    if (p != c)
      for (int k = 0; k < 6; k++) {
        double t = M[6 * c + k];
        M[6 * c + k] = M[6 * p + k];
        M[6 * p + k] = t;
        t = I[6 * c + k];
        I[6 * c + k] = I[6 * p + k];
        I[6 * p + k] = t;
      }
    double inv = 1.0 / M[7 * c];
    for (int k = 0; k < 6; k++) {
      M[6 * c + k] *= inv;
      I[6 * c + k] *= inv;
    }
    for (int r = 0; r < 6; r++) {
      if (r == c) continue;
      double f = M[6 * r + c];
      for (int k = 0; k < 6; k++) {
        M[6 * r + k] -= f * M[6 * c + k];
        I[6 * r + k] -= f * I[6 * c + k];
      }
    }
  }
  memcpy(Ainv, I, sizeof(I));
  return 0;
}

/* the 6x6 inverse above, for the multi-threaded factorization (cpu_parallel.c) */
int orc_inv6(const double *A, double *Ainv) { return inv6(A, Ainv); }

/* Copy A (pattern rowp/cols) into the factor pattern F (frowp/fcols). */
void orc_factor_fill(int n, const int *rowp, const int *cols, const double *A, const int *frowp,
                     const int *fcols, double *F) {
  memset(F, 0, sizeof(double) * 36 * (size_t)frowp[n]);
  for (int i = 0; i < n; i++)
    for (int j = rowp[i]; j < rowp[i + 1]; j++) {
      int p = find_block(frowp, fcols, i, cols[j]);
      memcpy(F + (size_t)p * 36, A + (size_t)j * 36, 36 * sizeof(double));
    }
}

/* BCSRMatFactor6: row i eliminated left to right (IKJ), L_ij = A_ij D_j^-1,
   A_ik -= L_ij U_jk on the pattern (merge scan), diagonal inverted last. */
int orc_factor(int n, const int *frowp, const int *fcols, const int *fdiag, double *F) {
  for (int i = 0; i < n; i++) {
    const int kend = frowp[i + 1];
    for (int j = frowp[i]; fcols[j] < i; j++) {
      const int cj = fcols[j];
      double *a = F + (size_t)j * 36;
      const double *b = F + (size_t)fdiag[cj] * 36;
      double d[36];
      for (int r = 0; r < 6; r++)
        for (int c = 0; c < 6; c++) {
          double s = 0.0;
          for (int k = 0; k < 6; k++) s += a[6 * r + k] * b[6 * k + c];
          d[6 * r + c] = s;
        }
      memcpy(a, d, sizeof(d));
      int k = j + 1;
      const int pend = frowp[cj + 1];
      for (int p = fdiag[cj] + 1; p < pend && k < kend; p++) {
        while (k < kend && fcols[k] < fcols[p]) k++;
        if (k < kend && fcols[k] == fcols[p]) {
          const double *u = F + (size_t)p * 36;
          double *t = F + (size_t)k * 36;
          for (int r = 0; r < 6; r++)
            for (int c = 0; c < 6; c++) {
              double s = 0.0;
              for (int q = 0; q < 6; q++) s += d[6 * r + q] * u[6 * q + c];
              t[6 * r + c] -= s;
            }
        }
      }
    }
    double inv[36];
    if (inv6(F + (size_t)fdiag[i] * 36, inv)) return i + 1;
    memcpy(F + (size_t)fdiag[i] * 36, inv, sizeof(inv));
  }
  return 0;
}

/* BCSRMatApplyLower6 + BCSRMatApplyUpper6: y = (LU)^-1 x */
void orc_apply_factor(int n, const int *frowp, const int *fcols, const int *fdiag,
                      const double *F, const double *x, double *y) {
  for (int i = 0; i < n; i++) {
    double z[6];
    for (int r = 0; r < 6; r++) z[r] = x[6 * (size_t)i + r];
    for (int k = frowp[i]; k < fdiag[i]; k++) {
      const double *a = F + (size_t)k * 36, *yy = y + 6 * (size_t)fcols[k];
      for (int r = 0; r < 6; r++)
        z[r] -= a[6 * r] * yy[0] + a[6 * r + 1] * yy[1] + a[6 * r + 2] * yy[2] +
                a[6 * r + 3] * yy[3] + a[6 * r + 4] * yy[4] + a[6 * r + 5] * yy[5];
    }
    for (int r = 0; r < 6; r++) y[6 * (size_t)i + r] = z[r];
  }
  for (int i = n - 1; i >= 0; i--) {
    double z[6];
    for (int r = 0; r < 6; r++) z[r] = y[6 * (size_t)i + r];
    for (int k = fdiag[i] + 1; k < frowp[i + 1]; k++) {
      const double *a = F + (size_t)k * 36, *yy = y + 6 * (size_t)fcols[k];
      for (int r = 0; r < 6; r++)
        z[r] -= a[6 * r] * yy[0] + a[6 * r + 1] * yy[1] + a[6 * r + 2] * yy[2] +
                a[6 * r + 3] * yy[3] + a[6 * r + 4] * yy[4] + a[6 * r + 5] * yy[5];
    }
    const double *d = F + (size_t)fdiag[i] * 36;
    for (int r = 0; r < 6; r++) {
      double s = 0.0;
      for (int c = 0; c < 6; c++) s += d[6 * r + c] * z[c];
      y[6 * (size_t)i + r] = s;
    }
  }
}

/* ----------------------------------------------------------- vector ops */
static double dot(size_t n, const double *x, const double *y) {
  double s = 0.0;
#pragma omp parallel for reduction(+ : s)
  for (long long i = 0; i < (long long)n; i++) s += x[i] * y[i];
  return s;
}
static void axpy(size_t n, double a, const double *x, double *y) {
#pragma omp parallel for
  for (long long i = 0; i < (long long)n; i++) y[i] += a * x[i];
}
static void zero_bc(double *x, int nbc, const int *bc_rows, const int *bc_masks) {
  for (int b = 0; b < nbc; b++)
    for (int k = 0; k < 6; k++)
      if (bc_masks[b] & (1 << k)) x[6 * (size_t)bc_rows[b] + k] = 0.0;
}

typedef struct {
  int n;
  const int *rowp, *cols;
  const double *A;  /* operator */
  const int *frowp, *fcols, *fdiag;
  const double *F;  /* preconditioner factor */
} orc_system;

/* GMRES::solve: right-preconditioned restarted GMRES(m) with modified
   Gram-Schmidt and Givens rotations; stops on rtol*|r0| or atol.  Returns
   the number of iterations. */
int orc_gmres(const orc_system *S, int m, int nrestart, double rtol, double atol,
              const double *b, double *x) {
  const size_t N = 6 * (size_t)S->n;
  double *W = (double *)malloc(sizeof(double) * N * (m + 1));
  double *Z = (double *)malloc(sizeof(double) * N);
  double *H = (double *)calloc((size_t)(m + 1) * m, sizeof(double));
  double *res = (double *)calloc(m + 1, sizeof(double));
  double *cs = (double *)calloc(m, sizeof(double)), *sn = (double *)calloc(m, sizeof(double));
  int total = 0;
  memset(x, 0, sizeof(double) * N);
  double rnorm0 = 0.0;
  for (int rs = 0; rs <= nrestart; rs++) {
    /* r = b - A x */
    orc_spmv(S->n, S->rowp, S->cols, S->A, x, W);
    for (size_t i = 0; i < N; i++) W[i] = b[i] - W[i];
    double beta = sqrt(dot(N, W, W));
    if (rs == 0) rnorm0 = beta;
    if (beta <= atol || beta <= rtol * rnorm0) break;
    for (size_t i = 0; i < N; i++) W[i] /= beta;
    memset(res, 0, sizeof(double) * (m + 1));
    res[0] = beta;
    int k = 0, done = 0;
    for (; k < m; k++) {
      orc_apply_factor(S->n, S->frowp, S->fcols, S->fdiag, S->F, W + N * k, Z);
      orc_spmv(S->n, S->rowp, S->cols, S->A, Z, W + N * (k + 1));
      for (int j = 0; j <= k; j++) {
        double h = dot(N, W + N * (k + 1), W + N * j);
        axpy(N, -h, W + N * j, W + N * (k + 1));
        H[j + (m + 1) * k] = h;
      }
      double hn = sqrt(dot(N, W + N * (k + 1), W + N * (k + 1)));
      H[k + 1 + (m + 1) * k] = hn;
      if (hn != 0.0)
        for (size_t i = 0; i < N; i++) W[N * (k + 1) + i] /= hn;
      for (int j = 0; j < k; j++) {
        double h1 = H[j + (m + 1) * k], h2 = H[j + 1 + (m + 1) * k];
        H[j + (m + 1) * k] = cs[j] * h1 + sn[j] * h2;
        H[j + 1 + (m + 1) * k] = -sn[j] * h1 + cs[j] * h2;
      }
      double h1 = H[k + (m + 1) * k], h2 = H[k + 1 + (m + 1) * k];
      double den = sqrt(h1 * h1 + h2 * h2);
      cs[k] = den != 0.0 ? h1 / den : 1.0;
      sn[k] = den != 0.0 ? h2 / den : 0.0;
      H[k + (m + 1) * k] = den;
      H[k + 1 + (m + 1) * k] = 0.0;
      res[k + 1] = -sn[k] * res[k];
      res[k] = cs[k] * res[k];
      total++;
      if (fabs(res[k + 1]) <= atol || fabs(res[k + 1]) <= rtol * rnorm0) {
        done = 1;
        k++;
        break;
      }
    }
    /* back substitution and x += M^-1 (W y) */
    double *y = (double *)calloc(k > 0 ? k : 1, sizeof(double));
    for (int i = k - 1; i >= 0; i--) {
      double s = res[i];
      for (int j = i + 1; j < k; j++) s -= H[i + (m + 1) * j] * y[j];
      y[i] = s / H[i + (m + 1) * i];
    }
    memset(Z, 0, sizeof(double) * N);
    for (int j = 0; j < k; j++) axpy(N, y[j], W + N * j, Z);
    double *t = (double *)malloc(sizeof(double) * N);
    orc_apply_factor(S->n, S->frowp, S->fcols, S->fdiag, S->F, Z, t);
    axpy(N, 1.0, t, x);
    free(t);
    free(y);
    if (done) break;
  }
  free(W);
  free(Z);
  free(H);
  free(res);
  free(cs);
  free(sn);
  return total;
}

/* Cyclic Jacobi eigen-solver of a small dense symmetric matrix (the
   reference calls LAPACK dstevr on the tridiagonal). */
static void small_eig(int m, double *A, double *w, double *V) {
  for (int i = 0; i < m * m; i++) V[i] = (i % (m + 1) == 0) ? 1.0 : 0.0;
  for (int sweep = 0; sweep < 100; sweep++) {
    double off = 0.0, tot = 0.0;
    for (int i = 0; i < m * m; i++) {
      tot += A[i] * A[i];
      if (i % (m + 1)) off += A[i] * A[i];
    }
    if (off <= 1e-30 * tot) break;
    for (int p = 0; p < m - 1; p++)
      for (int q = p + 1; q < m; q++) {
        double apq = A[p * m + q];
        if (apq == 0.0) continue;
        double theta = (A[q * m + q] - A[p * m + p]) / (2.0 * apq);
        double t = (theta >= 0 ? 1.0 : -1.0) / (fabs(theta) + sqrt(theta * theta + 1.0));
        double c = 1.0 / sqrt(t * t + 1.0), s = t * c;
        for (int k = 0; k < m; k++) {
          double akp = A[k * m + p], akq = A[k * m + q];
          A[k * m + p] = c * akp - s * akq;
          A[k * m + q] = s * akp + c * akq;
        }
        for (int k = 0; k < m; k++) {
          double apk = A[p * m + k], aqk = A[q * m + k];
          A[p * m + k] = c * apk - s * aqk;
          A[q * m + k] = s * apk + c * aqk;
        }
        for (int k = 0; k < m; k++) {
          double vkp = V[k * m + p], vkq = V[k * m + q];
          V[k * m + p] = c * vkp - s * vkq;
          V[k * m + q] = s * vkp + c * vkq;
        }
      }
  }
  for (int i = 0; i < m; i++) w[i] = A[i * m + i];
}

/* SEP::solve with EPBucklingShiftInvert (FULL orthogonalisation): the
   operator is y = A^{-1} K x by GMRES on A = K + sigma G preconditioned by
   the factor of K; every K-inner product is a K SpMV plus a dot.  Runs
   exactly `iters` steps (the reference's checkConverged returns 1 once
   n >= neigvals).  Outputs the num_eig buckling loads with the smallest
   magnitude.  Returns the total GMRES iterations. */
int orc_lanczos(const orc_system *Aop, int n, const int *rowp, const int *cols, const double *K,
                double sigma, int iters, int gm_m, int gm_restarts, double gm_tol, int nbc,
                const int *bc_rows, const int *bc_masks, unsigned seed, int num_eig,
                double *eigvals) {
  const size_t N = 6 * (size_t)n;
  double *Q = (double *)malloc(sizeof(double) * N * (iters + 1));
  double *t = (double *)malloc(sizeof(double) * N);
  double *alpha = (double *)calloc(iters, sizeof(double)), *beta = (double *)calloc(iters, sizeof(double));
  unsigned long long s = 0x9E3779B97F4A7C15ull * (seed + 1);
  for (size_t i = 0; i < N; i++) {
    unsigned long long z = (s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    z ^= z >> 31;
    Q[i] = (double)(z >> 11) * (1.0 / 9007199254740992.0);
  }
  zero_bc(Q, nbc, bc_rows, bc_masks);
  orc_spmv(n, rowp, cols, K, Q, t);
  double nrm = sqrt(dot(N, Q, t));
  for (size_t i = 0; i < N; i++) Q[i] /= nrm;
  int gm_total = 0;
  for (int i = 0; i < iters; i++) {
    double *qi = Q + N * i, *w = Q + N * (i + 1);
    orc_spmv(n, rowp, cols, K, qi, t);
    gm_total += orc_gmres(Aop, gm_m, gm_restarts, gm_tol, gm_tol, t, w);
    zero_bc(w, nbc, bc_rows, bc_masks);
    for (int j = i; j >= 0; j--) {
      orc_spmv(n, rowp, cols, K, Q + N * j, t); /* <w, q_j>_K: one SpMV per dot */
      double h = dot(N, w, t);
      axpy(N, -h, Q + N * j, w);
      if (j == i) alpha[i] = h;
    }
    orc_spmv(n, rowp, cols, K, w, t);
    beta[i] = sqrt(dot(N, w, t));
    for (size_t k = 0; k < N; k++) w[k] /= beta[i];
  }
  /* Ritz values of the tridiagonal, lambda = -mu sigma/(1-mu) */
  int m = iters;
  double *T = (double *)calloc((size_t)m * m, sizeof(double)), *V = (double *)malloc(sizeof(double) * m * m),
         *mu = (double *)malloc(sizeof(double) * m);
  for (int k = 0; k < m; k++) {
    T[k * m + k] = alpha[k];
    if (k + 1 < m) T[k * m + k + 1] = T[(k + 1) * m + k] = beta[k];
  }
  small_eig(m, T, mu, V);
  double *lam = (double *)malloc(sizeof(double) * m);
  for (int k = 0; k < m; k++) lam[k] = -mu[k] * sigma / (1.0 - mu[k]);
  /* selection by smallest |lambda| */
  for (int k = 0; k < num_eig && k < m; k++) {
    int best = -1;
    for (int q = 0; q < m; q++)
      if (lam[q] == lam[q] && (best < 0 || fabs(lam[q]) < fabs(lam[best]))) best = q;
    eigvals[k] = lam[best];
    lam[best] = NAN;
  }
  free(Q);
  free(t);
  free(alpha);
  free(beta);
  free(T);
  free(V);
  free(mu);
  free(lam);
  return gm_total;
}
