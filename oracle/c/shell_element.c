/*
  CPU restatement of the reference's director-based MITC shell element
  (TEST INFRASTRUCTURE ONLY -- the checker, never the product).

  Follows, function by function, the reference's header-only templates for
  TACSShellElement<quadrature, TACSShellQuadBasis<order>,
  TACSLinearizedRotation, TACSShellLinearModel | TACSShellNonlinearModel>,
  with the node count a run-time argument (order 2 = Quad4, 3 = Quad9).
  Each routine cites the reference function it restates.
*/
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "shell_oracle.h"

#define MAXO 3
#define MAXN 9
#define MAXV 54
#define MAXTY 28
#define MAXD 27 /* 3*MAXN */

/* ---------------------------------------------------------------- quadrature
   TACSGaussQuadrature.h:23-29 (15-digit literals kept as in the reference) */
static const double GP2[2] = {-0.577350269189626, 0.577350269189626};
static const double GW2[2] = {1.0, 1.0};
static const double GP3[3] = {-0.774596669241483, 0.0, 0.774596669241483};
static const double GW3[3] = {5.0 / 9.0, 8.0 / 9.0, 5.0 / 9.0};
static const double GP1[1] = {0.0};
static const double LINTY[2] = {-1.0, 1.0}; /* TacsShellLinearTyingPoints */

/* TACSQuadLinearQuadrature / TACSQuadQuadraticQuadrature::getQuadraturePoint
   (TACSShellElementQuadrature.h:22-27, 71-76) */
static double quad_point(int order, int n, double pt[2]) {
  if (order == 2) {
    pt[0] = GP2[n % 2];
    pt[1] = GP2[n / 2];
    return GW2[n % 2] * GW2[n / 2];
  }
  pt[0] = GP3[n % 3];
  pt[1] = GP3[n / 3];
  return GW3[n % 3] * GW3[n / 3];
}

/* ------------------------------------------------------------------- basis */
/* TacsLagrangeLobattoShapeFuncDerivative (TACSShellElementQuadBasis.h:96-124) */
static void lobatto(int order, double u, double *N, double *Nd) {
  if (order == 2) {
    N[0] = 0.5 * (1.0 - u);
    N[1] = 0.5 * (1.0 + u);
    if (Nd) {
      Nd[0] = -0.5;
      Nd[1] = 0.5;
    }
  } else {
    N[0] = -0.5 * u * (1.0 - u);
    N[1] = (1.0 - u) * (1.0 + u);
    N[2] = 0.5 * (1.0 + u) * u;
    if (Nd) {
      Nd[0] = -0.5 + u;
      Nd[1] = -2.0 * u;
      Nd[2] = 0.5 + u;
    }
  }
}

/* TacsLagrangeShapeFunction (TACSShellElementQuadBasis.h:18-30) */
static void lagrange(int n, double u, const double *knots, double *N) {
  for (int i = 0; i < n; i++) {
    N[i] = 1.0;
    for (int j = 0; j < n; j++) {
      if (i != j) {
        double d = 1.0 / (knots[i] - knots[j]);
        N[i] *= (u - knots[j]) * d;
      }
    }
  }
}

/* TACSShellQuadBasis::getNodePoint (TACSShellElementQuadBasis.h:150-153) */
static void node_point(int order, int n, double pt[2]) {
  pt[0] = -1.0 + (2.0 / (order - 1)) * (n % order);
  pt[1] = -1.0 + (2.0 / (order - 1)) * (n / order);
}

/* interpFields<vpn, m> (TACSShellElementQuadBasis.h:172-192) */
static void interp(int order, int vpn, int m, const double pt[], const double *v,
                   double *f) {
  double na[MAXO], nb[MAXO];
  lobatto(order, pt[0], na, NULL);
  lobatto(order, pt[1], nb, NULL);
  for (int k = 0; k < m; k++) f[k] = 0.0;
  for (int j = 0; j < order; j++) {
    for (int i = 0; i < order; i++) {
      for (int k = 0; k < m; k++) f[k] += na[i] * nb[j] * v[k];
      v += vpn;
    }
  }
}

/* addInterpFieldsTranspose<vpn, m> (:194-209) */
static void interp_t(int order, int vpn, int m, const double pt[], const double *f,
                     double *v) {
  double na[MAXO], nb[MAXO];
  lobatto(order, pt[0], na, NULL);
  lobatto(order, pt[1], nb, NULL);
  for (int j = 0; j < order; j++) {
    for (int i = 0; i < order; i++) {
      for (int k = 0; k < m; k++) v[k] += na[i] * nb[j] * f[k];
      v += vpn;
    }
  }
}

/* interpFieldsGrad<vpn, m> (:211-234) */
static void interp_grad(int order, int vpn, int m, const double pt[], const double *v,
                        double *g) {
  double na[MAXO], dna[MAXO], nb[MAXO], dnb[MAXO];
  lobatto(order, pt[0], na, dna);
  lobatto(order, pt[1], nb, dnb);
  for (int k = 0; k < m; k++) g[2 * k] = g[2 * k + 1] = 0.0;
  for (int j = 0; j < order; j++) {
    for (int i = 0; i < order; i++) {
      for (int k = 0; k < m; k++) {
        g[2 * k] += dna[i] * nb[j] * v[k];
        g[2 * k + 1] += na[i] * dnb[j] * v[k];
      }
      v += vpn;
    }
  }
}

/* addInterpFieldsGradTranspose<vpn, m> (:236-253) */
static void interp_grad_t(int order, int vpn, int m, const double pt[], const double *g,
                          double *v) {
  double na[MAXO], dna[MAXO], nb[MAXO], dnb[MAXO];
  lobatto(order, pt[0], na, dna);
  lobatto(order, pt[1], nb, dnb);
  for (int j = 0; j < order; j++) {
    for (int i = 0; i < order; i++) {
      for (int k = 0; k < m; k++)
        v[k] += (dna[i] * nb[j] * g[2 * k] + na[i] * dnb[j] * g[2 * k + 1]);
      v += vpn;
    }
  }
}

/* addInterpFieldsOuterProduct<nbr, nbc, njr, njc> (:271-305):
   mat[(J*nbr + jm), (I*nbc + im)] += N_I N_J jac[jm*njc + im] */
static void outer(int order, int nbr, int nbc, int njr, int njc, const double pt[],
                  const double *jac, double *mat) {
  double na[MAXO], nb[MAXO];
  lobatto(order, pt[0], na, NULL);
  lobatto(order, pt[1], nb, NULL);
  const int nn = order * order;
  const int ncols = nn * nbc;
  for (int J = 0; J < nn; J++) {
    double Nj = na[J % order] * nb[J / order];
    for (int jm = 0; jm < njr; jm++) {
      double *row = &mat[(J * nbr + jm) * ncols];
      for (int I = 0; I < nn; I++) {
        double Ni = na[I % order] * nb[I / order];
        for (int im = 0; im < njc; im++) row[I * nbc + im] += Ni * Nj * jac[jm * njc + im];
      }
    }
  }
}

/* addInterpGradOuterProduct<nbr, nbc, njr, njc> (:322-367) */
static void grad_outer(int order, int nbr, int nbc, int njr, int njc, const double pt[],
                       const double *jac, double *mat) {
  double na[MAXO], dna[MAXO], nb[MAXO], dnb[MAXO];
  lobatto(order, pt[0], na, dna);
  lobatto(order, pt[1], nb, dnb);
  const int nn = order * order;
  const int ncols = nn * nbc;
  for (int J = 0; J < nn; J++) {
    double Naj = dna[J % order] * nb[J / order];
    double Nbj = na[J % order] * dnb[J / order];
    for (int jm = 0; jm < njr; jm++) {
      const double *jac1 = &jac[4 * njc * jm];
      const double *jac2 = &jac[4 * njc * jm + 2 * njc];
      double *row = &mat[(J * nbr + jm) * ncols];
      for (int I = 0; I < nn; I++) {
        double Nai = dna[I % order] * nb[I / order];
        double Nbi = na[I % order] * dnb[I / order];
        double Naa = Naj * Nai, Nab = Naj * Nbi, Nba = Nbj * Nai, Nbb = Nbj * Nbi;
        for (int im = 0; im < njc; im++) {
          row[I * nbc + im] += (Naa * jac1[2 * im] + Nab * jac1[2 * im + 1] +
                                Nba * jac2[2 * im] + Nbb * jac2[2 * im + 1]);
        }
      }
    }
  }
}

/* addInterpGradMixedOuterProduct<nbr, nbc, njr, njc> (:388-486) */
static void grad_mixed_outer(int order, int nbr, int nbc, int njr, int njc,
                             const double pt[], const double *jac, const double *jacT,
                             double *mat) {
  double na[MAXO], dna[MAXO], nb[MAXO], dnb[MAXO];
  lobatto(order, pt[0], na, dna);
  lobatto(order, pt[1], nb, dnb);
  const int nn = order * order;
  const int ncols = nn * nbc;
  for (int J = 0; J < nn; J++) {
    double Nj = na[J % order] * nb[J / order];
    double Naj = dna[J % order] * nb[J / order];
    double Nbj = na[J % order] * dnb[J / order];
    for (int jm = 0; jm < njr; jm++) {
      double *row = &mat[(J * nbr + jm) * ncols];
      for (int I = 0; I < nn; I++) {
        double Ni = na[I % order] * nb[I / order];
        double Nai = dna[I % order] * nb[I / order];
        double Nbi = na[I % order] * dnb[I / order];
        for (int im = 0; im < njc; im++) {
          double v = 0.0;
          if (jac) v += Nj * Nai * jac[2 * njc * jm + 2 * im] +
                        Nj * Nbi * jac[2 * njc * jm + 2 * im + 1];
          if (jacT) v += Ni * Naj * jacT[2 * njc * im + 2 * jm] +
                         Ni * Nbj * jacT[2 * njc * im + 2 * jm + 1];
          row[I * nbc + im] += v;
        }
      }
    }
  }
}

/* ------------------------------------------------------------ tying points
   TACSShellQuadBasis tying layout (:125-142, 487-621):
   fields in the order G11, G22, G12, G23, G13 */
enum { F11 = 0, F22 = 1, F12 = 2, F23 = 3, F13 = 4 };

static int ntying_field(int order, int f) {
  if (f == F12) return (order - 1) * (order - 1);
  return order * (order - 1);
}
static int ntying(int order) {
  int n = 0;
  for (int f = 0; f < 5; f++) n += ntying_field(order, f);
  return n;
}
static void tying_knots(int order, const double **ko, const double **kr) {
  if (order == 2) {
    *ko = LINTY;
    *kr = GP1;
  } else {
    *ko = GP3;
    *kr = GP2;
  }
}
/* getTyingField (:490-502) */
static int tying_field(int order, int index) {
  int off = 0;
  for (int f = 0; f < 5; f++) {
    off += ntying_field(order, f);
    if (index < off) return f;
  }
  return F13;
}
/* getTyingPoint (:530-567) */
static void tying_point(int order, int index, double pt[2]) {
  const double *ko, *kr;
  tying_knots(order, &ko, &kr);
  int f = 0, off = 0;
  while (index >= off + ntying_field(order, f)) off += ntying_field(order, f++);
  int ty = index - off;
  if (f == F11 || f == F13) {
    pt[0] = kr[ty % (order - 1)];
    pt[1] = ko[ty / (order - 1)];
  } else if (f == F22 || f == F23) {
    pt[0] = ko[ty % order];
    pt[1] = kr[ty / order];
  } else {
    pt[0] = kr[ty % (order - 1)];
    pt[1] = kr[ty / (order - 1)];
  }
}
/* evalTyingInterp (:569-621) */
static void tying_interp(int order, const double pt[], double *N) {
  const double *ko, *kr;
  tying_knots(order, &ko, &kr);
  double na[MAXO], nb[MAXO], nar[MAXO], nbr[MAXO];
  lagrange(order, pt[0], ko, na);
  lagrange(order, pt[1], ko, nb);
  lagrange(order - 1, pt[0], kr, nar);
  lagrange(order - 1, pt[1], kr, nbr);
  for (int j = 0; j < order; j++)
    for (int i = 0; i < order - 1; i++) *N++ = nar[i] * nb[j];
  for (int j = 0; j < order - 1; j++)
    for (int i = 0; i < order; i++) *N++ = na[i] * nbr[j];
  for (int j = 0; j < order - 1; j++)
    for (int i = 0; i < order - 1; i++) *N++ = nar[i] * nbr[j];
  for (int j = 0; j < order - 1; j++)
    for (int i = 0; i < order; i++) *N++ = na[i] * nbr[j];
  for (int j = 0; j < order; j++)
    for (int i = 0; i < order - 1; i++) *N++ = nar[i] * nb[j];
}
static const int TY_INDEX[5] = {0, 3, 1, 4, 2};

/* interpTyingStrain (:651-669) */
static void interp_tying(int order, const double pt[], const double *ety, double gty[6]) {
  double N[MAXTY];
  tying_interp(order, pt, N);
  const double *N0 = N;
  for (int f = 0; f < 5; f++) {
    int np = ntying_field(order, f);
    gty[TY_INDEX[f]] = 0.0;
    for (int k = 0; k < np; k++, N0++, ety++) gty[TY_INDEX[f]] += N0[0] * ety[0];
  }
  gty[5] = 0.0;
}
/* addInterpTyingStrainTranspose (:678-693) */
static void interp_tying_t(int order, const double pt[], const double dgty[6], double *dety) {
  double N[MAXTY];
  tying_interp(order, pt, N);
  const double *N0 = N;
  for (int f = 0; f < 5; f++) {
    int np = ntying_field(order, f);
    for (int k = 0; k < np; k++, N0++, dety++) dety[0] += dgty[TY_INDEX[f]] * N0[0];
  }
}
/* addInterpTyingStrainHessian (:707-733) */
static void interp_tying_h(int order, const double pt[], const double d2gty[36],
                           double *d2ety) {
  double N[MAXTY];
  tying_interp(order, pt, N);
  const double *N1 = N;
  for (int f1 = 0; f1 < 5; f1++) {
    int np1 = ntying_field(order, f1);
    for (int k1 = 0; k1 < np1; k1++, N1++) {
      const double *N2 = N;
      for (int f2 = 0; f2 < 5; f2++) {
        int np2 = ntying_field(order, f2);
        double value = d2gty[6 * TY_INDEX[f1] + TY_INDEX[f2]];
        for (int k2 = 0; k2 < np2; k2++, N2++, d2ety++) d2ety[0] += N1[0] * N2[0] * value;
      }
    }
  }
}

/* ----------------------------------------------------------------- algebra
   TACSElementAlgebra.h (row-major 3x3) */
static void mm(const double A[], const double B[], double C[]) { /* C = A B */
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++)
      C[3 * i + j] = A[3 * i] * B[j] + A[3 * i + 1] * B[3 + j] + A[3 * i + 2] * B[6 + j];
}
static void mm_add(const double A[], const double B[], double C[]) { /* C += A B */
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++)
      C[3 * i + j] += A[3 * i] * B[j] + A[3 * i + 1] * B[3 + j] + A[3 * i + 2] * B[6 + j];
}
static void mmT(const double A[], const double B[], double C[]) { /* C = A B^T */
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++)
      C[3 * i + j] = A[3 * i] * B[3 * j] + A[3 * i + 1] * B[3 * j + 1] + A[3 * i + 2] * B[3 * j + 2];
}
static void mmT_add(const double A[], const double B[], double C[]) { /* C += A B^T */
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++)
      C[3 * i + j] += A[3 * i] * B[3 * j] + A[3 * i + 1] * B[3 * j + 1] + A[3 * i + 2] * B[3 * j + 2];
}
static void mTm(const double A[], const double B[], double C[]) { /* C = A^T B */
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++)
      C[3 * i + j] = A[i] * B[j] + A[3 + i] * B[3 + j] + A[6 + i] * B[6 + j];
}
static double dot3(const double a[], const double b[]) {
  return a[0] * b[0] + a[1] * b[1] + a[2] * b[2];
}
static void cross3(const double x[], const double y[], double o[]) {
  o[0] = (x[1] * y[2] - x[2] * y[1]);
  o[1] = (x[2] * y[0] - x[0] * y[2]);
  o[2] = (x[0] * y[1] - x[1] * y[0]);
}
static void cross3_add(double a, const double x[], const double y[], double o[]) {
  o[0] += a * (x[1] * y[2] - x[2] * y[1]);
  o[1] += a * (x[2] * y[0] - x[0] * y[2]);
  o[2] += a * (x[0] * y[1] - x[1] * y[0]);
}
/* inv3x3 (TACSElementAlgebra.h:1980-2000) */
static double inv3(const double A[], double Ai[]) {
  double det = (A[8] * (A[0] * A[4] - A[3] * A[1]) - A[7] * (A[0] * A[5] - A[3] * A[2]) +
                A[6] * (A[1] * A[5] - A[2] * A[4]));
  double di = 1.0 / det;
  Ai[0] = (A[4] * A[8] - A[5] * A[7]) * di;
  Ai[1] = -(A[1] * A[8] - A[2] * A[7]) * di;
  Ai[2] = (A[1] * A[5] - A[2] * A[4]) * di;
  Ai[3] = -(A[3] * A[8] - A[5] * A[6]) * di;
  Ai[4] = (A[0] * A[8] - A[2] * A[6]) * di;
  Ai[5] = -(A[0] * A[5] - A[2] * A[3]) * di;
  Ai[6] = (A[3] * A[7] - A[4] * A[6]) * di;
  Ai[7] = -(A[0] * A[7] - A[1] * A[6]) * di;
  Ai[8] = (A[0] * A[4] - A[1] * A[3]) * di;
  return det;
}
/* mat3x3SymmTransformTranspose: A = T^T S T (TACSElementAlgebra.h:1094-1125) */
static void symm_tt(const double T[], const double S[], double A[]) {
  double W[9];
  W[0] = S[0] * T[0] + S[1] * T[3] + S[2] * T[6];
  W[1] = S[0] * T[1] + S[1] * T[4] + S[2] * T[7];
  W[2] = S[0] * T[2] + S[1] * T[5] + S[2] * T[8];
  W[3] = S[1] * T[0] + S[3] * T[3] + S[4] * T[6];
  W[4] = S[1] * T[1] + S[3] * T[4] + S[4] * T[7];
  W[5] = S[1] * T[2] + S[3] * T[5] + S[4] * T[8];
  W[6] = S[2] * T[0] + S[4] * T[3] + S[5] * T[6];
  W[7] = S[2] * T[1] + S[4] * T[4] + S[5] * T[7];
  W[8] = S[2] * T[2] + S[4] * T[5] + S[5] * T[8];
  A[0] = T[0] * W[0] + T[3] * W[3] + T[6] * W[6];
  A[1] = T[0] * W[1] + T[3] * W[4] + T[6] * W[7];
  A[2] = T[0] * W[2] + T[3] * W[5] + T[6] * W[8];
  A[3] = T[1] * W[1] + T[4] * W[4] + T[7] * W[7];
  A[4] = T[1] * W[2] + T[4] * W[5] + T[7] * W[8];
  A[5] = T[2] * W[2] + T[5] * W[5] + T[8] * W[8];
}
/* mat3x3SymmTransformTransSens (:1179-1201): adjoint of symm_tt */
static void symm_tt_sens(const double T[], const double dA[], double dS[]) {
  double dW[9];
  dW[0] = T[0] * dA[0];
  dW[1] = T[0] * dA[1] + T[1] * dA[3];
  dW[2] = T[0] * dA[2] + T[1] * dA[4] + T[2] * dA[5];
  dW[3] = T[3] * dA[0];
  dW[4] = T[3] * dA[1] + T[4] * dA[3];
  dW[5] = T[3] * dA[2] + T[4] * dA[4] + T[5] * dA[5];
  dW[6] = T[6] * dA[0];
  dW[7] = T[6] * dA[1] + T[7] * dA[3];
  dW[8] = T[6] * dA[2] + T[7] * dA[4] + T[8] * dA[5];
  dS[0] = (T[0] * dW[0] + T[1] * dW[1] + T[2] * dW[2]);
  dS[1] = (T[3] * dW[0] + T[4] * dW[1] + T[5] * dW[2] + T[0] * dW[3] + T[1] * dW[4] +
           T[2] * dW[5]);
  dS[2] = (T[6] * dW[0] + T[7] * dW[1] + T[8] * dW[2] + T[0] * dW[6] + T[1] * dW[7] +
           T[2] * dW[8]);
  dS[3] = (T[3] * dW[3] + T[4] * dW[4] + T[5] * dW[5]);
  dS[4] = (T[6] * dW[3] + T[7] * dW[4] + T[8] * dW[5] + T[3] * dW[6] + T[4] * dW[7] +
           T[5] * dW[8]);
  dS[5] = (T[6] * dW[6] + T[7] * dW[7] + T[8] * dW[8]);
}
/* mat3x3SymmTransformTransHessian (:1220-1300): applies symm_tt_sens to the
   rows and then to the columns of a 6x6 second derivative. */
static void symm_tt_hess(const double T[], const double d2A[36], double d2S[36]) {
  double tmp[36], col[6], out[6];
  for (int i = 0; i < 6; i++) symm_tt_sens(T, &d2A[6 * i], &tmp[6 * i]);
  for (int i = 0; i < 6; i++) {
    for (int k = 0; k < 6; k++) col[k] = tmp[6 * k + i];
    symm_tt_sens(T, col, out);
    for (int k = 0; k < 6; k++) d2S[6 * k + i] = out[k];
  }
}
/* mat3x3TransMatMatHessian(T1, T2, B1, B2, d2C, d2A) and the Add / AddSymm
   variants (TACSShellUtilities.h:162-260): second derivative through
   C = T^T A B applied to the rows (T1, B1) and columns (T2, B2). */
static void tmm_hess(const double T1[], const double T2[], const double B1[], const double B2[],
                     const double d2C[81], double d2A[81], int mode /*0 set,1 add,2 addsymm*/) {
  double tmp2[81], t1[9], t2[9];
  for (int i = 0; i < 9; i++) {
    mmT(&d2C[9 * i], B1, t1);
    mm(T1, t1, &tmp2[9 * i]);
  }
  for (int i = 0; i < 9; i++) {
    for (int j = 0; j < 9; j++) t1[j] = tmp2[i + 9 * j];
    mmT(t1, B2, t2);
    mm(T2, t2, t1);
    for (int j = 0; j < 9; j++) {
      if (mode == 0) {
        d2A[i + 9 * j] = t1[j];
      } else if (mode == 1) {
        d2A[i + 9 * j] += t1[j];
      } else {
        d2A[i + 9 * j] += t1[j];
        d2A[j + 9 * i] += t1[j];
      }
    }
  }
}

/* --------------------------------------------------------------- transform
   TACSShellNaturalTransform::computeTransform (TACSShellElementTransform.h:
   25-88), including the in-plane projection that updates t1[0] three times
   and leaves t1[1], t1[2] unprojected. */
static void natural_transform(const double Xxi[6], const double n0[3], double T[9]) {
  double n[3] = {n0[0], n0[1], n0[2]};
  double inv = 1.0 / sqrt(dot3(n, n));
  n[0] *= inv;
  n[1] *= inv;
  n[2] *= inv;
  double t1[3] = {Xxi[0], Xxi[2], Xxi[4]};
  double d = dot3(n, t1);
  t1[0] = t1[0] - d * n[0];
  t1[0] = t1[0] - d * n[0];
  t1[0] = t1[0] - d * n[0];
  inv = 1.0 / sqrt(dot3(t1, t1));
  t1[0] *= inv;
  t1[1] *= inv;
  t1[2] *= inv;
  double t2[3];
  cross3(n, t1, t2);
  T[0] = t1[0];
  T[3] = t1[1];
  T[6] = t1[2];
  T[1] = t2[0];
  T[4] = t2[1];
  T[7] = t2[2];
  T[2] = n[0];
  T[5] = n[1];
  T[8] = n[2];
}

/* TacsShellAssembleFrame overloads (TACSShellUtilities.h:8-36) */
static void frame_xn(const double Xxi[6], const double n[3], double Xd[9]) {
  Xd[0] = Xxi[0]; Xd[1] = Xxi[1]; Xd[2] = n[0];
  Xd[3] = Xxi[2]; Xd[4] = Xxi[3]; Xd[5] = n[1];
  Xd[6] = Xxi[4]; Xd[7] = Xxi[5]; Xd[8] = n[2];
}
static void frame_x(const double nxi[6], double Xdz[9]) {
  Xdz[0] = nxi[0]; Xdz[1] = nxi[1]; Xdz[2] = 0.0;
  Xdz[3] = nxi[2]; Xdz[4] = nxi[3]; Xdz[5] = 0.0;
  Xdz[6] = nxi[4]; Xdz[7] = nxi[5]; Xdz[8] = 0.0;
}
/* TacsShellExtractFrame overloads (:68-92) */
static void extract_xn(const double Xd[9], double Xxi[6], double n[3]) {
  Xxi[0] = Xd[0]; Xxi[1] = Xd[1]; n[0] = Xd[2];
  Xxi[2] = Xd[3]; Xxi[3] = Xd[4]; n[1] = Xd[5];
  Xxi[4] = Xd[6]; Xxi[5] = Xd[7]; n[2] = Xd[8];
}
static void extract_x(const double Xd[9], double Xxi[6]) {
  Xxi[0] = Xd[0]; Xxi[1] = Xd[1];
  Xxi[2] = Xd[3]; Xxi[3] = Xd[4];
  Xxi[4] = Xd[6]; Xxi[5] = Xd[7];
}
/* TacsShellExtractFrameSens (:94-139) */
static void extract_sens(const double d2u0d[81], double d2u0xi[36], double *d2d0,
                         double *d2d0u0xi) {
  for (int j = 0; j < 6; j++) {
    int jj = 3 * (j / 2) + (j % 2);
    for (int i = 0; i < 6; i++) {
      int ii = 3 * (i / 2) + (i % 2);
      d2u0xi[6 * j + i] = d2u0d[9 * jj + ii];
    }
  }
  if (d2d0) {
    for (int j = 0; j < 3; j++)
      for (int i = 0; i < 3; i++) d2d0[3 * j + i] = d2u0d[9 * (3 * j + 2) + 3 * i + 2];
    for (int j = 0; j < 3; j++)
      for (int i = 0; i < 6; i++)
        d2d0u0xi[6 * j + i] = d2u0d[9 * (3 * j + 2) + 3 * (i / 2) + (i % 2)];
  }
}
/* TacsShellExtractFrameMixedSens (:141-160) */
static void extract_mixed_sens(const double d2u0du1d[81], double d2d0xiu0xi[36],
                               double d2d0d0xi[18]) {
  for (int j = 0; j < 6; j++) {
    int jj = 3 * (j / 2) + (j % 2);
    for (int i = 0; i < 6; i++) {
      int ii = 3 * (i / 2) + (i % 2);
      d2d0xiu0xi[6 * i + j] = d2u0du1d[9 * jj + ii];
    }
  }
  for (int j = 0; j < 3; j++)
    for (int i = 0; i < 6; i++)
      d2d0d0xi[6 * j + i] = d2u0du1d[9 * (3 * j + 2) + 3 * (i / 2) + (i % 2)];
}

/* ----------------------------------------------------------- constitutive
   TACSIsoShellConstitutive::evalTangentStiffness (TACSIsoShellConstitutive.cpp:
   192-226) with TACSMaterialProperties::evalTangentStiffness2D (:295-313) */
static void tangent_stiffness(const orc_material *m, double C[22]) {
  double G = 0.5 * m->E / (1.0 + m->nu);
  double D = m->E / (1.0 - m->nu * m->nu);
  double *A = &C[0], *B = &C[6], *Dm = &C[12], *As = &C[18];
  A[0] = D; A[1] = m->nu * D; A[2] = 0.0; A[3] = D; A[4] = 0.0; A[5] = G;
  for (int i = 0; i < 6; i++) B[i] = 0.0;
  double t = m->t, I = t * t * t / 12.0;
  for (int i = 0; i < 6; i++) {
    Dm[i] = I * A[i];
    A[i] *= t;
    B[i] += -m->t_offset * t * A[i];
    Dm[i] += m->t_offset * m->t_offset * t * t * A[i];
  }
  As[0] = As[2] = m->kcorr * A[5];
  As[1] = 0.0;
  C[21] = 0.5 * m->drill_reg * (As[0] + As[2]);
}
/* TACSShellConstitutive::computeStress (TACSShellConstitutive.h:125-150) */
static void compute_stress(const double C[22], const double e[9], double s[9]) {
  const double *A = &C[0], *B = &C[6], *D = &C[12], *As = &C[18];
  s[0] = A[0] * e[0] + A[1] * e[1] + A[2] * e[2] + B[0] * e[3] + B[1] * e[4] + B[2] * e[5];
  s[1] = A[1] * e[0] + A[3] * e[1] + A[4] * e[2] + B[1] * e[3] + B[3] * e[4] + B[4] * e[5];
  s[2] = A[2] * e[0] + A[4] * e[1] + A[5] * e[2] + B[2] * e[3] + B[4] * e[4] + B[5] * e[5];
  s[3] = B[0] * e[0] + B[1] * e[1] + B[2] * e[2] + D[0] * e[3] + D[1] * e[4] + D[2] * e[5];
  s[4] = B[1] * e[0] + B[3] * e[1] + B[4] * e[2] + D[1] * e[3] + D[3] * e[4] + D[4] * e[5];
  s[5] = B[2] * e[0] + B[4] * e[1] + B[5] * e[2] + D[2] * e[3] + D[4] * e[4] + D[5] * e[5];
  s[6] = As[0] * e[6] + As[1] * e[7];
  s[7] = As[1] * e[6] + As[2] * e[7];
  s[8] = C[21] * e[8];
}
/* TACSIsoShellConstitutive::evalThermalStrain (:438-456) */
static void thermal_strain(const orc_material *m, double theta, double e[9]) {
  for (int i = 0; i < 9; i++) e[i] = 0.0;
  e[0] = m->alpha * theta;
  e[1] = m->alpha * theta;
}

/* -------------------------------------------------------------- the model
   Strain e[0..7] as a function of z = (u0x[9], u1x[9], e0ty[6]):
   TACSShellLinearModel::evalStrain (TACSShellElementModel.h:440-458) and
   TACSShellNonlinearModel::evalStrain (:1115-1135). */
static void eval_strain(int nl, const double u0x[9], const double u1x[9], const double e0ty[6],
                        double e[9]) {
  e[0] = e0ty[0];
  e[1] = e0ty[3];
  e[2] = 2.0 * e0ty[1];
  if (nl) {
    e[3] = u1x[0] + (u0x[0] * u1x[0] + u0x[3] * u1x[3] + u0x[6] * u1x[6]);
    e[4] = u1x[4] + (u0x[1] * u1x[1] + u0x[4] * u1x[4] + u0x[7] * u1x[7]);
    e[5] = u1x[1] + u1x[3] +
           (u0x[0] * u1x[1] + u0x[3] * u1x[4] + u0x[6] * u1x[7] + u1x[0] * u0x[1] +
            u1x[3] * u0x[4] + u1x[6] * u0x[7]);
  } else {
    e[3] = u1x[0];
    e[4] = u1x[4];
    e[5] = u1x[1] + u1x[3];
  }
  e[6] = 2.0 * e0ty[4];
  e[7] = 2.0 * e0ty[2];
}

/* Jacobian de[i]/dz[j] for i < 8, z = (u0x, u1x, e0ty), 8 x 24 */
static void strain_jacobian(int nl, const double u0x[9], const double u1x[9], double De[8][24]) {
  memset(De, 0, sizeof(double) * 8 * 24);
  De[0][18 + 0] = 1.0;
  De[1][18 + 3] = 1.0;
  De[2][18 + 1] = 2.0;
  De[6][18 + 4] = 2.0;
  De[7][18 + 2] = 2.0;
  De[3][9 + 0] = 1.0;
  De[4][9 + 4] = 1.0;
  De[5][9 + 1] = 1.0;
  De[5][9 + 3] = 1.0;
  if (nl) {
    for (int r = 0; r < 3; r++) {
      int c0 = 3 * r, c1 = 3 * r + 1;
      /* e3 += u0x[c0] u1x[c0] */
      De[3][c0] += u1x[c0];
      De[3][9 + c0] += u0x[c0];
      /* e4 += u0x[c1] u1x[c1] */
      De[4][c1] += u1x[c1];
      De[4][9 + c1] += u0x[c1];
      /* e5 += u0x[c0] u1x[c1] + u1x[c0] u0x[c1] */
      De[5][c0] += u1x[c1];
      De[5][9 + c1] += u0x[c0];
      De[5][9 + c0] += u0x[c1];
      De[5][c1] += u1x[c0];
    }
  }
}

/* evalStrainSens (linear :463-497, nonlinear :1137-1170):
   du0x, du1x, de0ty = scale * (de/dz)^T dfde */
static void strain_sens(int nl, double scale, const double s[9], const double u0x[9],
                        const double u1x[9], double du0x[9], double du1x[9], double de0ty[6]) {
  double De[8][24];
  strain_jacobian(nl, u0x, u1x, De);
  double z[24];
  for (int j = 0; j < 24; j++) {
    double v = 0.0;
    for (int i = 0; i < 8; i++) v += De[i][j] * s[i];
    z[j] = scale * v;
  }
  memcpy(du0x, z, 9 * sizeof(double));
  memcpy(du1x, z + 9, 9 * sizeof(double));
  memcpy(de0ty, z + 18, 6 * sizeof(double));
}

/* evalStrainHessian (linear :528-620, nonlinear :1213-1720): the exact second
   derivative of scale * (1/2 e^T C e) w.r.t. z, i.e.
   scale * De^T C De + scale * sum_i s_i d2e_i/dz2; returned in the
   reference's blocks d2u0x, d2u1x, d2u0xu1x (9x9), d2e0ty (6x6),
   d2e0tyu0x, d2e0tyu1x (6x9). */
static void strain_hessian(int nl, double scale, const double s[9], const double C[22],
                           const double u0x[9], const double u1x[9], double d2u0x[81],
                           double d2u1x[81], double d2u0xu1x[81], double d2e0ty[36],
                           double d2e0tyu0x[54], double d2e0tyu1x[54]) {
  double De[8][24];
  strain_jacobian(nl, u0x, u1x, De);
  /* 8x8 stress-strain matrix */
  const double *A = &C[0], *B = &C[6], *D = &C[12], *As = &C[18];
  double M[8][8];
  memset(M, 0, sizeof(M));
  const int sym[3][3] = {{0, 1, 2}, {1, 3, 4}, {2, 4, 5}};
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) {
      M[i][j] = A[sym[i][j]];
      M[i][3 + j] = B[sym[i][j]];
      M[3 + i][j] = B[sym[i][j]];
      M[3 + i][3 + j] = D[sym[i][j]];
    }
  M[6][6] = As[0];
  M[6][7] = As[1];
  M[7][6] = As[1];
  M[7][7] = As[2];
  double MD[8][24];
  for (int i = 0; i < 8; i++)
    for (int j = 0; j < 24; j++) {
      double v = 0.0;
      for (int k = 0; k < 8; k++) v += M[i][k] * De[k][j];
      MD[i][j] = v;
    }
  double H[24][24];
  for (int a = 0; a < 24; a++)
    for (int b = 0; b < 24; b++) {
      double v = 0.0;
      for (int k = 0; k < 8; k++) v += De[k][a] * MD[k][b];
      H[a][b] = scale * v;
    }
  if (nl) {
    for (int r = 0; r < 3; r++) {
      int c0 = 3 * r, c1 = 3 * r + 1;
      H[c0][9 + c0] += scale * s[3];
      H[9 + c0][c0] += scale * s[3];
      H[c1][9 + c1] += scale * s[4];
      H[9 + c1][c1] += scale * s[4];
      H[c0][9 + c1] += scale * s[5];
      H[9 + c1][c0] += scale * s[5];
      H[c1][9 + c0] += scale * s[5];
      H[9 + c0][c1] += scale * s[5];
    }
  }
  for (int i = 0; i < 9; i++)
    for (int j = 0; j < 9; j++) {
      d2u0x[9 * i + j] = H[i][j];
      d2u1x[9 * i + j] = H[9 + i][9 + j];
      d2u0xu1x[9 * i + j] = H[i][9 + j];
    }
  for (int i = 0; i < 6; i++) {
    for (int j = 0; j < 6; j++) d2e0ty[6 * i + j] = H[18 + i][18 + j];
    for (int j = 0; j < 9; j++) {
      d2e0tyu0x[9 * i + j] = H[18 + i][j];
      d2e0tyu1x[9 * i + j] = H[18 + i][9 + j];
    }
  }
}

/* ---------------------------------------------------------- director (LR)
   TACSLinearizedRotation (TACSDirector.h:14-608) */
/* computeDirectorRates: d = q x t (:245-267) */
static void director_rates(int nn, const double *vars, const double *t, double *d) {
  for (int i = 0; i < nn; i++) cross3(&vars[6 * i + 3], &t[3 * i], &d[3 * i]);
}
/* computeRotationMat: C = I - q^x (:23-33) */
static void rotation_mat(const double q[3], double C[9]) {
  C[0] = 1.0; C[1] = q[2]; C[2] = -q[1];
  C[3] = -q[2]; C[4] = 1.0; C[5] = q[0];
  C[6] = q[1]; C[7] = -q[0]; C[8] = 1.0;
}
/* addRotationMatResidual (:72-86) */
static void rotation_mat_res(const double dC[9], double r[3]) {
  r[0] += -(dC[7] - dC[5]);
  r[1] += -(dC[2] - dC[6]);
  r[2] += -(dC[3] - dC[1]);
}
/* evalDrillStrain (:560-564) */
static double drill_strain(const double u0x[9], const double Ct[9]) {
  return 0.5 * (Ct[3] + u0x[3] - Ct[1] - u0x[1]);
}
/* evalDrillStrainSens (:566-589) */
static void drill_strain_sens(double scale, double du0x[9], double dCt[9]) {
  memset(du0x, 0, 9 * sizeof(double));
  memset(dCt, 0, 9 * sizeof(double));
  dCt[1] = -0.5 * scale;
  dCt[3] = 0.5 * scale;
  du0x[1] = -0.5 * scale;
  du0x[3] = 0.5 * scale;
}
/* addDirectorJacobian with beta = gamma = 0 (:369-478) */
static void director_jacobian(int nn, const double *t, const double *dd, const double *d2d,
                              const double *d2du, double *res, double *mat) {
  const int dsize = 3 * nn, nvars = 6 * nn;
  for (int i = 0; i < nn; i++) {
    const double *ti = &t[3 * i];
    for (int j = 0; j < nn; j++) {
      const double *tj = &t[3 * j];
      double B[9];
      for (int a = 0; a < 3; a++)
        for (int b = 0; b < 3; b++) B[3 * a + b] = d2d[(3 * i + a) * dsize + 3 * j + b];
      /* D = ti^x B tj^x (mat3x3SkewMatSkewTransform) */
      double tt[9], D[9];
      tt[0] = ti[1] * B[6] - ti[2] * B[3];
      tt[1] = ti[1] * B[7] - ti[2] * B[4];
      tt[2] = ti[1] * B[8] - ti[2] * B[5];
      tt[3] = ti[2] * B[0] - ti[0] * B[6];
      tt[4] = ti[2] * B[1] - ti[0] * B[7];
      tt[5] = ti[2] * B[2] - ti[0] * B[8];
      tt[6] = ti[0] * B[3] - ti[1] * B[0];
      tt[7] = ti[0] * B[4] - ti[1] * B[1];
      tt[8] = ti[0] * B[5] - ti[1] * B[2];
      D[0] = tj[2] * tt[1] - tj[1] * tt[2];
      D[3] = tj[2] * tt[4] - tj[1] * tt[5];
      D[6] = tj[2] * tt[7] - tj[1] * tt[8];
      D[1] = tj[0] * tt[2] - tj[2] * tt[0];
      D[4] = tj[0] * tt[5] - tj[2] * tt[3];
      D[7] = tj[0] * tt[8] - tj[2] * tt[6];
      D[2] = tj[1] * tt[0] - tj[0] * tt[1];
      D[5] = tj[1] * tt[3] - tj[0] * tt[4];
      D[8] = tj[1] * tt[6] - tj[0] * tt[7];
      for (int a = 0; a < 3; a++)
        for (int b = 0; b < 3; b++) mat[(6 * i + 3 + a) * nvars + 6 * j + 3 + b] -= D[3 * a + b];
    }
  }
  for (int i = 0; i < nn; i++) {
    const double *ti = &t[3 * i];
    for (int j = 0; j < nn; j++) {
      double B[9];
      for (int a = 0; a < 3; a++)
        for (int b = 0; b < 3; b++) B[3 * a + b] = d2du[(3 * i + a) * dsize + 3 * j + b];
      /* D = ti^x B (mat3x3SkewMatTransform) */
      double D[9];
      D[0] = ti[1] * B[6] - ti[2] * B[3];
      D[1] = ti[1] * B[7] - ti[2] * B[4];
      D[2] = ti[1] * B[8] - ti[2] * B[5];
      D[3] = ti[2] * B[0] - ti[0] * B[6];
      D[4] = ti[2] * B[1] - ti[0] * B[7];
      D[5] = ti[2] * B[2] - ti[0] * B[8];
      D[6] = ti[0] * B[3] - ti[1] * B[0];
      D[7] = ti[0] * B[4] - ti[1] * B[1];
      D[8] = ti[0] * B[5] - ti[1] * B[2];
      for (int a = 0; a < 3; a++)
        for (int b = 0; b < 3; b++) {
          mat[(6 * i + a + 3) * nvars + 6 * j + b] += D[3 * a + b];
          mat[(6 * j + b) * nvars + 6 * i + a + 3] += D[3 * a + b];
        }
    }
  }
  for (int i = 0; i < nn; i++) cross3_add(1.0, &t[3 * i], &dd[3 * i], &res[6 * i + 3]);
}

/* ------------------------------------------------------- shell utilities */
/* TacsShellComputeNodeNormals (TACSShellUtilities.h:302-344) */
static void node_normals(int order, const double *X, double *fn, double *Xdn) {
  const int nn = order * order;
  for (int i = 0; i < nn; i++) {
    double pt[2], Xxi[6];
    node_point(order, i, pt);
    interp_grad(order, 3, 3, pt, X, Xxi);
    double a[3] = {Xxi[0], Xxi[2], Xxi[4]}, b[3] = {Xxi[1], Xxi[3], Xxi[5]};
    cross3(a, b, &fn[3 * i]);
    double nrm = sqrt(dot3(&fn[3 * i], &fn[3 * i]));
    if (nrm != 0.0) {
      double s = 1.0 / nrm;
      fn[3 * i] *= s;
      fn[3 * i + 1] *= s;
      fn[3 * i + 2] *= s;
    }
    frame_xn(Xxi, &fn[3 * i], &Xdn[9 * i]);
  }
}

/* TacsShellComputeDispGrad (:362-418) */
static double disp_grad(int order, const double pt[], const double *fn, const double *vars,
                        const double *d, const double Xxi[6], const double n0[3],
                        const double T[9], double XdinvT[9], double XdinvzT[9], double u0x[9],
                        double u1x[9]) {
  double nxi[6], Xd[9], Xdz[9], Xdinv[9];
  interp_grad(order, 3, 3, pt, fn, nxi);
  frame_xn(Xxi, n0, Xd);
  frame_x(nxi, Xdz);
  double detXd = inv3(Xd, Xdinv);
  double neg[9];
  mm(Xdinv, Xdz, neg);
  for (int i = 0; i < 9; i++) neg[i] *= -1.0;
  mm(Xdinv, T, XdinvT);
  mm(neg, XdinvT, XdinvzT);
  double d0[3], d0xi[6], u0xi[6], tmp[9];
  interp(order, 3, 3, pt, d, d0);
  interp_grad(order, 3, 3, pt, d, d0xi);
  interp_grad(order, 6, 3, pt, vars, u0xi);
  frame_xn(u0xi, d0, u0x);
  frame_x(d0xi, u1x);
  mm(u1x, XdinvT, tmp);
  mm_add(u0x, XdinvzT, tmp);
  mTm(T, tmp, u1x);
  mm(u0x, XdinvT, tmp);
  mTm(T, tmp, u0x);
  return detXd;
}

/* TacsShellAddDispGradSens (:445-486) */
static void add_disp_grad_sens(int order, const double pt[], const double T[9],
                               const double XdinvT[9], const double XdinvzT[9],
                               const double du0x[9], const double du1x[9], double *res,
                               double *dd) {
  double du0d[9], tmp[9], du1d[9], du0xi[6], dd0[3], dd0xi[6];
  mmT(du1x, XdinvzT, tmp);
  mmT_add(du0x, XdinvT, tmp);
  mm(T, tmp, du0d);
  mmT(du1x, XdinvT, tmp);
  mm(T, tmp, du1d);
  extract_xn(du0d, du0xi, dd0);
  extract_x(du1d, dd0xi);
  interp_t(order, 3, 3, pt, dd0, dd);
  interp_grad_t(order, 3, 3, pt, dd0xi, dd);
  if (res) interp_grad_t(order, 6, 3, pt, du0xi, res);
}

/* TacsShellAddDispGradHessian (:583-646) */
static void add_disp_grad_hess(int order, const double pt[], const double T[9],
                               const double XdinvT[9], const double XdinvzT[9],
                               const double d2u0x[81], const double d2u1x[81],
                               const double d2u0xu1x[81], double *mat, double *d2d,
                               double *d2du) {
  double d2u0d[81], d2u1d[81], d2u0du1d[81];
  tmm_hess(T, T, XdinvT, XdinvT, d2u0x, d2u0d, 0);
  tmm_hess(T, T, XdinvzT, XdinvzT, d2u1x, d2u0d, 1);
  tmm_hess(T, T, XdinvzT, XdinvT, d2u0xu1x, d2u0d, 2);
  tmm_hess(T, T, XdinvT, XdinvT, d2u1x, d2u1d, 0);
  tmm_hess(T, T, XdinvT, XdinvT, d2u0xu1x, d2u0du1d, 0);
  tmm_hess(T, T, XdinvT, XdinvzT, d2u1x, d2u0du1d, 1);
  double d2u0xi[36], d2d0[9], d2d0u0xi[18], d2d0xi[36], d2d0xiu0xi[36], d2d0d0xi[18];
  extract_sens(d2u0d, d2u0xi, d2d0, d2d0u0xi);
  extract_sens(d2u1d, d2d0xi, NULL, NULL);
  extract_mixed_sens(d2u0du1d, d2d0xiu0xi, d2d0d0xi);
  outer(order, 3, 3, 3, 3, pt, d2d0, d2d);
  grad_outer(order, 3, 3, 3, 3, pt, d2d0xi, d2d);
  grad_mixed_outer(order, 3, 3, 3, 3, pt, d2d0d0xi, d2d0d0xi, d2d);
  grad_mixed_outer(order, 3, 3, 3, 3, pt, d2d0u0xi, NULL, d2du);
  grad_outer(order, 3, 3, 3, 3, pt, d2d0xiu0xi, d2du);
  if (mat) grad_outer(order, 6, 6, 3, 3, pt, d2u0xi, mat);
}

/* TacsShellComputeDrillStrain (:651-707) */
static void compute_drill(int order, const double *Xdn, const double *fn, const double *vars,
                          double *XdinvTn, double *Tn, double *u0xn, double *Ctn, double *etn) {
  const int nn = order * order;
  for (int i = 0; i < nn; i++) {
    double pt[2], Xxi[6], u0xi[6], Xdinv[9], C[9], tmp[9];
    node_point(order, i, pt);
    extract_x(&Xdn[9 * i], Xxi);
    natural_transform(Xxi, &fn[3 * i], &Tn[9 * i]);
    interp_grad(order, 6, 3, pt, vars, u0xi);
    inv3(&Xdn[9 * i], Xdinv);
    mm(Xdinv, &Tn[9 * i], &XdinvTn[9 * i]);
    frame_x(u0xi, &u0xn[9 * i]);
    rotation_mat(&vars[6 * i + 3], C);
    mTm(&Tn[9 * i], C, tmp);
    mm(tmp, &Tn[9 * i], &Ctn[9 * i]);
    mm(&u0xn[9 * i], &XdinvTn[9 * i], tmp);
    mTm(&Tn[9 * i], tmp, &u0xn[9 * i]);
    etn[i] = drill_strain(&u0xn[9 * i], &Ctn[9 * i]);
  }
}

/* d(et_i)/d(vars) row for node i, the drot rows of
   TacsShellAddDrillStrainHessian (:839-890) and the body of
   TacsShellAddDrillStrainSens (:782-821) with scale 1 */
static void drill_row(int order, int i, const double *XdinvTn, const double *Tn,
                      double *t /* len 6nn, accumulated */) {
  double pt[2], du0x[9], dCt[9], dCpt[9], tmp[9], du0d[9], du0xi[6];
  node_point(order, i, pt);
  drill_strain_sens(1.0, du0x, dCt);
  mm(&Tn[9 * i], dCt, tmp);
  mmT(tmp, &Tn[9 * i], dCpt);
  rotation_mat_res(dCpt, &t[6 * i + 3]);
  mmT(du0x, &XdinvTn[9 * i], tmp);
  mm(&Tn[9 * i], tmp, du0d);
  extract_x(du0d, du0xi);
  interp_grad_t(order, 6, 3, pt, du0xi, t);
}

/* TacsShellAddTyingDispCoupling (:962-1063) */
static void add_tying_disp_coupling(int order, const double pt[], const double T[9],
                                    const double XdinvT[9], const double XdinvzT[9],
                                    const double d2e0tyu0x[54], const double d2e0tyu1x[54],
                                    double *d2etyu, double *d2etyd) {
  const int nn = order * order, usize = 3 * nn, nty = ntying(order);
  double tmp0d[54], tmp1d[54], d2gtyu0d[54], d2gtyu1d[54];
  for (int k = 0; k < 6; k++) {
    double tmp[9];
    mmT(&d2e0tyu1x[9 * k], XdinvzT, tmp);
    mmT_add(&d2e0tyu0x[9 * k], XdinvT, tmp);
    mm(T, tmp, &tmp0d[9 * k]);
    mmT(&d2e0tyu1x[9 * k], XdinvT, tmp);
    mm(T, tmp, &tmp1d[9 * k]);
  }
  for (int k = 0; k < 9; k++) {
    double t0[6], out[6];
    for (int kk = 0; kk < 6; kk++) t0[kk] = tmp0d[9 * kk + k];
    symm_tt_sens(XdinvT, t0, out);
    for (int kk = 0; kk < 6; kk++) d2gtyu0d[9 * kk + k] = out[kk];
  }
  for (int k = 0; k < 9; k++) {
    double t0[6], out[6];
    for (int kk = 0; kk < 6; kk++) t0[kk] = tmp1d[9 * kk + k];
    symm_tt_sens(XdinvT, t0, out);
    for (int kk = 0; kk < 6; kk++) d2gtyu1d[9 * kk + k] = out[kk];
  }
  double d2gtyu[6 * MAXD], d2gtyd[6 * MAXD];
  memset(d2gtyu, 0, sizeof(double) * 6 * usize);
  memset(d2gtyd, 0, sizeof(double) * 6 * usize);
  for (int k = 0; k < 6; k++) {
    double du0xi[6], dd0[3], dd0xi[6];
    extract_xn(&d2gtyu0d[9 * k], du0xi, dd0);
    extract_x(&d2gtyu1d[9 * k], dd0xi);
    interp_t(order, 3, 3, pt, dd0, &d2gtyd[usize * k]);
    interp_grad_t(order, 3, 3, pt, dd0xi, &d2gtyd[usize * k]);
    interp_grad_t(order, 3, 3, pt, du0xi, &d2gtyu[usize * k]);
  }
  for (int k = 0; k < usize; k++) {
    double t1[6], t2[MAXTY];
    memset(t2, 0, sizeof(double) * nty);
    for (int kk = 0; kk < 6; kk++) t1[kk] = d2gtyu[usize * kk + k];
    interp_tying_t(order, pt, t1, t2);
    for (int kk = 0; kk < nty; kk++) d2etyu[kk * usize + k] += t2[kk];
  }
  for (int k = 0; k < usize; k++) {
    double t1[6], t2[MAXTY];
    memset(t2, 0, sizeof(double) * nty);
    for (int kk = 0; kk < 6; kk++) t1[kk] = d2gtyd[usize * kk + k];
    interp_tying_t(order, pt, t1, t2);
    for (int kk = 0; kk < nty; kk++) d2etyd[kk * usize + k] += t2[kk];
  }
}

/* ------------------------------------------------------ tying strains
   computeTyingStrain: linear (TACSShellElementModel.h:33-78),
   nonlinear (:644-698) */
static void compute_tying(int order, int nl, const double *X, const double *fn,
                          const double *vars, const double *d, double *ety) {
  const int nty = ntying(order);
  for (int index = 0; index < nty; index++) {
    int f = tying_field(order, index);
    double pt[2], Uxi[6], Xxi[6];
    tying_point(order, index, pt);
    interp_grad(order, 3, 3, pt, X, Xxi);
    interp_grad(order, 6, 3, pt, vars, Uxi);
    ety[index] = 0.0;
    if (f == F11) {
      ety[index] = (Uxi[0] * Xxi[0] + Uxi[2] * Xxi[2] + Uxi[4] * Xxi[4]);
      if (nl) ety[index] += 0.5 * (Uxi[0] * Uxi[0] + Uxi[2] * Uxi[2] + Uxi[4] * Uxi[4]);
    } else if (f == F22) {
      ety[index] = (Uxi[1] * Xxi[1] + Uxi[3] * Xxi[3] + Uxi[5] * Xxi[5]);
      if (nl) ety[index] += 0.5 * (Uxi[1] * Uxi[1] + Uxi[3] * Uxi[3] + Uxi[5] * Uxi[5]);
    } else if (f == F12) {
      double v = Uxi[0] * Xxi[1] + Uxi[2] * Xxi[3] + Uxi[4] * Xxi[5] + Uxi[1] * Xxi[0] +
                 Uxi[3] * Xxi[2] + Uxi[5] * Xxi[4];
      if (nl) v += Uxi[0] * Uxi[1] + Uxi[2] * Uxi[3] + Uxi[4] * Uxi[5];
      ety[index] = 0.5 * v;
    } else {
      double d0[3], n0[3], m[3];
      interp(order, 3, 3, pt, d, d0);
      interp(order, 3, 3, pt, fn, n0);
      for (int k = 0; k < 3; k++) m[k] = nl ? (n0[k] + d0[k]) : n0[k];
      if (f == F23) {
        ety[index] = 0.5 * (Xxi[1] * d0[0] + Xxi[3] * d0[1] + Xxi[5] * d0[2] + m[0] * Uxi[1] +
                            m[1] * Uxi[3] + m[2] * Uxi[5]);
      } else {
        ety[index] = 0.5 * (Xxi[0] * d0[0] + Xxi[2] * d0[1] + Xxi[4] * d0[2] + m[0] * Uxi[0] +
                            m[1] * Uxi[2] + m[2] * Uxi[4]);
      }
    }
  }
}

/* The first derivative of the tying strain at one point w.r.t. (Uxi, d0):
   the dUxi / dd0 vectors built in addComputeTyingStrainTranspose (:80-161,
   :700-780) with unit weight.  Uxi, d0 are the state at the tying point
   (zero / unused for the linear model). */
static void tying_deriv(int nl, int f, const double Xxi[6], const double n0[3],
                        const double Uxi[6], const double d0[3], double dUxi[6], double dd0[3]) {
  double a[6];
  for (int k = 0; k < 6; k++) a[k] = nl ? (Xxi[k] + Uxi[k]) : Xxi[k];
  double m[3];
  for (int k = 0; k < 3; k++) m[k] = nl ? (n0[k] + d0[k]) : n0[k];
  for (int k = 0; k < 6; k++) dUxi[k] = 0.0;
  dd0[0] = dd0[1] = dd0[2] = 0.0;
  if (f == F11) {
    dUxi[0] = a[0]; dUxi[2] = a[2]; dUxi[4] = a[4];
  } else if (f == F22) {
    dUxi[1] = a[1]; dUxi[3] = a[3]; dUxi[5] = a[5];
  } else if (f == F12) {
    dUxi[0] = 0.5 * a[1]; dUxi[1] = 0.5 * a[0]; dUxi[2] = 0.5 * a[3];
    dUxi[3] = 0.5 * a[2]; dUxi[4] = 0.5 * a[5]; dUxi[5] = 0.5 * a[4];
  } else if (f == F23) {
    dUxi[1] = 0.5 * m[0]; dUxi[3] = 0.5 * m[1]; dUxi[5] = 0.5 * m[2];
    dd0[0] = 0.5 * a[1]; dd0[1] = 0.5 * a[3]; dd0[2] = 0.5 * a[5];
  } else {
    dUxi[0] = 0.5 * m[0]; dUxi[2] = 0.5 * m[1]; dUxi[4] = 0.5 * m[2];
    dd0[0] = 0.5 * a[0]; dd0[1] = 0.5 * a[2]; dd0[2] = 0.5 * a[4];
  }
}

typedef struct {
  double Xxi[6], n0[3], Uxi[6], d0[3], pt[2];
  int f;
} tying_state;

static void tying_states(int order, const double *X, const double *fn, const double *vars,
                         const double *d, tying_state *ts) {
  const int nty = ntying(order);
  for (int i = 0; i < nty; i++) {
    tying_point(order, i, ts[i].pt);
    ts[i].f = tying_field(order, i);
    interp_grad(order, 3, 3, ts[i].pt, X, ts[i].Xxi);
    interp(order, 3, 3, ts[i].pt, fn, ts[i].n0);
    interp_grad(order, 6, 3, ts[i].pt, vars, ts[i].Uxi);
    interp(order, 3, 3, ts[i].pt, d, ts[i].d0);
  }
}

/* addComputeTyingStrainTranspose (:80-161 linear, :700-780 nonlinear) */
static void add_tying_transpose(int order, int nl, const tying_state *ts, const double *dety,
                                double *res, double *dd) {
  const int nty = ntying(order);
  for (int i = 0; i < nty; i++) {
    double dUxi[6], dd0[3];
    tying_deriv(nl, ts[i].f, ts[i].Xxi, ts[i].n0, ts[i].Uxi, ts[i].d0, dUxi, dd0);
    for (int k = 0; k < 6; k++) dUxi[k] *= dety[i];
    for (int k = 0; k < 3; k++) dd0[k] *= dety[i];
    if (ts[i].f == F23 || ts[i].f == F13) interp_t(order, 3, 3, ts[i].pt, dd0, dd);
    if (res) interp_grad_t(order, 6, 3, ts[i].pt, dUxi, res);
  }
}

/* addComputeTyingStrainHessian (:163-366 linear, :782-1032 nonlinear) */
static void add_tying_hessian(int order, int nl, double alpha, const tying_state *ts,
                              const double *dety, const double *d2ety, const double *d2etyu,
                              const double *d2etyd, double *mat, double *d2d, double *d2du) {
  const int nn = order * order, nty = ntying(order), usize = 3 * nn, nvars = 6 * nn;
  for (int i1 = 0; i1 < nty; i1++) {
    double du2[MAXD], dd2[MAXD];
    memset(du2, 0, sizeof(double) * usize);
    memset(dd2, 0, sizeof(double) * usize);
    for (int i2 = 0; i2 < nty; i2++) {
      double value = d2ety[nty * i1 + i2];
      double dUxi2[6], dd02[3];
      tying_deriv(nl, ts[i2].f, ts[i2].Xxi, ts[i2].n0, ts[i2].Uxi, ts[i2].d0, dUxi2, dd02);
      for (int k = 0; k < 6; k++) dUxi2[k] *= value;
      for (int k = 0; k < 3; k++) dd02[k] *= value;
      if (ts[i2].f == F23 || ts[i2].f == F13) interp_t(order, 3, 3, ts[i2].pt, dd02, dd2);
      interp_grad_t(order, 3, 3, ts[i2].pt, dUxi2, du2);
    }
    double du1[MAXD], dUxi1[6], dd01[3];
    memset(du1, 0, sizeof(double) * usize);
    const int f1 = ts[i1].f;
    tying_deriv(nl, f1, ts[i1].Xxi, ts[i1].n0, ts[i1].Uxi, ts[i1].d0, dUxi1, dd01);
    double d2Uxi[36];
    memset(d2Uxi, 0, sizeof(d2Uxi));
    if (nl) {
      double a = alpha * dety[i1];
      if (f1 == F11) {
        d2Uxi[0] = a; d2Uxi[14] = a; d2Uxi[28] = a;
      } else if (f1 == F22) {
        d2Uxi[7] = a; d2Uxi[21] = a; d2Uxi[35] = a;
      } else if (f1 == F12) {
        d2Uxi[1] = 0.5 * a; d2Uxi[6] = 0.5 * a; d2Uxi[15] = 0.5 * a;
        d2Uxi[20] = 0.5 * a; d2Uxi[29] = 0.5 * a; d2Uxi[34] = 0.5 * a;
      }
    }
    if (f1 == F23 || f1 == F13) {
      double dd1[MAXD];
      memset(dd1, 0, sizeof(double) * usize);
      interp_t(order, 3, 3, ts[i1].pt, dd01, dd1);
      const double *etd = &d2etyd[usize * i1];
      const double *etu = &d2etyu[usize * i1];
      for (int i = 0; i < usize; i++)
        for (int j = 0; j < usize; j++)
          d2d[usize * i + j] += dd1[i] * dd2[j] + dd1[i] * etd[j] + etd[i] * dd1[j];
      for (int i = 0; i < usize; i++)
        for (int j = 0; j < usize; j++) d2du[usize * i + j] += dd1[i] * du2[j] + dd1[i] * etu[j];
      if (nl) {
        double d2dUxi[18];
        memset(d2dUxi, 0, sizeof(d2dUxi));
        double a = 0.5 * alpha * dety[i1];
        if (f1 == F23) {
          d2dUxi[1] = a; d2dUxi[9] = a; d2dUxi[17] = a;
        } else {
          d2dUxi[0] = a; d2dUxi[8] = a; d2dUxi[16] = a;
        }
        grad_mixed_outer(order, 3, 3, 3, 3, ts[i1].pt, d2dUxi, NULL, d2du);
      }
    }
    interp_grad_t(order, 3, 3, ts[i1].pt, dUxi1, du1);
    const double *etd = &d2etyd[usize * i1];
    for (int i = 0; i < usize; i++)
      for (int j = 0; j < usize; j++) d2du[usize * i + j] += etd[i] * du1[j];
    const double *etu = &d2etyu[usize * i1];
    for (int i = 0; i < usize; i++) {
      int ii = 6 * (i / 3) + (i % 3);
      for (int j = 0; j < usize; j++) {
        int jj = 6 * (j / 3) + (j % 3);
        mat[nvars * ii + jj] += du1[i] * du2[j] + du1[i] * etu[j] + etu[i] * du1[j];
      }
    }
    if (nl) grad_outer(order, 6, 6, 3, 3, ts[i1].pt, d2Uxi, mat);
  }
}

/* ------------------------------------------------------- element routines */
void orc_add_residual(int order, int nl, const orc_material *m, const double *X,
                      const double *vars, double *res) {
  const int nn = order * order, nquad = nn, nty = ntying(order);
  double dd[MAXD], fn[MAXD], Xdn[9 * MAXN], etn[MAXN], detn[MAXN];
  double XdinvTn[9 * MAXN], Tn[9 * MAXN], u0xn[9 * MAXN], Ctn[9 * MAXN], d[MAXD];
  double ety[MAXTY], dety[MAXTY], C[22];
  memset(dd, 0, sizeof(dd));
  memset(detn, 0, sizeof(detn));
  memset(dety, 0, sizeof(dety));
  node_normals(order, X, fn, Xdn);
  compute_drill(order, Xdn, fn, vars, XdinvTn, Tn, u0xn, Ctn, etn);
  director_rates(nn, vars, fn, d);
  compute_tying(order, nl, X, fn, vars, d, ety);
  tangent_stiffness(m, C);
  for (int q = 0; q < nquad; q++) {
    double pt[2];
    double w = quad_point(order, q, pt);
    double Xq[3], Xxi[6], n0[3], T[9], et;
    interp(order, 3, 3, pt, X, Xq);
    interp_grad(order, 3, 3, pt, X, Xxi);
    interp(order, 3, 3, pt, fn, n0);
    interp(order, 1, 1, pt, etn, &et);
    natural_transform(Xxi, n0, T);
    double XdinvT[9], XdinvzT[9], u0x[9], u1x[9];
    double detXd = disp_grad(order, pt, fn, vars, d, Xxi, n0, T, XdinvT, XdinvzT, u0x, u1x);
    detXd *= w;
    double gty[6], e0ty[6], e[9], eth[9], em[9], s[9];
    interp_tying(order, pt, ety, gty);
    symm_tt(XdinvT, gty, e0ty);
    eval_strain(nl, u0x, u1x, e0ty, e);
    e[8] = et;
    thermal_strain(m, m->temperature, eth);
    for (int i = 0; i < 9; i++) em[i] = e[i] - eth[i];
    compute_stress(C, em, s);
    double du0x[9], du1x[9], de0ty[6];
    strain_sens(nl, detXd, s, u0x, u1x, du0x, du1x, de0ty);
    double det = detXd * s[8];
    interp_t(order, 1, 1, pt, &det, detn);
    add_disp_grad_sens(order, pt, T, XdinvT, XdinvzT, du0x, du1x, res, dd);
    double dgty[6];
    symm_tt_sens(XdinvT, de0ty, dgty);
    interp_tying_t(order, pt, dgty, dety);
  }
  /* TacsShellAddDrillStrainSens */
  for (int i = 0; i < nn; i++) {
    double t[MAXV];
    memset(t, 0, sizeof(double) * 6 * nn);
    drill_row(order, i, XdinvTn, Tn, t);
    for (int j = 0; j < 6 * nn; j++) res[j] += detn[i] * t[j];
  }
  tying_state ts[MAXTY];
  tying_states(order, X, fn, vars, d, ts);
  add_tying_transpose(order, nl, ts, dety, res, dd);
  /* addDirectorResidual: res_q += t x dd */
  for (int i = 0; i < nn; i++) cross3_add(1.0, &fn[3 * i], &dd[3 * i], &res[6 * i + 3]);
  (void)nty;
}

void orc_add_jacobian(int order, int nl, const orc_material *m, double alpha,
                      const double *X, const double *vars, double *res, double *mat) {
  const int nn = order * order, nquad = nn, nty = ntying(order), usize = 3 * nn,
            size = 6 * nn;
  double dd[MAXD], d2d[MAXD * MAXD], d2du[MAXD * MAXD];
  double dety[MAXTY], d2ety[MAXTY * MAXTY], d2etyu[MAXTY * MAXD], d2etyd[MAXTY * MAXD];
  double fn[MAXD], Xdn[9 * MAXN], etn[MAXN], detn[MAXN], d2etn[MAXN * MAXN];
  double XdinvTn[9 * MAXN], Tn[9 * MAXN], u0xn[9 * MAXN], Ctn[9 * MAXN], d[MAXD];
  double ety[MAXTY], C[22];
  memset(dd, 0, sizeof(dd));
  memset(d2d, 0, sizeof(d2d));
  memset(d2du, 0, sizeof(d2du));
  memset(dety, 0, sizeof(dety));
  memset(d2ety, 0, sizeof(d2ety));
  memset(d2etyu, 0, sizeof(d2etyu));
  memset(d2etyd, 0, sizeof(d2etyd));
  memset(detn, 0, sizeof(detn));
  memset(d2etn, 0, sizeof(d2etn));
  node_normals(order, X, fn, Xdn);
  compute_drill(order, Xdn, fn, vars, XdinvTn, Tn, u0xn, Ctn, etn);
  director_rates(nn, vars, fn, d);
  compute_tying(order, nl, X, fn, vars, d, ety);
  tangent_stiffness(m, C);
  for (int q = 0; q < nquad; q++) {
    double pt[2];
    double w = quad_point(order, q, pt);
    double Xq[3], Xxi[6], n0[3], T[9], et;
    interp(order, 3, 3, pt, X, Xq);
    interp_grad(order, 3, 3, pt, X, Xxi);
    interp(order, 3, 3, pt, fn, n0);
    interp(order, 1, 1, pt, etn, &et);
    natural_transform(Xxi, n0, T);
    double XdinvT[9], XdinvzT[9], u0x[9], u1x[9];
    double detXd = disp_grad(order, pt, fn, vars, d, Xxi, n0, T, XdinvT, XdinvzT, u0x, u1x);
    detXd *= w;
    double gty[6], e0ty[6], e[9], eth[9], em[9], s[9];
    interp_tying(order, pt, ety, gty);
    symm_tt(XdinvT, gty, e0ty);
    eval_strain(nl, u0x, u1x, e0ty, e);
    e[8] = et;
    thermal_strain(m, m->temperature, eth);
    for (int i = 0; i < 9; i++) em[i] = e[i] - eth[i];
    compute_stress(C, em, s);
    double du0x[9], du1x[9], de0ty[6];
    strain_sens(nl, detXd, s, u0x, u1x, du0x, du1x, de0ty);
    double d2u0x[81], d2u1x[81], d2u0xu1x[81], d2e0ty[36], d2e0tyu0x[54], d2e0tyu1x[54];
    strain_hessian(nl, alpha * detXd, s, C, u0x, u1x, d2u0x, d2u1x, d2u0xu1x, d2e0ty,
                   d2e0tyu0x, d2e0tyu1x);
    double det = detXd * s[8];
    interp_t(order, 1, 1, pt, &det, detn);
    add_disp_grad_sens(order, pt, T, XdinvT, XdinvzT, du0x, du1x, res, dd);
    double d2et = detXd * alpha * C[21];
    outer(order, 1, 1, 1, 1, pt, &d2et, d2etn);
    add_disp_grad_hess(order, pt, T, XdinvT, XdinvzT, d2u0x, d2u1x, d2u0xu1x, mat, d2d, d2du);
    double dgty[6], d2gty[36];
    symm_tt_sens(XdinvT, de0ty, dgty);
    symm_tt_hess(XdinvT, d2e0ty, d2gty);
    interp_tying_t(order, pt, dgty, dety);
    interp_tying_h(order, pt, d2gty, d2ety);
    add_tying_disp_coupling(order, pt, T, XdinvT, XdinvzT, d2e0tyu0x, d2e0tyu1x, d2etyu,
                            d2etyd);
  }
  /* TacsShellAddDrillStrainHessian: the drill strain is linear in the
     variables for the linearized rotation, so only the outer products of
     its first derivatives (and the residual) contribute. */
  {
    double drot[MAXN * MAXV];
    memset(drot, 0, sizeof(double) * nn * size);
    for (int i = 0; i < nn; i++) drill_row(order, i, XdinvTn, Tn, &drot[i * size]);
    if (res)
      for (int i = 0; i < nn; i++)
        for (int j = 0; j < size; j++) res[j] += detn[i] * drot[i * size + j];
    for (int i = 0; i < nn; i++) {
      double t[MAXV];
      memset(t, 0, sizeof(double) * size);
      for (int j = 0; j < nn; j++)
        for (int ii = 0; ii < size; ii++) t[ii] += d2etn[i * nn + j] * drot[j * size + ii];
      for (int ii = 0; ii < size; ii++)
        for (int jj = 0; jj < size; jj++) mat[ii * size + jj] += t[ii] * drot[i * size + jj];
    }
  }
  tying_state ts[MAXTY];
  tying_states(order, X, fn, vars, d, ts);
  add_tying_transpose(order, nl, ts, dety, res, dd);
  add_tying_hessian(order, nl, alpha, ts, dety, d2ety, d2etyu, d2etyd, mat, d2d, d2du);
  director_jacobian(nn, fn, dd, d2d, d2du, res, mat);
  (void)nty;
  (void)usize;
}

void orc_get_mat_type(int order, int nl, int kind, const orc_material *m, const double *X,
                      const double *vars, double *mat) {
  const int nn = order * order, size = 6 * nn;
  double res[MAXV];
  memset(mat, 0, sizeof(double) * size * size);
  memset(res, 0, sizeof(res));
  if (kind == ORC_GEOMETRIC) {
    /* Central difference of the nonlinear tangent along the normalised
       state, including the temperature (TACSShellElement.h:700-767). */
    double dh = 1e-4, norm = 0.0;
    for (int i = 0; i < size; i++) norm += vars[i] * vars[i];
    norm += m->temperature * m->temperature;
    norm = (norm == 0.0) ? 1.0 : sqrt(norm);
    double alpha = 0.5 * norm / dh;
    double path[MAXV];
    orc_material mp = *m;
    for (int i = 0; i < size; i++) path[i] = dh * vars[i] / norm;
    mp.temperature = m->temperature + dh * m->temperature / norm;
    orc_add_jacobian(order, 1, &mp, alpha, X, path, res, mat);
    for (int i = 0; i < size; i++) path[i] = -dh * vars[i] / norm;
    mp.temperature = m->temperature - dh * m->temperature / norm;
    orc_add_jacobian(order, 1, &mp, -alpha, X, path, res, mat);
    return;
  }
  if (kind == ORC_STIFFNESS) orc_add_jacobian(order, nl, m, 1.0, X, vars, res, mat);
}
