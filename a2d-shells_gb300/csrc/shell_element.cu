// GB300 element kernel for the director-based MITC shell (linearized
// rotation director, linear or nonlinear strain model), Quad4 and Quad9.
//
// What it computes, per element, matches TACSShellElement (reference
// src/elements/shell/TACSShellElement.h): the tangent stiffness
// (addJacobian / getMatType(TACS_STIFFNESS_MATRIX), :455-672), the geometric
// stiffness (getMatType(TACS_GEOMETRIC_STIFFNESS_MATRIX), :675-771) and the
// residual (addResidual, :303-449).  How it computes them is its own:
//
// * Every element DOF column j produces displacement gradients of rank one,
//   u0x = a_j b_j^T and u1x = a_j c_j^T (a_j = T^T e_c for a displacement,
//   T^T (e_r x n) for a rotation), so the strain-displacement matrix B
//   (9 x nv per Gauss point) is built column-parallel, one thread per DOF.
// * The strain is e(q) = B0 q + 1/2 P(q, q) with P a symmetric bilinear form
//   (zero for the linear model).  The tangent is
//   K_T(u) = sum_g wdet (B(u)^T C B(u) + s(u) . P),  B(u) = B0 + P(., u),
//   and the geometric stiffness the reference forms by central differences
//   of the nonlinear tangent is its exact directional derivative at zero,
//   G(w) = sum_g wdet (P(., w)^T C B0 + B0^T C P(., w) + C(B0 w - eth) . P).
// * Only the upper triangle of the symmetric element matrix is accumulated
//   (FP64 issue slots are the scarce resource on this part); each thread owns
//   a fixed set of (a, b) entries and scatters them, mirrored, straight into
//   the 6x6-block BCSR matrix through a precomputed element-slot map.  No
//   element matrix is ever stored in global memory.
#include <math.h>

#include "a2ds_internal.h"

namespace a2ds {

// ---------------------------------------------------------------- tables
template <int O>
struct Dims {
  static constexpr int NN = O * O;
  static constexpr int NV = 6 * NN;
  static constexpr int NGP = NN;
  static constexpr int NTY = 4 * O * (O - 1) + (O - 1) * (O - 1);
  static constexpr int TPE = NV <= 32 ? 32 : 64;  // threads per element
  static constexpr int NTRI = NV * (NV + 1) / 2;
  static constexpr int EPT = (NTRI + TPE - 1) / TPE;
  static constexpr int EPB = 128 / TPE;  // elements per block
};

// Parametric tables for one element order (shape functions evaluated at the
// Gauss, tying and node points; tying interpolation weights at the Gauss
// points).  Values follow the reference's formulas and 15-digit Gauss
// literals (TACSGaussQuadrature.h:23-29, TACSShellElementQuadBasis.h).
struct ShellTables {
  double gw[9];
  double gN[9][9], gNa[9][9], gNb[9][9];  // [gauss point][node]
  double gTy[9][28];                      // [gauss point][tying point]
  double tN[28][9], tNa[28][9], tNb[28][9];
  int tField[28];
  double nNa[9][9], nNb[9][9];            // [node point][node]
};
__constant__ ShellTables c_tab[2];
// The same tables with the node points in place of the Gauss points (element
// output at the visualization nodes, basis::getNodePoint order).
__constant__ ShellTables c_tab_vis[2];

enum { F11 = 0, F22 = 1, F12 = 2, F23 = 3, F13 = 4 };

static void h_lobatto(int o, double u, double *N, double *Nd) {
  if (o == 2) {
    N[0] = 0.5 * (1.0 - u);
    N[1] = 0.5 * (1.0 + u);
    Nd[0] = -0.5;
    Nd[1] = 0.5;
  } else {
    N[0] = -0.5 * u * (1.0 - u);
    N[1] = (1.0 - u) * (1.0 + u);
    N[2] = 0.5 * (1.0 + u) * u;
    Nd[0] = -0.5 + u;
    Nd[1] = -2.0 * u;
    Nd[2] = 0.5 + u;
  }
}
static void h_lagrange(int n, double u, const double *k, double *N) {
  for (int i = 0; i < n; i++) {
    N[i] = 1.0;
    for (int j = 0; j < n; j++)
      if (i != j) N[i] *= (u - k[j]) * (1.0 / (k[i] - k[j]));
  }
}
static void h_shape(int o, const double pt[2], double *N, double *Na, double *Nb) {
  double na[3], dna[3], nb[3], dnb[3];
  h_lobatto(o, pt[0], na, dna);
  h_lobatto(o, pt[1], nb, dnb);
  for (int j = 0; j < o; j++)
    for (int i = 0; i < o; i++) {
      N[i + o * j] = na[i] * nb[j];
      Na[i + o * j] = dna[i] * nb[j];
      Nb[i + o * j] = na[i] * dnb[j];
    }
}

static void build_tables(int o, ShellTables *T, bool at_nodes) {
  static const double gp2[2] = {-0.577350269189626, 0.577350269189626};
  static const double gp3[3] = {-0.774596669241483, 0.0, 0.774596669241483};
  static const double gw3[3] = {5.0 / 9.0, 8.0 / 9.0, 5.0 / 9.0};
  static const double lin[2] = {-1.0, 1.0}, zero1[1] = {0.0};
  memset(T, 0, sizeof(ShellTables));
  const int nn = o * o;
  for (int g = 0; g < nn; g++) {
    double pt[2];
    if (at_nodes) {
      pt[0] = -1.0 + (2.0 / (o - 1)) * (g % o);
      pt[1] = -1.0 + (2.0 / (o - 1)) * (g / o);
      T->gw[g] = 1.0;
    } else if (o == 2) {
      pt[0] = gp2[g % 2];
      pt[1] = gp2[g / 2];
      T->gw[g] = 1.0;
    } else {
      pt[0] = gp3[g % 3];
      pt[1] = gp3[g / 3];
      T->gw[g] = gw3[g % 3] * gw3[g / 3];
    }
    h_shape(o, pt, T->gN[g], T->gNa[g], T->gNb[g]);
    // tying interpolation at this gauss point (evalTyingInterp order)
    const double *ko = (o == 2) ? lin : gp3, *kr = (o == 2) ? zero1 : gp2;
    double na[3], nb[3], nar[3], nbr[3];
    h_lagrange(o, pt[0], ko, na);
    h_lagrange(o, pt[1], ko, nb);
    h_lagrange(o - 1, pt[0], kr, nar);
    h_lagrange(o - 1, pt[1], kr, nbr);
    double *N = T->gTy[g];
    for (int j = 0; j < o; j++)
      for (int i = 0; i < o - 1; i++) *N++ = nar[i] * nb[j];
    for (int j = 0; j < o - 1; j++)
      for (int i = 0; i < o; i++) *N++ = na[i] * nbr[j];
    for (int j = 0; j < o - 1; j++)
      for (int i = 0; i < o - 1; i++) *N++ = nar[i] * nbr[j];
    for (int j = 0; j < o - 1; j++)
      for (int i = 0; i < o; i++) *N++ = na[i] * nbr[j];
    for (int j = 0; j < o; j++)
      for (int i = 0; i < o - 1; i++) *N++ = nar[i] * nb[j];
  }
  // tying points (getTyingPoint order)
  const double *ko = (o == 2) ? lin : gp3, *kr = (o == 2) ? zero1 : gp2;
  int k = 0;
  const int nf[5] = {o * (o - 1), o * (o - 1), (o - 1) * (o - 1), o * (o - 1), o * (o - 1)};
  for (int f = 0; f < 5; f++) {
    for (int ty = 0; ty < nf[f]; ty++, k++) {
      double pt[2];
      if (f == F11 || f == F13) {
        pt[0] = kr[ty % (o - 1)];
        pt[1] = ko[ty / (o - 1)];
      } else if (f == F22 || f == F23) {
        pt[0] = ko[ty % o];
        pt[1] = kr[ty / o];
      } else {
        pt[0] = kr[ty % (o - 1)];
        pt[1] = kr[ty / (o - 1)];
      }
      T->tField[k] = f;
      h_shape(o, pt, T->tN[k], T->tNa[k], T->tNb[k]);
    }
  }
  for (int n = 0; n < nn; n++) {
    double pt[2] = {-1.0 + (2.0 / (o - 1)) * (n % o), -1.0 + (2.0 / (o - 1)) * (n / o)};
    double N[9];
    h_shape(o, pt, N, T->nNa[n], T->nNb[n]);
  }
}

int upload_shell_tables() {
  static ShellTables tabs[2], vis[2];
  build_tables(2, &tabs[0], false);
  build_tables(3, &tabs[1], false);
  build_tables(2, &vis[0], true);
  build_tables(3, &vis[1], true);
  A2DS_CUDA_TRY(cudaMemcpyToSymbol(c_tab, tabs, sizeof(tabs)));
  A2DS_CUDA_TRY(cudaMemcpyToSymbol(c_tab_vis, vis, sizeof(vis)));
  return 0;
}

// --------------------------------------------------------- device algebra
__device__ __forceinline__ void d_mm(const double *A, const double *B, double *C) {
#pragma unroll
  for (int i = 0; i < 3; i++)
#pragma unroll
    for (int j = 0; j < 3; j++)
      C[3 * i + j] = A[3 * i] * B[j] + A[3 * i + 1] * B[3 + j] + A[3 * i + 2] * B[6 + j];
}
__device__ __forceinline__ double d_inv3(const double *A, double *Ai) {
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
// T^T S T for symmetric S (6 entries: 11 12 13 22 23 33)
__device__ __forceinline__ void d_symm_tt(const double *T, const double *S, double *A) {
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
// adjoint of d_symm_tt
__device__ __forceinline__ void d_symm_tt_adj(const double *T, const double *dA, double *dS) {
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
// The natural shell frame, reproducing the reference's projection exactly
// (only t1[0] is updated, three times: TACSShellElementTransform.h:41-44).
__device__ __forceinline__ void d_transform(const double *Xxi, const double *n0, double *T) {
  double n[3] = {n0[0], n0[1], n0[2]};
  double inv = 1.0 / sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
  n[0] *= inv;
  n[1] *= inv;
  n[2] *= inv;
  double t1[3] = {Xxi[0], Xxi[2], Xxi[4]};
  double d = n[0] * t1[0] + n[1] * t1[1] + n[2] * t1[2];
  t1[0] = t1[0] - d * n[0];
  t1[0] = t1[0] - d * n[0];
  t1[0] = t1[0] - d * n[0];
  inv = 1.0 / sqrt(t1[0] * t1[0] + t1[1] * t1[1] + t1[2] * t1[2]);
  t1[0] *= inv;
  t1[1] *= inv;
  t1[2] *= inv;
  double t2[3] = {n[1] * t1[2] - n[2] * t1[1], n[2] * t1[0] - n[0] * t1[2],
                  n[0] * t1[1] - n[1] * t1[0]};
  T[0] = t1[0]; T[3] = t1[1]; T[6] = t1[2];
  T[1] = t2[0]; T[4] = t2[1]; T[7] = t2[2];
  T[2] = n[0];  T[5] = n[1];  T[8] = n[2];
}

// Isotropic shell stress resultants with zero offset: A = t Q, D = t^3/12 Q,
// As = 5/6 t G, drill = 10 As (TACSIsoShellConstitutive.cpp:192-226).
struct Stiff {
  double A0, A1, A3, A5, D0, D1, D3, D5, As, drill;
};
__device__ __forceinline__ Stiff d_stiff(double E, double nu, double t) {
  Stiff c;
  double Q = E / (1.0 - nu * nu), G = 0.5 * E / (1.0 + nu);
  double I = t * t * t / 12.0;
  c.A0 = t * Q;
  c.A1 = t * (nu * Q);
  c.A3 = t * Q;
  c.A5 = t * G;
  c.D0 = I * Q;
  c.D1 = I * (nu * Q);
  c.D3 = I * Q;
  c.D5 = I * G;
  c.As = (5.0 / 6.0) * c.A5;
  c.drill = 0.5 * 10.0 * (c.As + c.As);
  return c;
}
// d/dt of d_stiff: A' = Q, D' = t^2/4 Q, As' = 5/6 G, drill' = 10 As'
// (TACSIsoShellConstitutive::addStressDVSens, TACSIsoShellConstitutive.cpp:229-251).
__device__ __forceinline__ Stiff d_stiff_dt(double E, double nu, double t) {
  Stiff c;
  double Q = E / (1.0 - nu * nu), G = 0.5 * E / (1.0 + nu);
  double I = 0.25 * t * t;
  c.A0 = Q;
  c.A1 = nu * Q;
  c.A3 = Q;
  c.A5 = G;
  c.D0 = I * Q;
  c.D1 = I * (nu * Q);
  c.D3 = I * Q;
  c.D5 = I * G;
  c.As = (5.0 / 6.0) * c.A5;
  c.drill = 0.5 * 10.0 * (c.As + c.As);
  return c;
}
__device__ __forceinline__ void d_stress(const Stiff &c, const double *e, double *s) {
  s[0] = c.A0 * e[0] + c.A1 * e[1];
  s[1] = c.A1 * e[0] + c.A3 * e[1];
  s[2] = c.A5 * e[2];
  s[3] = c.D0 * e[3] + c.D1 * e[4];
  s[4] = c.D1 * e[3] + c.D3 * e[4];
  s[5] = c.D5 * e[5];
  s[6] = c.As * e[6];
  s[7] = c.As * e[7];
  s[8] = c.drill * e[8];
}

// ------------------------------------------------------- shared workspace
template <int O>
struct ElemShared {
  using D = Dims<O>;
  double X[D::NN * 3], fn[D::NN * 3], Tn[D::NN * 9], XdinvTn[D::NN * 9];
  double st[D::NV];
  double drot[D::NN * D::NV];
  double ety0[D::NTY * D::NV];  // d(tying strain)/dq at the zero state
  double ety1[D::NTY * D::NV];  // P_k(e_j, state): state-dependent part
  double tyX[D::NTY * 6], tyn[D::NTY * 3], tyU[D::NTY * 6], tyd[D::NTY * 3];
  double omega[D::NTY];
  double gT[D::NGP * 9], gXT[D::NGP * 9], gXzT[D::NGP * 9], gwdet[D::NGP];
  double gU[D::NGP * 12];
  double B0[9 * D::NV], B1[9 * D::NV], CBL[9 * D::NV], CBR[9 * D::NV];
  double A[3 * D::NV], bcv[4 * D::NV];
  double s[9], e[9];
  double Sdd[D::NN * D::NN], Srd[D::NN * D::NN];
};

template <int O>
__device__ __forceinline__ void esync() {
  if (Dims<O>::TPE == 32)
    __syncwarp();
  else
    __syncthreads();
}

// triangular index -> (a, b), a <= b, idx = b(b+1)/2 + a
__device__ __forceinline__ void tri_ab(int idx, int &a, int &b) {
  int bb = (int)((sqrtf(8.0f * (float)idx + 1.0f) - 1.0f) * 0.5f);
  while (bb * (bb + 1) / 2 > idx) bb--;
  while ((bb + 1) * (bb + 2) / 2 <= idx) bb++;
  b = bb;
  a = idx - bb * (bb + 1) / 2;
}

template <int O, int MODE, int NL>
__global__ void __launch_bounds__(128) shell_kernel(ElemLaunch L) {
  using D = Dims<O>;
  constexpr int NN = D::NN, NV = D::NV, NTY = D::NTY, NGP = D::NGP, TPE = D::TPE;
  const ShellTables &tb = (MODE == MODE_OUT) ? c_tab_vis[O - 2] : c_tab[O - 2];
  extern __shared__ double smem_raw[];
  const int eslot = threadIdx.x / TPE;
  const int tid = threadIdx.x % TPE;
  ElemShared<O> &S = reinterpret_cast<ElemShared<O> *>(smem_raw)[eslot];

  const int ei = blockIdx.x * D::EPB + eslot;
  // Multi-warp elements use __syncthreads, so whole blocks stay resident
  // even past the end; their work is masked.
  const bool active = ei < L.num_elements;
  const int e = active ? (L.elem_list ? L.elem_list[ei] : ei) : 0;
  const int *conn = L.conn + (size_t)e * NN;

  // Variants that need the state (nonlinear tangent, G direction, residual)
  constexpr bool OUT = (MODE == MODE_OUT);
  constexpr bool NEED_STATE = (MODE == MODE_G) || (MODE == MODE_R) || (MODE == MODE_KR) || NL || OUT;
  constexpr bool NEED_P = (MODE == MODE_G) || NL;  // bilinear-form terms present
  constexpr bool NEED_STRESS =
      (MODE == MODE_G) || (MODE == MODE_R) || (MODE == MODE_KR) || NL || OUT;
  constexpr bool NEED_MAT = (MODE != MODE_R) && !OUT;
  constexpr bool NEED_RES = (MODE == MODE_R) || (MODE == MODE_KR);

  // ---- gather
  if (active) {
    for (int i = tid; i < NN * 3; i += TPE) {
      double x = L.X[(size_t)conn[i / 3] * 3 + i % 3];
      if (L.cstride && !L.xstate && i == L.xk) x += L.xh;  // coordinate step
      S.X[i] = x;
    }
    for (int i = tid; i < NV; i += TPE) {
      double q = (NEED_STATE && L.state) ? L.state[(size_t)conn[i / 6] * 6 + i % 6] : 0.0;
      if (NEED_STATE && L.cstride && L.xstate && i == L.xk) q += L.xh;  // state step
      S.st[i] = q;
    }
  }
  const double t = active ? L.tvals[L.tgroup[e]] : 1.0;
  const Stiff C = L.dconst ? d_stiff_dt(L.E, L.nu, t) : d_stiff(L.E, L.nu, t);
  esync<O>();

  // ---- node normals and node frames (TacsShellComputeNodeNormals,
  //      TacsShellComputeDrillStrain geometry)
  if (tid < NN) {
    double Xxi[6] = {0, 0, 0, 0, 0, 0};
    for (int m = 0; m < NN; m++) {
      double a = tb.nNa[tid][m], b = tb.nNb[tid][m];
      for (int c = 0; c < 3; c++) {
        Xxi[2 * c] += a * S.X[3 * m + c];
        Xxi[2 * c + 1] += b * S.X[3 * m + c];
      }
    }
    double a[3] = {Xxi[0], Xxi[2], Xxi[4]}, b[3] = {Xxi[1], Xxi[3], Xxi[5]};
    double n[3] = {a[1] * b[2] - a[2] * b[1], a[2] * b[0] - a[0] * b[2], a[0] * b[1] - a[1] * b[0]};
    double nrm = sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
    if (nrm != 0.0) {
      double s = 1.0 / nrm;
      n[0] *= s;
      n[1] *= s;
      n[2] *= s;
    }
    for (int c = 0; c < 3; c++) S.fn[3 * tid + c] = n[c];
    double Xd[9] = {Xxi[0], Xxi[1], n[0], Xxi[2], Xxi[3], n[1], Xxi[4], Xxi[5], n[2]};
    double T[9], Xdinv[9];
    d_transform(Xxi, n, T);
    d_inv3(Xd, Xdinv);
    double XT[9];
    d_mm(Xdinv, T, XT);
    for (int c = 0; c < 9; c++) {
      S.Tn[9 * tid + c] = T[c];
      S.XdinvTn[9 * tid + c] = XT[c];
    }
  }
  esync<O>();

  // ---- tying-point geometry and state; Gauss-point geometry and state
  for (int k = tid; k < NTY; k += TPE) {
    double Xxi[6] = {0, 0, 0, 0, 0, 0}, n0[3] = {0, 0, 0}, U[6] = {0, 0, 0, 0, 0, 0},
           d0[3] = {0, 0, 0};
    for (int m = 0; m < NN; m++) {
      double N = tb.tN[k][m], a = tb.tNa[k][m], b = tb.tNb[k][m];
      const double *fm = &S.fn[3 * m];
      for (int c = 0; c < 3; c++) {
        Xxi[2 * c] += a * S.X[3 * m + c];
        Xxi[2 * c + 1] += b * S.X[3 * m + c];
        n0[c] += N * fm[c];
      }
      if (NEED_STATE) {
        const double *q = &S.st[6 * m + 3];
        double dm[3] = {q[1] * fm[2] - q[2] * fm[1], q[2] * fm[0] - q[0] * fm[2],
                        q[0] * fm[1] - q[1] * fm[0]};
        for (int c = 0; c < 3; c++) {
          U[2 * c] += a * S.st[6 * m + c];
          U[2 * c + 1] += b * S.st[6 * m + c];
          d0[c] += N * dm[c];
        }
      }
    }
    for (int c = 0; c < 6; c++) {
      S.tyX[6 * k + c] = Xxi[c];
      S.tyU[6 * k + c] = U[c];
    }
    for (int c = 0; c < 3; c++) {
      S.tyn[3 * k + c] = n0[c];
      S.tyd[3 * k + c] = d0[c];
    }
    S.omega[k] = 0.0;
  }
  for (int g = tid; g < NGP; g += TPE) {
    double Xxi[6] = {0, 0, 0, 0, 0, 0}, n0[3] = {0, 0, 0}, nxi[6] = {0, 0, 0, 0, 0, 0};
    double u0xi[6] = {0, 0, 0, 0, 0, 0}, d0[3] = {0, 0, 0}, d0xi[6] = {0, 0, 0, 0, 0, 0};
    for (int m = 0; m < NN; m++) {
      double N = tb.gN[g][m], a = tb.gNa[g][m], b = tb.gNb[g][m];
      const double *fm = &S.fn[3 * m];
      for (int c = 0; c < 3; c++) {
        Xxi[2 * c] += a * S.X[3 * m + c];
        Xxi[2 * c + 1] += b * S.X[3 * m + c];
        n0[c] += N * fm[c];
        nxi[2 * c] += a * fm[c];
        nxi[2 * c + 1] += b * fm[c];
      }
      if (NEED_STATE) {
        const double *q = &S.st[6 * m + 3];
        double dm[3] = {q[1] * fm[2] - q[2] * fm[1], q[2] * fm[0] - q[0] * fm[2],
                        q[0] * fm[1] - q[1] * fm[0]};
        for (int c = 0; c < 3; c++) {
          u0xi[2 * c] += a * S.st[6 * m + c];
          u0xi[2 * c + 1] += b * S.st[6 * m + c];
          d0[c] += N * dm[c];
          d0xi[2 * c] += a * dm[c];
          d0xi[2 * c + 1] += b * dm[c];
        }
      }
    }
    double T[9], Xd[9] = {Xxi[0], Xxi[1], n0[0], Xxi[2], Xxi[3], n0[1], Xxi[4], Xxi[5], n0[2]};
    double Xdz[9] = {nxi[0], nxi[1], 0.0, nxi[2], nxi[3], 0.0, nxi[4], nxi[5], 0.0};
    d_transform(Xxi, n0, T);
    double Xdinv[9], XT[9], XzT[9], neg[9];
    double det = d_inv3(Xd, Xdinv);
    d_mm(Xdinv, Xdz, neg);
    for (int c = 0; c < 9; c++) neg[c] = -neg[c];
    d_mm(Xdinv, T, XT);
    d_mm(neg, XT, XzT);
    for (int c = 0; c < 9; c++) {
      S.gT[9 * g + c] = T[c];
      S.gXT[9 * g + c] = XT[c];
      S.gXzT[9 * g + c] = XzT[c];
    }
    S.gwdet[g] = det * tb.gw[g];
    if (NEED_STATE) {
      // u0x = T^T u0d XT, u1x = T^T (u1d XT + u0d XzT); keep columns 0, 1
      double u0d[9] = {u0xi[0], u0xi[1], d0[0], u0xi[2], u0xi[3], d0[1], u0xi[4], u0xi[5], d0[2]};
      double u1d[9] = {d0xi[0], d0xi[1], 0.0, d0xi[2], d0xi[3], 0.0, d0xi[4], d0xi[5], 0.0};
      double t0[9], t1[9], u0x[9], u1x[9];
      d_mm(u0d, XT, t0);
      d_mm(u1d, XT, t1);
      double t2[9];
      d_mm(u0d, XzT, t2);
      for (int c = 0; c < 9; c++) t1[c] += t2[c];
      for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) {
          u0x[3 * i + j] = T[i] * t0[j] + T[3 + i] * t0[3 + j] + T[6 + i] * t0[6 + j];
          u1x[3 * i + j] = T[i] * t1[j] + T[3 + i] * t1[3 + j] + T[6 + i] * t1[6 + j];
        }
      double *gu = &S.gU[12 * g];
      for (int i = 0; i < 3; i++) {
        gu[i] = u0x[3 * i];          // U0c0
        gu[3 + i] = u0x[3 * i + 1];  // U0c1
        gu[6 + i] = u1x[3 * i];      // U1c0
        gu[9 + i] = u1x[3 * i + 1];  // U1c1
      }
    }
  }
  esync<O>();

  // ---- per-column element-level derivatives: drill rows and tying strains
  for (int j = tid; j < NV; j += TPE) {
    const int mj = j / 6, cj = j % 6;
    // drill strain at each node n: et_n = 1/2 (Ct[3] + u0x[3] - Ct[1] - u0x[1])
    for (int n = 0; n < NN; n++) {
      const double *Tm = &S.Tn[9 * n];
      double v = 0.0;
      if (cj < 3) {
        const double *XT = &S.XdinvTn[9 * n];
        double a = tb.nNa[n][mj], b = tb.nNb[n][mj];
        double w0 = a * XT[0] + b * XT[3], w1 = a * XT[1] + b * XT[4];
        v = 0.5 * (Tm[3 * cj + 1] * w0 - Tm[3 * cj] * w1);
      } else if (mj == n) {
        // d/dq_r of 1/2 (Ct[3]-Ct[1]) with Ct = T^T (I - q^x) T is
        // -(t0 x t1)_r, t0 and t1 the first two columns of T
        const int r = cj - 3;
        double c0[3] = {Tm[0], Tm[3], Tm[6]}, c1[3] = {Tm[1], Tm[4], Tm[7]};
        double cr[3] = {c0[1] * c1[2] - c0[2] * c1[1], c0[2] * c1[0] - c0[0] * c1[2],
                        c0[0] * c1[1] - c0[1] * c1[0]};
        v = -cr[r];
      }
      S.drot[n * NV + j] = v;
    }
    // tying strain derivatives: zero-state part and state-dependent part
    double dv[3] = {0, 0, 0};
    if (cj >= 3) {
      const double *fm = &S.fn[3 * mj];
      const int r = cj - 3;  // e_r x fn
      if (r == 0) { dv[1] = -fm[2]; dv[2] = fm[1]; }
      if (r == 1) { dv[0] = fm[2]; dv[2] = -fm[0]; }
      if (r == 2) { dv[0] = -fm[1]; dv[1] = fm[0]; }
    }
    for (int k = 0; k < NTY; k++) {
      const int f = tb.tField[k];
      const double *Xx = &S.tyX[6 * k], *n0 = &S.tyn[3 * k], *U = &S.tyU[6 * k],
                   *d0 = &S.tyd[3 * k];
      double v0 = 0.0, v1 = 0.0;
      if (cj < 3) {
        const double a = tb.tNa[k][mj], b = tb.tNb[k][mj];
        const int c = cj;
        if (f == F11) {
          v0 = a * Xx[2 * c];
          v1 = a * U[2 * c];
        } else if (f == F22) {
          v0 = b * Xx[2 * c + 1];
          v1 = b * U[2 * c + 1];
        } else if (f == F12) {
          v0 = 0.5 * (a * Xx[2 * c + 1] + b * Xx[2 * c]);
          v1 = 0.5 * (a * U[2 * c + 1] + b * U[2 * c]);
        } else if (f == F23) {
          v0 = 0.5 * b * n0[c];
          v1 = 0.5 * b * d0[c];
        } else {
          v0 = 0.5 * a * n0[c];
          v1 = 0.5 * a * d0[c];
        }
      } else {
        const double N = tb.tN[k][mj];
        if (f == F23) {
          v0 = 0.5 * N * (Xx[1] * dv[0] + Xx[3] * dv[1] + Xx[5] * dv[2]);
          v1 = 0.5 * N * (U[1] * dv[0] + U[3] * dv[1] + U[5] * dv[2]);
        } else if (f == F13) {
          v0 = 0.5 * N * (Xx[0] * dv[0] + Xx[2] * dv[1] + Xx[4] * dv[2]);
          v1 = 0.5 * N * (U[0] * dv[0] + U[2] * dv[1] + U[4] * dv[2]);
        }
      }
      S.ety0[k * NV + j] = v0;
      S.ety1[k * NV + j] = NEED_P ? v1 : 0.0;
    }
  }
  esync<O>();

  double acc[D::EPT];
#pragma unroll
  for (int m = 0; m < D::EPT; m++) acc[m] = 0.0;
  double racc[(NV + TPE - 1) / TPE];
#pragma unroll
  for (int m = 0; m < (NV + TPE - 1) / TPE; m++) racc[m] = 0.0;

  // Thermal strain of the current temperature (TACSIsoShellConstitutive::
  // evalThermalStrain): only membrane e0, e1.
  const double eth = L.alpha * L.temperature;

  for (int g = 0; g < NGP; g++) {
    const double *T = &S.gT[9 * g], *XT = &S.gXT[9 * g], *XzT = &S.gXzT[9 * g];
    const double wdet = S.gwdet[g];
    // ---- columns of B0 (and P(e_j, state))
    for (int j = tid; j < NV; j += TPE) {
      const int mj = j / 6, cj = j % 6;
      double a[3], b[3], c[3];
      const double N = tb.gN[g][mj], Na = tb.gNa[g][mj], Nb = tb.gNb[g][mj];
      if (cj < 3) {
        a[0] = T[3 * cj];
        a[1] = T[3 * cj + 1];
        a[2] = T[3 * cj + 2];
        for (int i = 0; i < 3; i++) {
          b[i] = Na * XT[i] + Nb * XT[3 + i];
          c[i] = Na * XzT[i] + Nb * XzT[3 + i];
        }
      } else {
        const double *fm = &S.fn[3 * mj];
        const int r = cj - 3;
        double dv[3] = {0, 0, 0};
        if (r == 0) { dv[1] = -fm[2]; dv[2] = fm[1]; }
        if (r == 1) { dv[0] = fm[2]; dv[2] = -fm[0]; }
        if (r == 2) { dv[0] = -fm[1]; dv[1] = fm[0]; }
        for (int i = 0; i < 3; i++) a[i] = T[i] * dv[0] + T[3 + i] * dv[1] + T[6 + i] * dv[2];
        for (int i = 0; i < 3; i++) {
          b[i] = N * XT[6 + i];
          c[i] = Na * XT[i] + Nb * XT[3 + i] + N * XzT[6 + i];
        }
      }
      // membrane / transverse shear through the tying strains
      double gty[6] = {0, 0, 0, 0, 0, 0}, gty1[6] = {0, 0, 0, 0, 0, 0};
      for (int k = 0; k < NTY; k++) {
        const double w = tb.gTy[g][k];
        const int f = tb.tField[k];
        const int slot = (f == F11) ? 0 : (f == F22) ? 3 : (f == F12) ? 1 : (f == F23) ? 4 : 2;
        gty[slot] += w * S.ety0[k * NV + j];
        if (NEED_P) gty1[slot] += w * S.ety1[k * NV + j];
      }
      double e0ty[6];
      d_symm_tt(XT, gty, e0ty);
      double *B0 = S.B0;
      B0[0 * NV + j] = e0ty[0];
      B0[1 * NV + j] = e0ty[3];
      B0[2 * NV + j] = 2.0 * e0ty[1];
      B0[3 * NV + j] = a[0] * c[0];
      B0[4 * NV + j] = a[1] * c[1];
      B0[5 * NV + j] = a[0] * c[1] + a[1] * c[0];
      B0[6 * NV + j] = 2.0 * e0ty[4];
      B0[7 * NV + j] = 2.0 * e0ty[2];
      double et = 0.0;
      for (int n = 0; n < NN; n++) et += tb.gN[g][n] * S.drot[n * NV + j];
      B0[8 * NV + j] = et;
      if (NEED_P) {
        double e1ty[6];
        d_symm_tt(XT, gty1, e1ty);
        const double *gu = &S.gU[12 * g];
        double aU0c0 = a[0] * gu[0] + a[1] * gu[1] + a[2] * gu[2];
        double aU0c1 = a[0] * gu[3] + a[1] * gu[4] + a[2] * gu[5];
        double aU1c0 = a[0] * gu[6] + a[1] * gu[7] + a[2] * gu[8];
        double aU1c1 = a[0] * gu[9] + a[1] * gu[10] + a[2] * gu[11];
        double *B1 = S.B1;
        B1[0 * NV + j] = e1ty[0];
        B1[1 * NV + j] = e1ty[3];
        B1[2 * NV + j] = 2.0 * e1ty[1];
        B1[3 * NV + j] = b[0] * aU1c0 + c[0] * aU0c0;
        B1[4 * NV + j] = b[1] * aU1c1 + c[1] * aU0c1;
        B1[5 * NV + j] = b[0] * aU1c1 + c[0] * aU0c1 + b[1] * aU1c0 + c[1] * aU0c0;
        B1[6 * NV + j] = 2.0 * e1ty[4];
        B1[7 * NV + j] = 2.0 * e1ty[2];
        B1[8 * NV + j] = 0.0;
        S.A[3 * j] = a[0];
        S.A[3 * j + 1] = a[1];
        S.A[3 * j + 2] = a[2];
        S.bcv[4 * j] = b[0];
        S.bcv[4 * j + 1] = b[1];
        S.bcv[4 * j + 2] = c[0];
        S.bcv[4 * j + 3] = c[1];
      }
    }
    esync<O>();

    // ---- stress at the state (scaled by wdet)
    if (NEED_STRESS) {
      if (tid < 9) {
        // MODE_G: derivative of the strain along the path, B0 w.
        // Otherwise the strain at the state, (B0 + 1/2 P(., u)) u.
        const double half = (MODE == MODE_G) ? 0.0 : 0.5;
        double v = 0.0;
        for (int j = 0; j < NV; j++) {
          double bj = S.B0[tid * NV + j];
          if (NEED_P) bj += half * S.B1[tid * NV + j];
          v += S.st[j] * bj;
        }
        S.e[tid] = v;
      }
      esync<O>();
      if (OUT) {
        // output at node point g: the strain and C e (evalStress of the
        // total strain, as getOutputData)
        if (tid == 0 && active && L.out) {
          double em[9], s[9];
          for (int i = 0; i < 9; i++) em[i] = S.e[i];
          d_stress(C, em, s);
          double *o = L.out + ((size_t)e * NN + g) * 18;
          for (int i = 0; i < 9; i++) {
            o[i] = em[i];
            o[9 + i] = s[i];
          }
        }
        esync<O>();
        continue;  // nothing else at this point (uniform over the element)
      }
      if (tid == 0) {
        double em[9];
        for (int i = 0; i < 9; i++) em[i] = S.e[i];
        em[0] -= eth;
        em[1] -= eth;
        double s[9];
        d_stress(C, em, s);
        for (int i = 0; i < 9; i++) S.s[i] = wdet * s[i];
      }
      esync<O>();
      if (NEED_P) {
        // tying-point weights: omega_k += N_k(g) (T-adjoint of de0ty)
        for (int k = tid; k < NTY; k += TPE) {
          double de0ty[6] = {S.s[0], 2.0 * S.s[2], 2.0 * S.s[7], S.s[1], 2.0 * S.s[6], 0.0};
          double dg[6];
          d_symm_tt_adj(XT, de0ty, dg);
          const int f = tb.tField[k];
          const int slot = (f == F11) ? 0 : (f == F22) ? 3 : (f == F12) ? 1 : (f == F23) ? 4 : 2;
          S.omega[k] += tb.gTy[g][k] * dg[slot];
        }
      }
    }

    // ---- left/right strain operators and their stress images
    for (int j = tid, m = 0; j < NV; j += TPE, m++) {
      double BL[9], BR[9];
      for (int r = 0; r < 9; r++) {
        double b0 = S.B0[r * NV + j];
        double b1 = NEED_P ? S.B1[r * NV + j] : 0.0;
        if (MODE == MODE_G) {
          BL[r] = b0;
          BR[r] = b1;
        } else {
          BL[r] = NL ? (b0 + b1) : b0;
          BR[r] = BL[r];
        }
      }
      if (NEED_RES) {
        double v = 0.0;
        for (int r = 0; r < 9; r++) v += BL[r] * S.s[r];
        racc[m] += v;
      }
      if (NEED_MAT) {
        double sL[9], sR[9];
        d_stress(C, BL, sL);
        for (int r = 0; r < 9; r++) S.CBL[r * NV + j] = wdet * sL[r];
        if (MODE == MODE_G) {
          d_stress(C, BR, sR);
          for (int r = 0; r < 9; r++) S.CBR[r * NV + j] = wdet * sR[r];
        } else if (NL) {
          for (int r = 0; r < 9; r++) S.B1[r * NV + j] = BL[r];  // B(u) kept in B1
        }
      }
    }
    esync<O>();

    // ---- entries of the upper triangle
    if (NEED_MAT) {
      const double *BLs = (NL && MODE != MODE_G) ? S.B1 : S.B0;
#pragma unroll
      for (int m = 0; m < D::EPT; m++) {
        int idx = tid + TPE * m;
        if (idx < D::NTRI) {
          int a, b;
          tri_ab(idx, a, b);
          double v = 0.0;
          if (MODE == MODE_G) {
            // P(., w)^T C B0 + B0^T C P(., w)  (CBL = C B0, CBR = C P)
#pragma unroll
            for (int r = 0; r < 9; r++)
              v += S.B1[r * NV + a] * S.CBL[r * NV + b] + S.B0[r * NV + a] * S.CBR[r * NV + b];
          } else {
#pragma unroll
            for (int r = 0; r < 9; r++) v += BLs[r * NV + a] * S.CBL[r * NV + b];
          }
          if (NEED_P) {
            // bending part of s . P(e_a, e_b)
            const double *Aa = &S.A[3 * a], *Ab = &S.A[3 * b];
            const double *pa = &S.bcv[4 * a], *pb = &S.bcv[4 * b];
            double AA = Aa[0] * Ab[0] + Aa[1] * Ab[1] + Aa[2] * Ab[2];
            double br = S.s[3] * (pa[0] * pb[2] + pb[0] * pa[2]) +
                        S.s[4] * (pa[1] * pb[3] + pb[1] * pa[3]) +
                        S.s[5] * (pa[0] * pb[3] + pa[2] * pb[1] + pb[0] * pa[3] + pb[2] * pa[1]);
            v += AA * br;
          }
          acc[m] += v;
        }
      }
    }
    esync<O>();
  }

  // ---- tying part of s . P(e_a, e_b), through node-pair tables
  if (NEED_MAT && NEED_P) {
    for (int p = tid; p < NN * NN; p += TPE) {
      const int ma = p / NN, mb = p % NN;
      double sdd = 0.0, srd = 0.0;
      for (int k = 0; k < NTY; k++) {
        const int f = tb.tField[k];
        const double w = S.omega[k];
        if (f == F11) sdd += w * tb.tNa[k][ma] * tb.tNa[k][mb];
        else if (f == F22) sdd += w * tb.tNb[k][ma] * tb.tNb[k][mb];
        else if (f == F12)
          sdd += w * 0.5 * (tb.tNa[k][ma] * tb.tNb[k][mb] + tb.tNb[k][ma] * tb.tNa[k][mb]);
        else if (f == F23) srd += w * 0.5 * tb.tN[k][ma] * tb.tNb[k][mb];
        else srd += w * 0.5 * tb.tN[k][ma] * tb.tNa[k][mb];
      }
      S.Sdd[p] = sdd;
      S.Srd[p] = srd;  // rows: rotation node ma, cols: displacement node mb
    }
    esync<O>();
#pragma unroll
    for (int m = 0; m < D::EPT; m++) {
      int idx = tid + TPE * m;
      if (idx < D::NTRI) {
        int a, b;
        tri_ab(idx, a, b);
        const int ma = a / 6, ca = a % 6, mb = b / 6, cb = b % 6;
        double v = 0.0;
        if (ca < 3 && cb < 3) {
          if (ca == cb) v = S.Sdd[ma * NN + mb];
        } else if (ca >= 3 && cb < 3) {
          const double *fm = &S.fn[3 * ma];
          const int r = ca - 3;
          double dv[3] = {0, 0, 0};
          if (r == 0) { dv[1] = -fm[2]; dv[2] = fm[1]; }
          if (r == 1) { dv[0] = fm[2]; dv[2] = -fm[0]; }
          if (r == 2) { dv[0] = -fm[1]; dv[1] = fm[0]; }
          v = S.Srd[ma * NN + mb] * dv[cb];
        } else if (ca < 3 && cb >= 3) {
          const double *fm = &S.fn[3 * mb];
          const int r = cb - 3;
          double dv[3] = {0, 0, 0};
          if (r == 0) { dv[1] = -fm[2]; dv[2] = fm[1]; }
          if (r == 1) { dv[0] = fm[2]; dv[2] = -fm[0]; }
          if (r == 2) { dv[0] = -fm[1]; dv[1] = fm[0]; }
          v = S.Srd[mb * NN + ma] * dv[ca];
        }
        acc[m] += v;
      }
    }
  }

  if (!active) return;

  // ---- contractions ccoef cx^T M_e cy (+ ccoef2 cx2^T M_e cy2) into the
  //      element's design group, or into slot xk of the element's row of
  //      cout when cstride != 0 (a warp belongs to one element: reduce in
  //      the warp, one atomic per warp)
  if (NEED_MAT && L.cout) {
    double v = 0.0, v2 = 0.0;
#pragma unroll
    for (int m = 0; m < D::EPT; m++) {
      int idx = tid + TPE * m;
      if (idx < D::NTRI) {
        int a, b;
        tri_ab(idx, a, b);
        const size_t ga = (size_t)conn[a / 6] * 6 + a % 6, gb = (size_t)conn[b / 6] * 6 + b % 6;
        const double xy = (a == b) ? L.cx[ga] * L.cy[ga] : L.cx[ga] * L.cy[gb] + L.cx[gb] * L.cy[ga];
        v += acc[m] * xy;
        if (L.cx2) {
          const double xy2 =
              (a == b) ? L.cx2[ga] * L.cy2[ga] : L.cx2[ga] * L.cy2[gb] + L.cx2[gb] * L.cy2[ga];
          v2 += acc[m] * xy2;
        }
      }
    }
    v = L.ccoef * v + L.ccoef2 * v2;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    double *dst = L.cstride ? L.cout + (size_t)e * L.cstride + L.xk : L.cout + L.tgroup[e];
    if ((threadIdx.x & 31) == 0) atomicAdd(dst, v);
    return;
  }

  // ---- residual contraction ccoef cx^T R_e into slot xk of the element's
  //      row of cout (coordinate derivatives of adjoint-residual products)
  if (NEED_RES && L.cout) {
    double v = 0.0;
    for (int j = tid, m = 0; j < NV; j += TPE, m++)
      v += racc[m] * L.cx[(size_t)conn[j / 6] * 6 + j % 6];
    v *= L.ccoef;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    double *dst = L.cstride ? L.cout + (size_t)e * L.cstride + L.xk : L.cout + L.tgroup[e];
    if ((threadIdx.x & 31) == 0) atomicAdd(dst, v);
    return;
  }

  // ---- scatter into the BCSR blocks (mirrored)
  if (NEED_MAT && L.vals) {
    const int *slots = L.slots + (size_t)e * NN * NN;
#pragma unroll
    for (int m = 0; m < D::EPT; m++) {
      int idx = tid + TPE * m;
      if (idx < D::NTRI) {
        int a, b;
        tri_ab(idx, a, b);
        const int ma = a / 6, ia = a % 6, mb = b / 6, ib = b % 6;
        double *p1 = L.vals + (size_t)slots[ma * NN + mb] * 36 + ia * 6 + ib;
        double *p2 = L.vals + (size_t)slots[mb * NN + ma] * 36 + ib * 6 + ia;
        if (L.atomic_scatter) {
          atomicAdd(p1, acc[m]);
          if (a != b) atomicAdd(p2, acc[m]);
        } else {
          *p1 += acc[m];
          if (a != b) *p2 += acc[m];
        }
      }
    }
  }
  if (NEED_RES && L.res) {
    for (int j = tid, m = 0; j < NV; j += TPE, m++) {
      double *p = L.res + (size_t)conn[j / 6] * 6 + j % 6;
      if (L.atomic_scatter)
        atomicAdd(p, racc[m]);
      else
        *p += racc[m];
    }
  }
}

template <int O, int MODE, int NL>
static int launch_one(const ElemLaunch &L, cudaStream_t s) {
  using D = Dims<O>;
  const size_t shm = sizeof(ElemShared<O>) * D::EPB;
  static bool configured = false;
  if (!configured) {
    A2DS_CUDA_TRY(cudaFuncSetAttribute(shell_kernel<O, MODE, NL>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int)shm));
    configured = true;
  }
  const int blocks = (L.num_elements + D::EPB - 1) / D::EPB;
  if (blocks == 0) return 0;
  shell_kernel<O, MODE, NL><<<blocks, 128, shm, s>>>(L);
  A2DS_CUDA_TRY(cudaGetLastError());
  return 0;
}

template <int O>
static int launch_order(const ElemLaunch &L, cudaStream_t s) {
  const bool nl = L.nonlinear != 0;
  switch (L.mode) {
    case MODE_K: return nl ? launch_one<O, MODE_K, 1>(L, s) : launch_one<O, MODE_K, 0>(L, s);
    case MODE_G: return launch_one<O, MODE_G, 0>(L, s);
    case MODE_R: return nl ? launch_one<O, MODE_R, 1>(L, s) : launch_one<O, MODE_R, 0>(L, s);
    case MODE_KR: return nl ? launch_one<O, MODE_KR, 1>(L, s) : launch_one<O, MODE_KR, 0>(L, s);
    case MODE_OUT: return nl ? launch_one<O, MODE_OUT, 1>(L, s) : launch_one<O, MODE_OUT, 0>(L, s);
  }
  return fail(A2DS_ERR_ARG, "unknown element kernel mode");
}

int launch_element_kernel(const ElemLaunch &L, cudaStream_t s) {
  if (L.order == 2) return launch_order<2>(L, s);
  if (L.order == 3) return launch_order<3>(L, s);
  return fail(A2DS_ERR_ARG, "element order must be 2 (Quad4) or 3 (Quad9)");
}

}  // namespace a2ds
