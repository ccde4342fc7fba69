// Factorization handles, BLAS-1 kernels and the shift-invert Lanczos
// buckling solve.
//
// Reference path (TACSLinearBuckling::solve, src/TACSBuckling.cpp:197-278):
// K at the zero state, the load path from K u = f, G along u, the shifted
// operator and SEP::solve (src/bpmat/GSEP.cpp:485-596), a Lanczos iteration
// on (K + sigma G)^{-1} K with full K-orthogonalisation.
//
// Differences by design (results agree to the eigenvalue tolerance):
// * the shifted matrix A = K + sigma G is factored directly and applied with
//   iterative refinement, instead of GMRES on A preconditioned by a factor
//   of K (one triangular-solve pair per Lanczos step instead of tens);
// * K q_j is kept for every Lanczos vector, so the K-inner products of the
//   full orthogonalisation are dot products, not one K SpMV each;
// * Ritz pairs are tested for convergence (residual estimate
//   |beta_m y_m| relative to |mu|) instead of stopping after exactly
//   num_eigvals steps (SEP::checkConverged returns 1 as soon as
//   n >= neigvals, src/bpmat/GSEP.cpp:754-789).
#include <math.h>
#include <stdint.h>
#include <string.h>

#include <algorithm>
#include <chrono>
#include <vector>

#include "a2ds_internal.h"
#include "host_graph.h"
#include "ilu.h"
#include "kernels.h"
#include "runtime.h"

struct a2ds_pc_s {
  a2ds_bcsr mat = nullptr;
  a2ds::Factor f;
};

namespace a2ds {

// ------------------------------------------------------------- BLAS-1
__global__ void k_scale(double *x, double a, size_t n) {
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x)
    x[i] *= a;
}
__global__ void k_axpby(double *y, double a, const double *x, double b, size_t n) {
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x)
    y[i] = a * x[i] + b * y[i];
}
__global__ void k_f64_to_f32(float *y, const double *x, size_t n) {
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x)
    y[i] = (float)x[i];
}
__global__ void k_add_f32(double *y, const float *x, size_t n) {
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x)
    y[i] += (double)x[i];
}
// zero the Dirichlet DOFs of a row-ordered vector
__global__ void k_zero_bc(double *x, const int *bc_rows, const int *bc_masks, int nbc) {
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nbc * 6) return;
  int b = t / 6, k = t % 6;
  if (bc_masks[b] & (1 << k)) x[(size_t)bc_rows[b] * 6 + k] = 0.0;
}

// out[j] = sum_i X[j][i] * y[i] for j < m (X rows are vectors of length n);
// block partial sums then one atomic add per (block, j).
__global__ void __launch_bounds__(256) k_multidot(const double *X, size_t ldx, int m,
                                                  const double *y, size_t n, double *out) {
  __shared__ double red[8];
  for (int j = 0; j < m; j++) {
    double s = 0.0;
    const double *xj = X + (size_t)j * ldx;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (size_t)gridDim.x * blockDim.x)
      s += xj[i] * y[i];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x < 32) {
      double v = threadIdx.x < (blockDim.x >> 5) ? red[threadIdx.x] : 0.0;
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
      if (threadIdx.x == 0) atomicAdd(&out[j], v);
    }
    __syncthreads();
  }
}

// y -= sum_j c[j] X[j]  (c on the device)
__global__ void k_sub_combination(double *y, const double *X, size_t ldx, int m, const double *c,
                                  size_t n) {
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x) {
    double s = 0.0;
    for (int j = 0; j < m; j++) s += c[j] * X[(size_t)j * ldx + i];
    y[i] -= s;
  }
}

static int grid_for(size_t n) { return (int)std::min<size_t>((n + 255) / 256, 152 * 8); }

struct Blas {
  cudaStream_t s;
  DBuf<double> dwork;
  std::vector<double> hwork;
  long long *launches;
  int dots(const double *X, size_t ldx, int m, const double *y, size_t n, double *h) {
    int rc;
    if ((rc = dwork.alloc(std::max<size_t>(m, 1)))) return rc;
    A2DS_CUDA_TRY(cudaMemsetAsync(dwork.p, 0, m * sizeof(double), s));
    k_multidot<<<grid_for(n) / 2 + 1, 256, 0, s>>>(X, ldx, m, y, n, dwork.p);
    (*launches)++;
    A2DS_CUDA_TRY(cudaGetLastError());
    A2DS_CUDA_TRY(cudaMemcpyAsync(h, dwork.p, m * sizeof(double), cudaMemcpyDeviceToHost, s));
    A2DS_CUDA_TRY(cudaStreamSynchronize(s));
    return 0;
  }
  double dot(const double *x, const double *y, size_t n) {
    double h = 0.0;
    if (dots(x, n, 1, y, n, &h)) return NAN;
    return h;
  }
  int sub_combination(double *y, const double *X, size_t ldx, int m, const double *hc, size_t n) {
    int rc;
    if ((rc = dwork.alloc(std::max<size_t>(m, 1)))) return rc;
    A2DS_CUDA_TRY(cudaMemcpyAsync(dwork.p, hc, m * sizeof(double), cudaMemcpyHostToDevice, s));
    k_sub_combination<<<grid_for(n), 256, 0, s>>>(y, X, ldx, m, dwork.p, n);
    (*launches)++;
    A2DS_CUDA_TRY(cudaGetLastError());
    return 0;
  }
  void scale(double *x, double a, size_t n) {
    k_scale<<<grid_for(n), 256, 0, s>>>(x, a, n);
    (*launches)++;
  }
  void axpby(double *y, double a, const double *x, double b, size_t n) {
    k_axpby<<<grid_for(n), 256, 0, s>>>(y, a, x, b, n);
    (*launches)++;
  }
};

// ------------------------------------------------------------ factor
int factor_setup(Mesh &m, int lev_fill, int precision, Factor &f) {
  int rc;
  f.n = m.nn;
  f.lev_fill = lev_fill;
  f.precision = precision;
  if ((rc = ilu_symbolic(m.nn, m.rowp, m.cols, lev_fill, f.frowp, f.fcols, f.fdiag)))
    return fail(A2DS_ERR_STATE, "symbolic factorization failed");
  std::vector<int> lev;
  build_levels(m.nn, f.frowp, f.fcols, f.fdiag, false, f.flv, &lev);
  build_update_tasks(f, lev);
  build_solve_schedule(f, lev, 48);
  if ((rc = upload_schedules(f, m.stream))) return rc;
  if ((rc = f.d_frowp.upload(f.frowp.data(), f.frowp.size(), m.stream))) return rc;
  if ((rc = f.d_fcols.upload(f.fcols.data(), f.fcols.size(), m.stream))) return rc;
  if ((rc = f.d_fdiag.upload(f.fdiag.data(), f.fdiag.size(), m.stream))) return rc;
  if ((rc = f.d_status.alloc(1))) return rc;
  if (precision == 32) {
    if ((rc = f.F32.alloc((size_t)f.nnzb() * 36))) return rc;
  } else {
    if ((rc = f.F64.alloc((size_t)f.nnzb() * 36))) return rc;
  }
  A2DS_CUDA_TRY(cudaStreamSynchronize(m.stream));
  return 0;
}

// A second factor with the same symbolic pattern (no second symbolic
// factorization), values in the given precision.
static int factor_clone(Mesh &m, const Factor &src, int precision, Factor &f) {
  int rc;
  f.n = src.n;
  f.lev_fill = src.lev_fill;
  f.precision = precision;
  f.frowp = src.frowp;
  f.fcols = src.fcols;
  f.fdiag = src.fdiag;
  f.flv.nlevels = src.flv.nlevels;
  f.flv.ptr = src.flv.ptr;
  f.flv.rows = src.flv.rows;
  f.lower.nlevels = src.lower.nlevels;
  f.lower.ptr = src.lower.ptr;
  f.lower.rows = src.lower.rows;
  f.upper.nlevels = src.upper.nlevels;
  f.upper.ptr = src.upper.ptr;
  f.upper.rows = src.upper.rows;
  f.task_level_ptr = src.task_level_ptr;
  f.task_row = src.task_row;
  f.task_ptr = src.task_ptr;
  f.task_jp = src.task_jp;
  f.tail_s = src.tail_s;
  f.lsplit = src.lsplit;
  f.tl_ptr = src.tl_ptr;
  f.tl_row = src.tl_row;
  f.tl_pos = src.tl_pos;
  f.tl_col = src.tl_col;
  f.tu_ptr = src.tu_ptr;
  f.tu_row = src.tu_row;
  f.tu_pos = src.tu_pos;
  f.tu_col = src.tu_col;
  f.flop_count = src.flop_count;
  if ((rc = upload_schedules(f, m.stream))) return rc;
  if ((rc = f.d_frowp.upload(f.frowp.data(), f.frowp.size(), m.stream))) return rc;
  if ((rc = f.d_fcols.upload(f.fcols.data(), f.fcols.size(), m.stream))) return rc;
  if ((rc = f.d_fdiag.upload(f.fdiag.data(), f.fdiag.size(), m.stream))) return rc;
  if ((rc = f.d_status.alloc(1))) return rc;
  if (precision == 32) {
    if ((rc = f.F32.alloc((size_t)f.nnzb() * 36))) return rc;
  } else {
    if ((rc = f.F64.alloc((size_t)f.nnzb() * 36))) return rc;
  }
  A2DS_CUDA_TRY(cudaStreamSynchronize(m.stream));
  return 0;
}

int factor_numeric(Mesh &m, Factor &f, const double *A, const double *A2, double alpha2) {
  int rc;
  A2DS_CUDA_TRY(cudaMemsetAsync(f.d_status.p, 0, sizeof(int), m.stream));
  if (f.precision == 32) {
    if ((rc = factor_scatter<float>(m.nn, m.d_rowp.p, m.d_cols.p, A, A2, alpha2, f.d_frowp.p,
                                    f.d_fcols.p, f.F32.p, m.stream)))
      return rc;
    m.launches++;
    return factor_levels<float>(f, f.F32.p, f.d_status.p, m.stream, &m.launches);
  }
  if ((rc = factor_scatter<double>(m.nn, m.d_rowp.p, m.d_cols.p, A, A2, alpha2, f.d_frowp.p,
                                   f.d_fcols.p, f.F64.p, m.stream)))
    return rc;
  m.launches++;
  return factor_levels<double>(f, f.F64.p, f.d_status.p, m.stream, &m.launches);
}

int factor_check(Mesh &m, Factor &f) {
  int st = 0;
  A2DS_CUDA_TRY(cudaMemcpyAsync(&st, f.d_status.p, sizeof(int), cudaMemcpyDeviceToHost, m.stream));
  A2DS_CUDA_TRY(cudaStreamSynchronize(m.stream));
  if (st) return fail(A2DS_ERR_SINGULAR, "singular diagonal block in factor row " + std::to_string(st - 1));
  return 0;
}

// y = (LU)^{-1} x in FP64 (x, y row-ordered FP64; y may alias x).  For an
// FP32 factor the right-hand side is rounded to FP32 and the FP32 solution
// accumulated into y (y must not alias x then).
static int factor_apply(Mesh &m, Factor &f, const double *x, double *y, DBuf<float> &w32) {
  const size_t n6 = (size_t)m.nn * 6;
  if (f.precision == 32) {
    int rc;
    if ((rc = w32.alloc(n6))) return rc;
    k_f64_to_f32<<<grid_for(n6), 256, 0, m.stream>>>(w32.p, x, n6);
    m.launches++;
    if ((rc = solve_levels<float, float>(f, f.F32.p, w32.p, w32.p, 1, m.stream, &m.launches)))
      return rc;
    A2DS_CUDA_TRY(cudaMemsetAsync(y, 0, n6 * sizeof(double), m.stream));
    k_add_f32<<<grid_for(n6), 256, 0, m.stream>>>(y, w32.p, n6);
    m.launches++;
    return 0;
  }
  return solve_levels<double, double>(f, f.F64.p, x, y, 1, m.stream, &m.launches);
}

// ------------------------------------------------- small dense eigensolver
// Cyclic Jacobi for a symmetric m x m matrix (row-major, destroyed);
// eigenvalues in w, eigenvectors as columns of V.
static void jacobi_eig(int m, std::vector<double> &A, std::vector<double> &w,
                       std::vector<double> &V) {
  V.assign((size_t)m * m, 0.0);
  for (int i = 0; i < m; i++) V[(size_t)i * m + i] = 1.0;
  for (int sweep = 0; sweep < 100; sweep++) {
    double off = 0.0, tot = 0.0;
    for (int i = 0; i < m; i++)
      for (int j = 0; j < m; j++) {
        double v = A[(size_t)i * m + j] * A[(size_t)i * m + j];
        tot += v;
        if (i != j) off += v;
      }
    if (off <= 1e-30 * tot || off == 0.0) break;
    for (int p = 0; p < m - 1; p++)
      for (int q = p + 1; q < m; q++) {
        double apq = A[(size_t)p * m + q];
        if (apq == 0.0) continue;
        double app = A[(size_t)p * m + p], aqq = A[(size_t)q * m + q];
        double theta = (aqq - app) / (2.0 * apq);
        double t = (theta >= 0 ? 1.0 : -1.0) / (fabs(theta) + sqrt(theta * theta + 1.0));
        double c = 1.0 / sqrt(t * t + 1.0), s = t * c;
        for (int k = 0; k < m; k++) {
          double akp = A[(size_t)k * m + p], akq = A[(size_t)k * m + q];
          A[(size_t)k * m + p] = c * akp - s * akq;
          A[(size_t)k * m + q] = s * akp + c * akq;
        }
        for (int k = 0; k < m; k++) {
          double apk = A[(size_t)p * m + k], aqk = A[(size_t)q * m + k];
          A[(size_t)p * m + k] = c * apk - s * aqk;
          A[(size_t)q * m + k] = s * apk + c * aqk;
        }
        for (int k = 0; k < m; k++) {
          double vkp = V[(size_t)k * m + p], vkq = V[(size_t)k * m + q];
          V[(size_t)k * m + p] = c * vkp - s * vkq;
          V[(size_t)k * m + q] = s * vkp + c * vkq;
        }
      }
  }
  w.resize(m);
  for (int i = 0; i < m; i++) w[i] = A[(size_t)i * m + i];
}

// --------------------------------------------------------- buckling state
struct BucklingState {
  Factor fk, fa;
  DBuf<double> K, G, Aux;
  DBuf<double> Q, KQ;  // (m+1) x n6 Lanczos basis and K times it
  DBuf<double> w, r, t, path, rhs;
  DBuf<float> w32;
  std::vector<double> lam, err, phi_ritz;  // converged data
  int niters = 0, nconv = 0;
  double sigma = 0.0;
  int lev_fill = -1, precision = 0;
  cudaEvent_t ev[6] = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
  BucklingState() {
    for (auto &e : ev) cudaEventCreate(&e);
  }
  ~BucklingState() {
    for (auto &e : ev)
      if (e) cudaEventDestroy(e);
  }
};

void release_solver(Mesh &m) {
  delete (BucklingState *)m.solver;
  m.solver = nullptr;
}

static double now() {
  return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

// Solve A x = b (row ordering) with the factor and FP64 iterative
// refinement (residual with A = Avals (+ alpha2 A2vals) in FP64).
static int refined_solve(Mesh &m, Factor &f, const double *Avals, const double *A2vals,
                         double alpha2, const double *b, double *x, BucklingState &S, Blas &B,
                         double rtol, int max_steps, int *steps) {
  const size_t n6 = (size_t)m.nn * 6;
  int rc;
  if ((rc = factor_apply(m, f, b, x, S.w32))) return rc;
  double bn = sqrt(B.dot(b, b, n6));
  if (bn == 0.0) return 0;
  for (int it = 0; it < max_steps; it++) {
    // r = b - A x
    if ((rc = launch_spmv_f64(m.nn, m.d_rowp.p, m.d_cols.p, Avals, x, S.r.p, m.stream))) return rc;
    m.launches++;
    if (A2vals) {
      if ((rc = launch_spmv_f64(m.nn, m.d_rowp.p, m.d_cols.p, A2vals, x, S.t.p, m.stream)))
        return rc;
      m.launches++;
      B.axpby(S.r.p, alpha2, S.t.p, 1.0, n6);
    }
    B.axpby(S.r.p, 1.0, b, -1.0, n6);  // r = b - r
    double rn = sqrt(B.dot(S.r.p, S.r.p, n6));
    if (steps) (*steps)++;
    if (rn <= rtol * bn) return 0;
    if ((rc = factor_apply(m, f, S.r.p, S.t.p, S.w32))) return rc;
    B.axpby(x, 1.0, S.t.p, 1.0, n6);
  }
  return 0;
}

}  // namespace a2ds

using namespace a2ds;

extern "C" {

int a2ds_pc_create(a2ds_bcsr A, int lev_fill, int precision, a2ds_pc *out) {
  if (!A || !out) return fail(A2DS_ERR_ARG, "null argument");
  if (precision != 64 && precision != 32) return fail(A2DS_ERR_ARG, "precision must be 64 or 32");
  if (lev_fill < 0) return fail(A2DS_ERR_ARG, "lev_fill must be >= 0");
  a2ds_pc pc = new a2ds_pc_s();
  pc->mat = A;
  int rc = factor_setup(A->mesh->m, lev_fill, precision, pc->f);
  if (rc) {
    delete pc;
    return rc;
  }
  *out = pc;
  return 0;
}

int a2ds_pc_destroy(a2ds_pc pc) {
  delete pc;
  return 0;
}

int a2ds_pc_factor(a2ds_pc pc, a2ds_bcsr from) {
  if (!pc) return fail(A2DS_ERR_ARG, "null preconditioner");
  a2ds_bcsr A = from ? from : pc->mat;
  if (A->mesh != pc->mat->mesh) return fail(A2DS_ERR_ARG, "matrix belongs to another mesh");
  Mesh &m = A->mesh->m;
  int rc = factor_numeric(m, pc->f, A->vals.p, nullptr, 0.0);
  if (rc) return rc;
  return factor_check(m, pc->f);
}

int a2ds_pc_apply(a2ds_pc pc, const double *x, double *y) {
  if (!pc || !x || !y) return fail(A2DS_ERR_ARG, "null argument");
  Mesh &m = pc->mat->mesh->m;
  DBuf<double> dx, dy;
  DBuf<float> w32;
  int rc;
  if ((rc = m.to_rows(x, dx))) return rc;
  if ((rc = dy.alloc((size_t)m.nn * 6))) return rc;
  if ((rc = factor_apply(m, pc->f, dx.p, dy.p, w32))) return rc;
  return m.from_rows(dy.p, y);
}

int a2ds_pc_get(a2ds_pc pc, int *nrows, int *nnzb, int *rowp, int *cols, double *vals) {
  if (!pc) return fail(A2DS_ERR_ARG, "null preconditioner");
  Factor &f = pc->f;
  Mesh &m = pc->mat->mesh->m;
  if (nrows) *nrows = f.n;
  if (nnzb) *nnzb = (int)f.nnzb();
  if (rowp) std::copy(f.frowp.begin(), f.frowp.end(), rowp);
  if (cols) std::copy(f.fcols.begin(), f.fcols.end(), cols);
  if (vals) {
    const size_t nv = (size_t)f.nnzb() * 36;
    if (f.precision == 32) {
      std::vector<float> tmp(nv);
      A2DS_CUDA_TRY(cudaMemcpyAsync(tmp.data(), f.F32.p, nv * sizeof(float), cudaMemcpyDeviceToHost,
                                    m.stream));
      A2DS_CUDA_TRY(cudaStreamSynchronize(m.stream));
      for (size_t i = 0; i < nv; i++) vals[i] = tmp[i];
    } else {
      A2DS_CUDA_TRY(cudaMemcpyAsync(vals, f.F64.p, nv * sizeof(double), cudaMemcpyDeviceToHost,
                                    m.stream));
      A2DS_CUDA_TRY(cudaStreamSynchronize(m.stream));
    }
  }
  return 0;
}

void a2ds_buckling_default_opts(a2ds_buckling_opts *o) {
  if (!o) return;
  o->sigma = 0.0;
  o->max_lanczos = 100;
  o->num_eigvals = 10;
  o->eig_tol = 1e-10;
  o->lev_fill = 1000000;
  o->gmres_m = 30;
  o->gmres_restarts = 15;
  o->gmres_rtol = 1e-12;
  o->gmres_atol = 1e-30;
  o->precision = 64;
  o->seed = 0;
}

int a2ds_buckling_solve(a2ds_mesh mesh, const a2ds_buckling_opts *opts, const double *rhs,
                        double *eigvals, double *errors, double *eigvecs, double *path_out) {
  if (!mesh || !opts || !eigvals) return fail(A2DS_ERR_ARG, "null argument");
  Mesh &m = mesh->m;
  if (!m.initialized) return fail(A2DS_ERR_STATE, "mesh not initialized");
  const int nev = opts->num_eigvals, mmax = opts->max_lanczos;
  if (nev <= 0 || mmax < nev) return fail(A2DS_ERR_ARG, "need 0 < num_eigvals <= max_lanczos");
  if (!(opts->sigma > 0.0)) return fail(A2DS_ERR_ARG, "sigma must be positive");
  if (opts->precision != 64 && opts->precision != 32)
    return fail(A2DS_ERR_ARG, "precision must be 64 or 32");
  const size_t n6 = (size_t)m.nn * 6;
  const size_t nv = (size_t)m.nnzb * 36;
  int rc;
  double t0 = now();
  long long launches0 = m.launches;

  BucklingState *Sp = (BucklingState *)m.solver;
  if (!Sp || Sp->lev_fill != opts->lev_fill || Sp->precision != opts->precision) {
    delete Sp;
    Sp = new BucklingState();
    m.solver = Sp;
    Sp->lev_fill = opts->lev_fill;
    Sp->precision = opts->precision;
    if ((rc = factor_setup(m, opts->lev_fill, 64, Sp->fk))) return rc;
    if ((rc = factor_clone(m, Sp->fk, opts->precision, Sp->fa))) return rc;
  }
  BucklingState &S = *Sp;
  S.sigma = opts->sigma;
  if ((rc = S.K.alloc(nv)) || (rc = S.G.alloc(nv)) || (rc = S.Aux.alloc(nv))) return rc;
  if ((rc = S.Q.alloc((size_t)(mmax + 1) * n6)) || (rc = S.KQ.alloc((size_t)(mmax + 1) * n6)))
    return rc;
  if ((rc = S.w.alloc(n6)) || (rc = S.r.alloc(n6)) || (rc = S.t.alloc(n6)) ||
      (rc = S.path.alloc(n6)) || (rc = S.rhs.alloc(n6)))
    return rc;
  Blas B{m.stream};
  B.launches = &m.launches;

  // 1. K at the zero state
  A2DS_CUDA_TRY(cudaEventRecord(S.ev[0], m.stream));
  double ta = now();
  if ((rc = m.assemble_device(MODE_K, nullptr, S.K.p, nullptr, A2DS_SCATTER_ATOMIC))) return rc;
  A2DS_CUDA_TRY(cudaStreamSynchronize(m.stream));
  double t_k = now() - ta;

  // 2. load path: res = R(0) - f (BC rows: 0 - bcval), path = -K^{-1} res
  ta = now();
  A2DS_CUDA_TRY(cudaEventRecord(S.ev[4], m.stream));
  if ((rc = factor_numeric(m, S.fk, S.K.p, nullptr, 0.0))) return rc;
  A2DS_CUDA_TRY(cudaEventRecord(S.ev[5], m.stream));
  if ((rc = factor_check(m, S.fk))) return rc;
  double t_fk = now() - ta;
  ta = now();
  if ((rc = m.assemble_device(MODE_R, nullptr, nullptr, S.r.p, A2DS_SCATTER_ATOMIC))) return rc;
  {
    std::vector<double> h((size_t)m.nn * 6, 0.0), hr(n6);
    if (rhs) {
      for (int i = 0; i < m.nn; i++)
        for (int k = 0; k < 6; k++) h[(size_t)i * 6 + k] = rhs[(size_t)m.perm[i] * 6 + k];
    }
    for (size_t b = 0; b < m.bc_rows.size(); b++)
      for (int k = 0; k < 6; k++)
        if (m.bc_masks[b] & (1 << k)) h[(size_t)m.bc_rows[b] * 6 + k] = m.bc_vals[b * 6 + k];
    // rhs' = f with BC rows replaced by the BC values; res = R(0) - rhs'
    A2DS_CUDA_TRY(cudaMemcpyAsync(S.rhs.p, h.data(), n6 * sizeof(double), cudaMemcpyHostToDevice,
                                  m.stream));
    k_zero_bc<<<((int)m.bc_rows.size() * 6 + 255) / 256 + 1, 256, 0, m.stream>>>(
        S.r.p, m.d_bc_rows.p, m.d_bc_masks.p, (int)m.bc_rows.size());
    m.launches++;
    B.axpby(S.rhs.p, -1.0, S.r.p, 1.0, n6);  // rhs = rhs - R(0): K path = rhs
  }
  int inner = 0;
  if ((rc = refined_solve(m, S.fk, S.K.p, nullptr, 0.0, S.rhs.p, S.path.p, S, B, 1e-13, 4, &inner)))
    return rc;
  A2DS_CUDA_TRY(cudaStreamSynchronize(m.stream));
  double t_path = now() - ta;

  // 3. G along the path; A = K + sigma G with identity BC rows
  ta = now();
  if ((rc = m.assemble_device(MODE_G, S.path.p, S.G.p, nullptr, A2DS_SCATTER_ATOMIC))) return rc;
  A2DS_CUDA_TRY(cudaStreamSynchronize(m.stream));
  double t_g = now() - ta;
  ta = now();
  A2DS_CUDA_TRY(cudaMemcpyAsync(S.Aux.p, S.K.p, nv * sizeof(double), cudaMemcpyDeviceToDevice,
                                m.stream));
  if ((rc = launch_axpy(S.Aux.p, S.sigma, S.G.p, nv, m.stream))) return rc;
  if ((rc = launch_apply_bc_rows(S.Aux.p, m.d_rowp.p, m.d_cols.p, m.d_bc_rows.p, m.d_bc_masks.p,
                                 (int)m.bc_rows.size(), m.stream)))
    return rc;
  m.launches += 2;
  A2DS_CUDA_TRY(cudaEventRecord(S.ev[2], m.stream));
  if ((rc = factor_numeric(m, S.fa, S.Aux.p, nullptr, 0.0))) return rc;
  A2DS_CUDA_TRY(cudaEventRecord(S.ev[3], m.stream));
  if ((rc = factor_check(m, S.fa))) return rc;
  double t_fa = now() - ta;

  // 4. Lanczos on A^{-1} K with the K inner product
  ta = now();
  const int nbc = (int)m.bc_rows.size();
  auto zero_bc = [&](double *x) {
    if (nbc) {
      k_zero_bc<<<(nbc * 6 + 255) / 256, 256, 0, m.stream>>>(x, m.d_bc_rows.p, m.d_bc_masks.p, nbc);
      m.launches++;
    }
  };
  {
    // seeded start vector (splitmix64), BC DOFs zeroed, K-normalised
    std::vector<double> h(n6);
    uint64_t st = 0x9E3779B97F4A7C15ull * (uint64_t)(opts->seed + 1);
    for (size_t i = 0; i < n6; i++) {
      uint64_t z = (st += 0x9E3779B97F4A7C15ull);
      z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
      z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
      z ^= z >> 31;
      h[i] = (double)(z >> 11) * (1.0 / 9007199254740992.0) * 2.0 - 1.0;
    }
    A2DS_CUDA_TRY(cudaMemcpyAsync(S.Q.p, h.data(), n6 * sizeof(double), cudaMemcpyHostToDevice,
                                  m.stream));
  }
  zero_bc(S.Q.p);
  if ((rc = launch_spmv_f64(m.nn, m.d_rowp.p, m.d_cols.p, S.K.p, S.Q.p, S.KQ.p, m.stream))) return rc;
  m.launches++;
  {
    double nrm = sqrt(B.dot(S.Q.p, S.KQ.p, n6));
    B.scale(S.Q.p, 1.0 / nrm, n6);
    B.scale(S.KQ.p, 1.0 / nrm, n6);
  }
  std::vector<double> alpha, beta, h((size_t)mmax + 1), h2((size_t)mmax + 1);
  std::vector<double> ritz_mu, ritz_vec;  // of the converged set
  std::vector<int> order;
  int m_iter = 0, converged = 0;
  double last_beta = 0.0;
  std::vector<double> Tw, TV;
  for (int i = 0; i < mmax; i++) {
    double *qi = S.Q.p + (size_t)i * n6, *kqi = S.KQ.p + (size_t)i * n6;
    double *w = S.Q.p + (size_t)(i + 1) * n6, *kw = S.KQ.p + (size_t)(i + 1) * n6;
    // w = A^{-1} K q_i
    if ((rc = refined_solve(m, S.fa, S.Aux.p, nullptr, 0.0, kqi, w, S, B, 1e-10, 2, &inner)))
      return rc;
    zero_bc(w);
    // full K-orthogonalisation, two classical Gram-Schmidt passes using K q_j
    if ((rc = B.dots(S.KQ.p, n6, i + 1, w, n6, h.data()))) return rc;
    if ((rc = B.sub_combination(w, S.Q.p, n6, i + 1, h.data(), n6))) return rc;
    if ((rc = B.dots(S.KQ.p, n6, i + 1, w, n6, h2.data()))) return rc;
    if ((rc = B.sub_combination(w, S.Q.p, n6, i + 1, h2.data(), n6))) return rc;
    alpha.push_back(h[i] + h2[i]);
    if ((rc = launch_spmv_f64(m.nn, m.d_rowp.p, m.d_cols.p, S.K.p, w, kw, m.stream))) return rc;
    m.launches++;
    double b2 = B.dot(w, kw, n6);
    double b = sqrt(std::max(b2, 0.0));
    if (!(b > 0.0) || !std::isfinite(b)) return fail(A2DS_ERR_BREAKDOWN, "Lanczos breakdown");
    beta.push_back(b);
    B.scale(w, 1.0 / b, n6);
    B.scale(kw, 1.0 / b, n6);
    m_iter = i + 1;
    last_beta = b;
    if (m_iter < nev) continue;
    // Ritz values of the tridiagonal T (m_iter x m_iter)
    std::vector<double> T((size_t)m_iter * m_iter, 0.0);
    for (int k = 0; k < m_iter; k++) {
      T[(size_t)k * m_iter + k] = alpha[k];
      if (k + 1 < m_iter) T[(size_t)k * m_iter + k + 1] = T[(size_t)(k + 1) * m_iter + k] = beta[k];
    }
    jacobi_eig(m_iter, T, Tw, TV);
    // lambda = -mu sigma / (1 - mu); sort by |lambda|
    order.resize(m_iter);
    for (int k = 0; k < m_iter; k++) order[k] = k;
    auto lamof = [&](double mu) { return -mu * S.sigma / (1.0 - mu); };
    std::sort(order.begin(), order.end(),
              [&](int a, int c) { return fabs(lamof(Tw[a])) < fabs(lamof(Tw[c])); });
    converged = 1;
    for (int k = 0; k < nev; k++) {
      int idx = order[k];
      double est = fabs(b * TV[(size_t)(m_iter - 1) * m_iter + idx]);
      if (!(est <= opts->eig_tol * fabs(Tw[idx]))) {
        converged = 0;
        break;
      }
    }
    if (converged) break;
  }
  A2DS_CUDA_TRY(cudaStreamSynchronize(m.stream));
  double t_lan = now() - ta;
  (void)last_beta;
  if (!converged) {
    // fill what we have, report non-convergence
  }
  // eigenvalues, eigenvectors phi = Q y, residual check ||K phi + lam G phi|| / ||K phi||
  S.lam.assign(nev, 0.0);
  S.err.assign(nev, 0.0);
  S.phi_ritz.assign((size_t)nev * m_iter, 0.0);
  for (int k = 0; k < nev && k < m_iter; k++) {
    int idx = order[k];
    double mu = Tw[idx];
    double lam = -mu * S.sigma / (1.0 - mu);
    S.lam[k] = lam;
    std::vector<double> y(m_iter);
    for (int j = 0; j < m_iter; j++) y[j] = TV[(size_t)j * m_iter + idx];
    for (int j = 0; j < m_iter; j++) S.phi_ritz[(size_t)k * m_iter + j] = y[j];
    // phi = sum_j y_j q_j  (w <- 0; w -= sum (-y_j) q_j)
    A2DS_CUDA_TRY(cudaMemsetAsync(S.w.p, 0, n6 * sizeof(double), m.stream));
    for (int j = 0; j < m_iter; j++) y[j] = -y[j];
    if ((rc = B.sub_combination(S.w.p, S.Q.p, n6, m_iter, y.data(), n6))) return rc;
    if ((rc = launch_spmv_f64(m.nn, m.d_rowp.p, m.d_cols.p, S.K.p, S.w.p, S.r.p, m.stream))) return rc;
    if ((rc = launch_spmv_f64(m.nn, m.d_rowp.p, m.d_cols.p, S.G.p, S.w.p, S.t.p, m.stream))) return rc;
    m.launches += 2;
    zero_bc(S.r.p);
    zero_bc(S.t.p);
    double kn = sqrt(B.dot(S.r.p, S.r.p, n6));
    B.axpby(S.r.p, lam, S.t.p, 1.0, n6);
    double rn = sqrt(B.dot(S.r.p, S.r.p, n6));
    S.err[k] = kn > 0 ? rn / kn : rn;
    if (eigvecs) {
      if ((rc = m.from_rows(S.w.p, eigvecs + (size_t)k * n6))) return rc;
    }
  }
  for (int k = 0; k < nev; k++) {
    eigvals[k] = S.lam[k];
    if (errors) errors[k] = S.err[k];
  }
  if (path_out && (rc = m.from_rows(S.path.p, path_out))) return rc;
  S.niters = m_iter;
  A2DS_CUDA_TRY(cudaEventRecord(S.ev[1], m.stream));
  A2DS_CUDA_TRY(cudaStreamSynchronize(m.stream));
  double total = now() - t0;
  float ms_solve = 0.f, ms_fa = 0.f, ms_fk = 0.f;
  cudaEventElapsedTime(&ms_solve, S.ev[0], S.ev[1]);
  cudaEventElapsedTime(&ms_fa, S.ev[2], S.ev[3]);
  cudaEventElapsedTime(&ms_fk, S.ev[4], S.ev[5]);
  m.stats = {total, t_k, t_g, t_fk + t_fa, t_path, t_lan, (double)m_iter, (double)inner,
             (double)(m.launches - launches0), (double)ms_solve, (double)ms_fa, (double)ms_fk,
             (double)S.fa.nnzb(), (double)S.fa.flv.nlevels, (double)S.fa.flops()};
  if (!converged) return fail(A2DS_ERR_NOCONV, "Lanczos did not converge within max_lanczos (results returned are the current Ritz pairs)");
  return 0;
}

int a2ds_buckling_stats(a2ds_mesh mesh, int n, double *out) {
  if (!mesh || !out) return fail(A2DS_ERR_ARG, "null argument");
  Mesh &m = mesh->m;
  for (int i = 0; i < n && i < (int)m.stats.size(); i++) out[i] = m.stats[i];
  return 0;
}

int a2ds_eig_sens_thickness(a2ds_mesh, int, double *) {
  return fail(A2DS_ERR_STATE, "eigenvalue sensitivities are not available yet");
}

}  // extern "C"
