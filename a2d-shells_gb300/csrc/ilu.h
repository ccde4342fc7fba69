// Block ILU(k) factorization and level-scheduled triangular solves.
#pragma once
#include <vector>

#include "a2ds_internal.h"

namespace a2ds {

// Rows grouped by dependency level (host copy + device copy of the rows).
struct LevelSchedule {
  int nlevels = 0;
  std::vector<int> ptr;   // nlevels + 1
  std::vector<int> rows;  // rows ordered by level
  DBuf<int> d_rows;
};

// An instantiated CUDA graph of one whole triangular solve, keyed by the
// factor values and the vectors it was captured with.
struct SolveGraph {
  const void *F, *x;
  void *y;
  int nrhs, tv_size;
  cudaGraphExec_t exec;
  long long nlaunch;  // kernels in the graph
};

// A factorization handle (the TACSSchurPc role on one GPU).
struct Factor {
  int n = 0, lev_fill = 0, precision = 64;
  std::vector<int> frowp, fcols, fdiag;
  DBuf<int> d_frowp, d_fcols, d_fdiag, d_status;
  DBuf<double> F64;
  DBuf<float> F32;
  LevelSchedule flv;           // dependency levels of all rows (factorization)
  LevelSchedule lower, upper;  // head rows [0, tail_s): row-oriented solves
  // right-looking update tasks, grouped by level
  std::vector<int> task_level_ptr, task_row, task_ptr, task_jp;
  DBuf<int> d_task_row, d_task_ptr, d_task_jp;
  // dense tail rows [tail_s, n): head pull split and column push lists
  int tail_s = 0;
  std::vector<int> lsplit, tl_ptr, tl_row, tl_pos, tl_col, tu_ptr, tu_row, tu_pos, tu_col;
  DBuf<int> d_lsplit, d_tl_row, d_tl_pos, d_tl_col, d_tu_row, d_tu_pos, d_tu_col;
  // algorithmic FP operations of one numeric factorization: 432 per L block
  // (L_ij = A_ij D_j^{-1}), 432 per block update, 432 per diagonal inverse
  double flop_count = 0.0;
  std::vector<SolveGraph> graphs;  // solve_graph cache (at most 8)
  Factor() = default;
  ~Factor();
  long long nnzb() const { return frowp.empty() ? 0 : frowp.back(); }
  double flops() const { return flop_count; }
};

void build_levels(int n, const std::vector<int> &frowp, const std::vector<int> &fcols,
                  const std::vector<int> &fdiag, bool upper, LevelSchedule &L,
                  std::vector<int> *level_of = nullptr);
void build_update_tasks(Factor &f, const std::vector<int> &lev);
// Split rows into the head (row-oriented level solves) and the dense tail
// (column-oriented pushes) and build both schedules; lev = factor levels.
void build_solve_schedule(Factor &f, const std::vector<int> &lev, int narrow);
int upload_schedules(Factor &f, cudaStream_t s);

// F <- pattern-embedded copy of A (+ alpha2 * A2 when A2 != NULL), as T.
template <typename T>
int factor_scatter(int n, const int *rowp, const int *cols, const double *A, const double *A2,
                   double alpha2, const int *frowp, const int *fcols, T *F, cudaStream_t s);

// In-place numeric factorization of F.  *status receives max(row+1) of any
// singular diagonal block (0 = none).
template <typename T>
int factor_levels(const Factor &f, T *F, int *status, cudaStream_t s, long long *launches);

// y = (LU)^{-1} x for nrhs in {1, 2, 4, 8, 16} right-hand sides, layout
// (row, dof, rhs); y may alias x.  solve_levels launches the level kernels
// on s; solve_graph does the same through a CUDA graph captured on the
// first call with these (F, x, y, nrhs) and replayed afterwards (s must not
// be capturing already).
template <typename T, typename TV>
int solve_levels(const Factor &f, const T *F, const TV *x, TV *y, int nrhs, cudaStream_t s,
                 long long *launches);
template <typename T, typename TV>
int solve_graph(Factor &f, const T *F, const TV *x, TV *y, int nrhs, cudaStream_t s,
                long long *launches);

struct Mesh;
int factor_setup(Mesh &m, int lev_fill, int precision, Factor &f);
// Factor A (+ alpha2 * A2) -- both in the mesh pattern -- into f.
int factor_numeric(Mesh &m, Factor &f, const double *A, const double *A2, double alpha2);
int factor_check(Mesh &m, Factor &f);  // reads the singular-pivot status

}  // namespace a2ds
