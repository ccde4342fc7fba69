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

void build_levels(int n, const std::vector<int> &frowp, const std::vector<int> &fcols,
                  const std::vector<int> &fdiag, bool upper, LevelSchedule &L);

// F <- pattern-embedded copy of A (+ alpha2 * A2 when A2 != NULL), as T.
template <typename T>
int factor_scatter(int n, const int *rowp, const int *cols, const double *A, const double *A2,
                   double alpha2, const int *frowp, const int *fcols, T *F, cudaStream_t s);

// In-place numeric factorization of F (levels of the L pattern).  *status
// receives max(row+1) of any singular diagonal block (0 = none).
template <typename T>
int factor_levels(const LevelSchedule &L, const int *frowp, const int *fcols, const int *fdiag,
                  T *F, int *status, cudaStream_t s, long long *launches);

// y = (LU)^{-1} x for nrhs right-hand sides, layout (row, dof, rhs); y may
// alias x.
template <typename T, typename TV>
int solve_levels(const LevelSchedule &Lo, const LevelSchedule &Up, const int *frowp,
                 const int *fcols, const int *fdiag, const T *F, const TV *x, TV *y, int nrhs,
                 cudaStream_t s, long long *launches);

// A factorization handle (the TACSSchurPc role on one GPU).
struct Factor {
  int n = 0, lev_fill = 0, precision = 64;
  std::vector<int> frowp, fcols, fdiag;
  DBuf<int> d_frowp, d_fcols, d_fdiag, d_status;
  DBuf<double> F64;
  DBuf<float> F32;
  LevelSchedule lower, upper;
  long long nnzb() const { return frowp.empty() ? 0 : frowp.back(); }
};

struct Mesh;
int factor_setup(Mesh &m, int lev_fill, int precision, Factor &f);
// Factor A (+ alpha2 * A2) -- both in the mesh pattern -- into f.
int factor_numeric(Mesh &m, Factor &f, const double *A, const double *A2, double alpha2);
int factor_check(Mesh &m, Factor &f);  // reads the singular-pivot status

}  // namespace a2ds
