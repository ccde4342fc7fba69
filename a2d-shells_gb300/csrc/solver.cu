// Buckling solve, ILU(k) factorization and eigenvalue sensitivities.
#include "a2ds_internal.h"
#include "runtime.h"

namespace a2ds {
void release_solver(Mesh &m) { (void)m; }
}  // namespace a2ds

using namespace a2ds;

extern "C" {
int a2ds_pc_create(a2ds_bcsr, int, int, a2ds_pc *) { return fail(A2DS_ERR_STATE, "not available yet"); }
int a2ds_pc_destroy(a2ds_pc) { return 0; }
int a2ds_pc_factor(a2ds_pc, a2ds_bcsr) { return fail(A2DS_ERR_STATE, "not available yet"); }
int a2ds_pc_apply(a2ds_pc, const double *, double *) { return fail(A2DS_ERR_STATE, "not available yet"); }
int a2ds_pc_get(a2ds_pc, int *, int *, int *, int *, double *) { return fail(A2DS_ERR_STATE, "not available yet"); }
void a2ds_buckling_default_opts(a2ds_buckling_opts *o) {
  o->sigma = 0.0; o->max_lanczos = 100; o->num_eigvals = 10; o->eig_tol = 1e-10;
  o->lev_fill = 1000000; o->gmres_m = 30; o->gmres_restarts = 15; o->gmres_rtol = 1e-12;
  o->gmres_atol = 1e-30; o->precision = 64; o->seed = 0;
}
int a2ds_buckling_solve(a2ds_mesh, const a2ds_buckling_opts *, const double *, double *, double *, double *, double *) { return fail(A2DS_ERR_STATE, "not available yet"); }
int a2ds_buckling_stats(a2ds_mesh, int, double *) { return fail(A2DS_ERR_STATE, "not available yet"); }
int a2ds_eig_sens_thickness(a2ds_mesh, int, double *) { return fail(A2DS_ERR_STATE, "not available yet"); }
}
