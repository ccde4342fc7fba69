// The extern "C" entry points declared in include/a2ds.h.
#include <string.h>

#include <algorithm>
#include <new>
#include <string>
#include <vector>

#include "a2ds.h"
#include "a2ds_internal.h"
#include "block.h"
#include "host_graph.h"
#include "kernels.h"
#include "runtime.h"

using namespace a2ds;

#define A2DS_GUARD_BEGIN try {
#define A2DS_GUARD_END                                                      \
  }                                                                         \
  catch (const std::bad_alloc &) {                                          \
    return fail(A2DS_ERR_NOMEM, "host allocation failed");                  \
  }                                                                         \
  catch (...) {                                                             \
    return fail(A2DS_ERR_STATE, "unexpected host exception");               \
  }

namespace a2ds {
Mesh::~Mesh() {
  if (stream) cudaStreamDestroy(stream);
}
}  // namespace a2ds

static int check_mesh(a2ds_mesh m, bool need_init) {
  if (!m) return fail(A2DS_ERR_ARG, "null mesh handle");
  if (need_init && !m->m.initialized)
    return fail(A2DS_ERR_STATE, "mesh not initialized (call a2ds_mesh_initialize)");
  return 0;
}

extern "C" {

const char *a2ds_last_error(void) { return last_error_cstr(); }

int a2ds_device_count(void) {
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess) return 0;
  return n;
}

int a2ds_mesh_create(int num_nodes, int num_elements, int nodes_per_elem, const int *conn,
                     const double *X, int nonlinear, a2ds_mesh *out) {
  A2DS_GUARD_BEGIN
  if (!out) return fail(A2DS_ERR_ARG, "out is null");
  *out = nullptr;
  if (num_nodes <= 0 || num_elements <= 0)
    return fail(A2DS_ERR_ARG, "num_nodes and num_elements must be positive");
  if (nodes_per_elem != 4 && nodes_per_elem != 9)
    return fail(A2DS_ERR_ARG, "nodes_per_elem must be 4 (Quad4) or 9 (Quad9)");
  if (!conn || !X) return fail(A2DS_ERR_ARG, "conn and X are required");
  for (size_t k = 0; k < (size_t)num_elements * nodes_per_elem; k++)
    if (conn[k] < 0 || conn[k] >= num_nodes)
      return fail(A2DS_ERR_ARG, "connectivity entry " + std::to_string(k) + " out of range");
  a2ds_mesh h = new a2ds_mesh_s();
  Mesh &m = h->m;
  m.nn = num_nodes;
  m.ne = num_elements;
  m.npe = nodes_per_elem;
  m.order = nodes_per_elem == 4 ? 2 : 3;
  m.nonlinear = nonlinear ? 1 : 0;
  m.conn.assign(conn, conn + (size_t)num_elements * nodes_per_elem);
  m.X.assign(X, X + (size_t)num_nodes * 3);
  m.tgroup.assign(num_elements, 0);
  *out = h;
  return 0;
  A2DS_GUARD_END
}

int a2ds_mesh_destroy(a2ds_mesh mesh) {
  if (!mesh) return 0;
  if (mesh->m.stream) cudaStreamSynchronize(mesh->m.stream);
  release_solver(mesh->m);
  delete mesh;
  return 0;
}

int a2ds_mesh_set_material(a2ds_mesh mesh, double E, double nu, double alpha, double temperature) {
  int rc = check_mesh(mesh, false);
  if (rc) return rc;
  if (!(E > 0.0) || !(nu > -1.0 && nu < 0.5)) return fail(A2DS_ERR_ARG, "invalid E or nu");
  mesh->m.E = E;
  mesh->m.nu = nu;
  mesh->m.alpha = alpha;
  mesh->m.temperature = temperature;
  return 0;
}

int a2ds_mesh_set_yield_stress(a2ds_mesh mesh, double ys) {
  int rc = check_mesh(mesh, false);
  if (rc) return rc;
  if (!(ys > 0.0)) return fail(A2DS_ERR_ARG, "yield stress must be positive");
  mesh->m.ys = ys;
  return 0;
}

int a2ds_mesh_set_thickness(a2ds_mesh mesh, int num_groups, const double *t, const int *elem_group) {
  A2DS_GUARD_BEGIN
  int rc = check_mesh(mesh, false);
  if (rc) return rc;
  Mesh &m = mesh->m;
  if (num_groups <= 0 || !t) return fail(A2DS_ERR_ARG, "need at least one thickness value");
  for (int g = 0; g < num_groups; g++)
    if (!(t[g] > 0.0)) return fail(A2DS_ERR_ARG, "thickness must be positive");
  std::vector<int> grp(m.ne, 0);
  if (elem_group) {
    for (int e = 0; e < m.ne; e++) {
      if (elem_group[e] < 0 || elem_group[e] >= num_groups)
        return fail(A2DS_ERR_ARG, "element group out of range");
      grp[e] = elem_group[e];
    }
  }
  m.tvals.assign(t, t + num_groups);
  m.tgroup = grp;
  if (m.initialized) {
    if ((rc = m.d_tvals.upload(m.tvals.data(), m.tvals.size(), m.stream))) return rc;
    if ((rc = m.d_tgroup.upload(m.tgroup.data(), m.tgroup.size(), m.stream))) return rc;
    A2DS_CUDA_TRY(cudaStreamSynchronize(m.stream));
  }
  return 0;
  A2DS_GUARD_END
}

int a2ds_mesh_add_bcs(a2ds_mesh mesh, int num_bcs, const int *nodes, const int *masks,
                      const double *vals) {
  A2DS_GUARD_BEGIN
  int rc = check_mesh(mesh, false);
  if (rc) return rc;
  Mesh &m = mesh->m;
  if (m.planned) return fail(A2DS_ERR_STATE, "add Dirichlet conditions before planning");
  if (num_bcs < 0 || (num_bcs > 0 && (!nodes || !masks)))
    return fail(A2DS_ERR_ARG, "invalid boundary condition arrays");
  for (int b = 0; b < num_bcs; b++) {
    if (nodes[b] < 0 || nodes[b] >= m.nn) return fail(A2DS_ERR_ARG, "BC node out of range");
    m.bc_nodes.push_back(nodes[b]);
    m.bc_masks.push_back(masks[b] & 63);
    for (int k = 0; k < 6; k++) m.bc_vals.push_back(vals ? vals[(size_t)b * 6 + k] : 0.0);
  }
  return 0;
  A2DS_GUARD_END
}

int a2ds_mesh_plan(a2ds_mesh mesh, int order_type) {
  A2DS_GUARD_BEGIN
  int rc = check_mesh(mesh, false);
  if (rc) return rc;
  Mesh &m = mesh->m;
  if (m.planned) return fail(A2DS_ERR_STATE, "mesh already planned");
  if (order_type == A2DS_ND_ORDER)
    return fail(A2DS_ERR_ARG, "A2DS_ND_ORDER needs METIS (METIS_NodeND), which is not available");
  if (order_type != A2DS_NATURAL_ORDER && order_type != A2DS_RCM_ORDER &&
      order_type != A2DS_AMD_ORDER && order_type != A2DS_TACS_AMD_ORDER &&
      order_type != A2DS_MULTICOLOR_ORDER)
    return fail(A2DS_ERR_ARG, "unknown order_type");
  m.order_type = order_type;
  if ((rc = m.build_pattern())) return rc;
  m.planned = true;
  return 0;
  A2DS_GUARD_END
}

int a2ds_mesh_initialize(a2ds_mesh mesh, int order_type) {
  A2DS_GUARD_BEGIN
  int rc = check_mesh(mesh, false);
  if (rc) return rc;
  Mesh &m = mesh->m;
  if (m.initialized) return fail(A2DS_ERR_STATE, "mesh already initialized");
  if (m.planned && order_type != m.order_type)
    return fail(A2DS_ERR_ARG, "order_type differs from the planned ordering");
  if ((rc = ensure_device())) return rc;
  if (!m.planned && (rc = a2ds_mesh_plan(mesh, order_type))) return rc;
  if (!m.stream && cudaStreamCreateWithFlags(&m.stream, cudaStreamNonBlocking) != cudaSuccess)
    return fail(A2DS_ERR_CUDA, "cudaStreamCreate failed");
  A2DS_CUDA_TRY(cudaGetDevice(&m.device));
  if ((rc = m.upload())) return rc;
  m.initialized = true;
  return 0;
  A2DS_GUARD_END
}

int a2ds_mesh_get_pattern(a2ds_mesh mesh, int *nnzb, int *rowp, int *cols) {
  if (!mesh) return fail(A2DS_ERR_ARG, "null mesh handle");
  Mesh &m = mesh->m;
  if (!m.planned) return fail(A2DS_ERR_STATE, "mesh not planned");
  if (nnzb) *nnzb = m.nnzb;
  if (rowp) std::copy(m.rowp.begin(), m.rowp.end(), rowp);
  if (cols) std::copy(m.cols.begin(), m.cols.end(), cols);
  return 0;
}

int a2ds_mesh_ilu_pattern(a2ds_mesh mesh, int lev_fill, int *nnzb, int *rowp, int *cols) {
  A2DS_GUARD_BEGIN
  if (!mesh) return fail(A2DS_ERR_ARG, "null mesh handle");
  Mesh &m = mesh->m;
  if (!m.planned) return fail(A2DS_ERR_STATE, "mesh not planned");
  if (lev_fill < 0) return fail(A2DS_ERR_ARG, "lev_fill must be >= 0");
  std::vector<int> fr, fc, fd;
  int rc = ilu_symbolic(m.nn, m.rowp, m.cols, lev_fill, fr, fc, fd);
  if (rc) return fail(A2DS_ERR_STATE, "symbolic factorization failed");
  if (nnzb) *nnzb = fr[m.nn];
  if (rowp) std::copy(fr.begin(), fr.end(), rowp);
  if (cols) std::copy(fc.begin(), fc.end(), cols);
  return 0;
  A2DS_GUARD_END
}

int a2ds_mesh_get_ordering(a2ds_mesh mesh, int *perm) {
  if (!mesh) return fail(A2DS_ERR_ARG, "null mesh handle");
  if (!mesh->m.planned) return fail(A2DS_ERR_STATE, "mesh not planned");
  if (!perm) return fail(A2DS_ERR_ARG, "perm is null");
  std::copy(mesh->m.perm.begin(), mesh->m.perm.end(), perm);
  return 0;
}

int a2ds_mesh_node_csr(a2ds_mesh mesh, int nodiag, int *nnz, int *rowp, int *cols) {
  A2DS_GUARD_BEGIN
  int rc = check_mesh(mesh, false);
  if (rc) return rc;
  Mesh &m = mesh->m;
  std::vector<int> r, c;
  node_csr(m.nn, m.ne, m.npe, m.conn.data(), nodiag ? 1 : 0, r, c);
  if (nnz) *nnz = r[m.nn];
  if (rowp) std::copy(r.begin(), r.end(), rowp);
  if (cols) std::copy(c.begin(), c.end(), cols);
  return 0;
  A2DS_GUARD_END
}

int a2ds_bcsr_create(a2ds_mesh mesh, a2ds_bcsr *out) {
  A2DS_GUARD_BEGIN
  int rc = check_mesh(mesh, true);
  if (rc) return rc;
  if (!out) return fail(A2DS_ERR_ARG, "out is null");
  a2ds_bcsr A = new a2ds_bcsr_s();
  A->mesh = mesh;
  if ((rc = A->vals.alloc((size_t)mesh->m.nnzb * 36))) {
    delete A;
    return rc;
  }
  cudaMemsetAsync(A->vals.p, 0, A->vals.n * sizeof(double), mesh->m.stream);
  *out = A;
  return 0;
  A2DS_GUARD_END
}

int a2ds_bcsr_destroy(a2ds_bcsr mat) {
  delete mat;
  return 0;
}

int a2ds_bcsr_get(a2ds_bcsr mat, int *nrows, int *nnzb, int *rowp, int *cols, double *vals) {
  if (!mat) return fail(A2DS_ERR_ARG, "null matrix");
  Mesh &m = mat->mesh->m;
  if (nrows) *nrows = m.nn;
  if (nnzb) *nnzb = m.nnzb;
  if (rowp) std::copy(m.rowp.begin(), m.rowp.end(), rowp);
  if (cols) std::copy(m.cols.begin(), m.cols.end(), cols);
  if (vals) {
    A2DS_CUDA_TRY(cudaMemcpyAsync(vals, mat->vals.p, mat->vals.n * sizeof(double),
                                  cudaMemcpyDeviceToHost, m.stream));
    A2DS_CUDA_TRY(cudaStreamSynchronize(m.stream));
  }
  return 0;
}

int a2ds_bcsr_set_values(a2ds_bcsr mat, const double *vals) {
  if (!mat || !vals) return fail(A2DS_ERR_ARG, "null argument");
  Mesh &m = mat->mesh->m;
  A2DS_CUDA_TRY(cudaMemcpyAsync(mat->vals.p, vals, mat->vals.n * sizeof(double),
                                cudaMemcpyHostToDevice, m.stream));
  A2DS_CUDA_TRY(cudaStreamSynchronize(m.stream));
  return 0;
}

static int assemble(a2ds_mesh mesh, int mode, const double *vars, a2ds_bcsr A, double *res,
                    int scatter) {
  A2DS_GUARD_BEGIN
  int rc = check_mesh(mesh, true);
  if (rc) return rc;
  Mesh &m = mesh->m;
  if (A && A->mesh != mesh) return fail(A2DS_ERR_ARG, "matrix belongs to another mesh");
  const double *dst = nullptr;
  if (vars) {
    if ((rc = m.to_rows(vars, m.d_state))) return rc;
    dst = m.d_state.p;
  }
  if ((rc = m.assemble_device(mode, dst, A ? A->vals.p : nullptr, res ? m.d_res.p : nullptr,
                              scatter)))
    return rc;
  if (res) {
    if ((rc = m.from_rows(m.d_res.p, res))) return rc;
    // Dirichlet rows of the residual: vars - bcval (TACSBVec::applyBCs)
    for (size_t b = 0; b < m.bc_nodes.size(); b++)
      for (int k = 0; k < 6; k++)
        if (m.bc_masks[b] & (1 << k)) {
          size_t i = (size_t)m.bc_nodes[b] * 6 + k;
          res[i] = (vars ? vars[i] : 0.0) - m.bc_vals[b * 6 + k];
        }
  } else {
    A2DS_CUDA_TRY(cudaStreamSynchronize(m.stream));
  }
  return 0;
  A2DS_GUARD_END
}

int a2ds_assemble_mat_ex(a2ds_mesh mesh, int mat_type, const double *vars, a2ds_bcsr A,
                         int scatter) {
  if (!A) return fail(A2DS_ERR_ARG, "null matrix");
  if (scatter != A2DS_SCATTER_ATOMIC && scatter != A2DS_SCATTER_COLORED)
    return fail(A2DS_ERR_ARG, "unknown scatter strategy");
  int mode;
  if (mat_type == A2DS_STIFFNESS_MATRIX)
    mode = MODE_K;
  else if (mat_type == A2DS_GEOMETRIC_STIFFNESS_MATRIX)
    mode = MODE_G;
  else
    return fail(A2DS_ERR_ARG, "mat_type must be STIFFNESS (0) or GEOMETRIC_STIFFNESS (2)");
  return assemble(mesh, mode, vars, A, nullptr, scatter);
}

int a2ds_assemble_mat(a2ds_mesh mesh, int mat_type, const double *vars, a2ds_bcsr A) {
  return a2ds_assemble_mat_ex(mesh, mat_type, vars, A, A2DS_SCATTER_ATOMIC);
}

int a2ds_add_mat_xpt_sens_inner_product(a2ds_mesh mesh, int mat_type, double scale,
                                        const double *psi, const double *phi,
                                        const double *vars, double dh, double *dfdX) {
  A2DS_GUARD_BEGIN
  int rc = check_mesh(mesh, true);
  if (rc) return rc;
  if (!psi || !phi || !dfdX) return fail(A2DS_ERR_ARG, "null argument");
  int mode;
  if (mat_type == A2DS_STIFFNESS_MATRIX)
    mode = MODE_K;
  else if (mat_type == A2DS_GEOMETRIC_STIFFNESS_MATRIX)
    mode = MODE_G;
  else
    return fail(A2DS_ERR_ARG, "mat_type must be STIFFNESS (0) or GEOMETRIC_STIFFNESS (2)");
  if (dh == 0.0) dh = 1e-7;  // the reference's real-mode element step
  Mesh &m = mesh->m;
  DBuf<double> dpsi, dphi;
  if ((rc = m.to_rows(psi, dpsi)) || (rc = m.to_rows(phi, dphi))) return rc;
  const double *dst = nullptr;
  if (vars) {
    if ((rc = m.to_rows(vars, m.d_state))) return rc;
    dst = m.d_state.p;
  }
  ElemLaunch L = m.launch_params(mode, dst, nullptr, nullptr);
  L.cx = dpsi.p;
  L.cy = dphi.p;
  L.ccoef = scale;
  return m.fd_sens(L, dh, 0, dfdX);
  A2DS_GUARD_END
}

int a2ds_add_mat_dv_sens_inner_product(a2ds_mesh mesh, int mat_type, double scale,
                                       const double *psi, const double *phi,
                                       const double *vars, double *dfdx) {
  A2DS_GUARD_BEGIN
  int rc = check_mesh(mesh, true);
  if (rc) return rc;
  if (!psi || !phi || !dfdx) return fail(A2DS_ERR_ARG, "null argument");
  int mode;
  if (mat_type == A2DS_STIFFNESS_MATRIX)
    mode = MODE_K;
  else if (mat_type == A2DS_GEOMETRIC_STIFFNESS_MATRIX)
    mode = MODE_G;
  else
    return fail(A2DS_ERR_ARG, "mat_type must be STIFFNESS (0) or GEOMETRIC_STIFFNESS (2)");
  Mesh &m = mesh->m;
  const int ng = (int)m.tvals.size();
  DBuf<double> dpsi, dphi, dd;
  if ((rc = m.to_rows(psi, dpsi)) || (rc = m.to_rows(phi, dphi)) || (rc = dd.alloc(ng)))
    return rc;
  const double *dst = nullptr;
  if (vars) {
    if ((rc = m.to_rows(vars, m.d_state))) return rc;
    dst = m.d_state.p;
  }
  A2DS_CUDA_TRY(cudaMemsetAsync(dd.p, 0, ng * sizeof(double), m.stream));
  ElemLaunch L = m.launch_params(mode, dst, nullptr, nullptr);
  L.dconst = 1;  // element matrices with dC/dt: exact, they are linear in C
  L.cout = dd.p;
  L.cx = dpsi.p;
  L.cy = dphi.p;
  L.ccoef = scale;
  if ((rc = launch_element_kernel(L, m.stream))) return rc;
  m.launches++;
  std::vector<double> h(ng);
  A2DS_CUDA_TRY(cudaMemcpyAsync(h.data(), dd.p, ng * sizeof(double), cudaMemcpyDeviceToHost,
                                m.stream));
  A2DS_CUDA_TRY(cudaStreamSynchronize(m.stream));
  for (int g = 0; g < ng; g++) dfdx[g] += h[g];
  return 0;
  A2DS_GUARD_END
}

int a2ds_add_adjoint_res_xpt_sens_product(a2ds_mesh mesh, double scale, const double *psi,
                                          const double *vars, double dh, double *dfdX) {
  A2DS_GUARD_BEGIN
  int rc = check_mesh(mesh, true);
  if (rc) return rc;
  if (!psi || !dfdX) return fail(A2DS_ERR_ARG, "null argument");
  if (dh == 0.0) dh = 1e-7;  // the reference's real-mode element step
  Mesh &m = mesh->m;
  DBuf<double> dpsi;
  if ((rc = m.to_rows(psi, dpsi))) return rc;
  const double *dst = nullptr;
  if (vars) {
    if ((rc = m.to_rows(vars, m.d_state))) return rc;
    dst = m.d_state.p;
  }
  ElemLaunch L = m.launch_params(MODE_R, dst, nullptr, nullptr);
  L.cx = dpsi.p;
  L.ccoef = scale;
  return m.fd_sens(L, dh, 0, dfdX);
  A2DS_GUARD_END
}

int a2ds_eval_mat_sv_sens_inner_product(a2ds_mesh mesh, int mat_type, const double *psi,
                                        const double *phi, const double *vars, double dh,
                                        double *dfdu) {
  A2DS_GUARD_BEGIN
  int rc = check_mesh(mesh, true);
  if (rc) return rc;
  if (!psi || !phi || !dfdu) return fail(A2DS_ERR_ARG, "null argument");
  int mode;
  if (mat_type == A2DS_STIFFNESS_MATRIX)
    mode = MODE_K;
  else if (mat_type == A2DS_GEOMETRIC_STIFFNESS_MATRIX)
    mode = MODE_G;
  else
    return fail(A2DS_ERR_ARG, "mat_type must be STIFFNESS (0) or GEOMETRIC_STIFFNESS (2)");
  if (dh == 0.0) dh = 1e-7;
  Mesh &m = mesh->m;
  DBuf<double> dpsi, dphi;
  if ((rc = m.to_rows(psi, dpsi)) || (rc = m.to_rows(phi, dphi))) return rc;
  if ((rc = m.to_rows(vars, m.d_state))) return rc;  // NULL = zero state
  ElemLaunch L = m.launch_params(mode, m.d_state.p, nullptr, nullptr);
  L.cx = dpsi.p;
  L.cy = dphi.p;
  L.ccoef = 1.0;
  const size_t n6 = (size_t)m.nn * 6;
  std::fill(dfdu, dfdu + n6, 0.0);
  if ((rc = m.fd_sens(L, dh, 1, dfdu))) return rc;
  for (size_t b = 0; b < m.bc_nodes.size(); b++)
    for (int k = 0; k < 6; k++)
      if (m.bc_masks[b] & (1 << k)) dfdu[(size_t)m.bc_nodes[b] * 6 + k] = 0.0;
  return 0;
  A2DS_GUARD_END
}

int a2ds_assemble_res(a2ds_mesh mesh, const double *vars, double *res) {
  if (!res) return fail(A2DS_ERR_ARG, "res is null");
  return assemble(mesh, MODE_R, vars, nullptr, res, A2DS_SCATTER_ATOMIC);
}

int a2ds_assemble_jacobian(a2ds_mesh mesh, const double *vars, double *res, a2ds_bcsr A) {
  if (!A) return fail(A2DS_ERR_ARG, "null matrix");
  return assemble(mesh, res ? MODE_KR : MODE_K, vars, A, res, A2DS_SCATTER_ATOMIC);
}

int a2ds_bcsr_mult_rows(a2ds_bcsr A, const double *x, double *y) {
  A2DS_GUARD_BEGIN
  if (!A || !x || !y) return fail(A2DS_ERR_ARG, "null argument");
  Mesh &m = A->mesh->m;
  if (!m.initialized || !m.d_rowp.p || !m.d_cols.p || !A->vals.p)
    return fail(A2DS_ERR_STATE, "matrix of an uninitialized mesh");
  DBuf<double> dx, dy;
  int rc;
  if ((rc = dx.upload(x, (size_t)m.nn * 6, m.stream))) return rc;
  if ((rc = dy.alloc((size_t)m.nn * 6))) return rc;
  if ((rc = launch_spmv_f64(m.nn, m.d_rowp.p, m.d_cols.p, A->vals.p, dx.p, dy.p, m.stream)))
    return rc;
  A2DS_CUDA_TRY(cudaMemcpyAsync(y, dy.p, dy.n * sizeof(double), cudaMemcpyDeviceToHost, m.stream));
  A2DS_CUDA_TRY(cudaStreamSynchronize(m.stream));
  return 0;
  A2DS_GUARD_END
}

int a2ds_bcsr_time_mult_df(a2ds_bcsr A, int nvec, int iters, double *ms_per_mult) {
  A2DS_GUARD_BEGIN
  if (!A || !ms_per_mult) return fail(A2DS_ERR_ARG, "null argument");
  if (iters < 1 || iters > 100000) return fail(A2DS_ERR_ARG, "iters must be in [1, 100000]");
  if (nvec != 1 && nvec != 2 && nvec != 4 && nvec != 8 && nvec != 16)
    return fail(A2DS_ERR_ARG, "nvec must be 1, 2, 4, 8 or 16");
  Mesh &m = A->mesh->m;
  const size_t n = (size_t)m.nn * 6 * nvec, nv = (size_t)m.nnzb * 36;
  // double-float arrays held as float pairs
  DBuf<float> ad, dx, dy;
  int rc;
  if ((rc = ad.alloc(2 * nv)) || (rc = dx.alloc(n)) || (rc = dy.alloc(2 * n))) return rc;
  df64 *Ad = reinterpret_cast<df64 *>(ad.p), *Y = reinterpret_cast<df64 *>(dy.p);
  if ((rc = df_from_f64(Ad, A->vals.p, nv, m.stream))) return rc;
  A2DS_CUDA_TRY(cudaMemsetAsync(dx.p, 0, n * sizeof(float), m.stream));
  auto mult = [&]() { return df_spmm(m.nn, m.d_rowp.p, m.d_cols.p, Ad, dx.p, Y, nvec, m.stream); };
  for (int w = 0; w < 3; w++)
    if ((rc = mult())) return rc;
  cudaEvent_t e0, e1;
  A2DS_CUDA_TRY(cudaEventCreate(&e0));
  if (cudaEventCreate(&e1) != cudaSuccess) {
    cudaEventDestroy(e0);
    return fail(A2DS_ERR_CUDA, "cudaEventCreate failed");
  }
  float ms = 0.0f;
  cudaEventRecord(e0, m.stream);
  for (int it = 0; it < iters && !rc; it++) rc = mult();
  cudaEventRecord(e1, m.stream);
  cudaError_t e = cudaEventSynchronize(e1);
  if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (rc) return rc;
  if (e != cudaSuccess) return fail(A2DS_ERR_CUDA, cudaGetErrorString(e));
  m.launches += iters + 4;
  *ms_per_mult = (double)ms / iters;
  return 0;
  A2DS_GUARD_END
}

int a2ds_bcsr_time_mult(a2ds_bcsr A, int nvec, int iters, double *ms_per_mult) {
  A2DS_GUARD_BEGIN
  if (!A || !ms_per_mult) return fail(A2DS_ERR_ARG, "null argument");
  if (iters < 1 || iters > 100000) return fail(A2DS_ERR_ARG, "iters must be in [1, 100000]");
  if (nvec != 1 && nvec != 2 && nvec != 4 && nvec != 8 && nvec != 16)
    return fail(A2DS_ERR_ARG, "nvec must be 1, 2, 4, 8 or 16");
  Mesh &m = A->mesh->m;
  const size_t n = (size_t)m.nn * 6 * nvec;
  DBuf<double> dx, dy;
  int rc;
  if ((rc = dx.alloc(n)) || (rc = dy.alloc(n))) return rc;
  A2DS_CUDA_TRY(cudaMemsetAsync(dx.p, 0, n * sizeof(double), m.stream));
  auto mult = [&]() {
    return nvec == 1 ? launch_spmv_f64(m.nn, m.d_rowp.p, m.d_cols.p, A->vals.p, dx.p, dy.p,
                                       m.stream)
                     : blk_spmm(m.nn, m.d_rowp.p, m.d_cols.p, A->vals.p, dx.p, nullptr, dy.p,
                                nvec, m.stream);
  };
  for (int w = 0; w < 3; w++)
    if ((rc = mult())) return rc;
  cudaEvent_t e0, e1;
  A2DS_CUDA_TRY(cudaEventCreate(&e0));
  if (cudaEventCreate(&e1) != cudaSuccess) {
    cudaEventDestroy(e0);
    return fail(A2DS_ERR_CUDA, "cudaEventCreate failed");
  }
  float ms = 0.0f;
  cudaEventRecord(e0, m.stream);
  for (int it = 0; it < iters && !rc; it++) rc = mult();
  cudaEventRecord(e1, m.stream);
  cudaError_t e = cudaEventSynchronize(e1);
  if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (rc) return rc;
  if (e != cudaSuccess) return fail(A2DS_ERR_CUDA, cudaGetErrorString(e));
  m.launches += iters + 3;
  *ms_per_mult = (double)ms / iters;
  return 0;
  A2DS_GUARD_END
}

int a2ds_bcsr_mult(a2ds_bcsr A, const double *x, double *y) {
  A2DS_GUARD_BEGIN
  if (!A || !x || !y) return fail(A2DS_ERR_ARG, "null argument");
  Mesh &m = A->mesh->m;
  DBuf<double> dx, dy;
  int rc;
  if ((rc = m.to_rows(x, dx))) return rc;
  if ((rc = dy.alloc((size_t)m.nn * 6))) return rc;
  if ((rc = launch_spmv_f64(m.nn, m.d_rowp.p, m.d_cols.p, A->vals.p, dx.p, dy.p, m.stream)))
    return rc;
  return m.from_rows(dy.p, y);
  A2DS_GUARD_END
}

int a2ds_bcsr_copy(a2ds_bcsr Y, a2ds_bcsr X) {
  if (!Y || !X || Y->mesh != X->mesh) return fail(A2DS_ERR_ARG, "matrices must share a mesh");
  Mesh &m = Y->mesh->m;
  A2DS_CUDA_TRY(cudaMemcpyAsync(Y->vals.p, X->vals.p, X->vals.n * sizeof(double),
                                cudaMemcpyDeviceToDevice, m.stream));
  A2DS_CUDA_TRY(cudaStreamSynchronize(m.stream));
  return 0;
}

int a2ds_bcsr_axpy(a2ds_bcsr Y, double alpha, a2ds_bcsr X) {
  if (!Y || !X || Y->mesh != X->mesh) return fail(A2DS_ERR_ARG, "matrices must share a mesh");
  Mesh &m = Y->mesh->m;
  int rc = launch_axpy(Y->vals.p, alpha, X->vals.p, X->vals.n, m.stream);
  if (rc) return rc;
  A2DS_CUDA_TRY(cudaStreamSynchronize(m.stream));
  return 0;
}

int a2ds_bcsr_apply_bcs(a2ds_bcsr A) {
  if (!A) return fail(A2DS_ERR_ARG, "null matrix");
  Mesh &m = A->mesh->m;
  int rc = launch_apply_bc_rows(A->vals.p, m.d_rowp.p, m.d_cols.p, m.d_bc_rows.p, m.d_bc_masks.p,
                                (int)m.bc_rows.size(), m.stream);
  if (rc) return rc;
  A2DS_CUDA_TRY(cudaStreamSynchronize(m.stream));
  return 0;
}

}  // extern "C"
