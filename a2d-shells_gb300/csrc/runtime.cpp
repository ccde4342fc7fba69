// Host runtime behind the C ABI: mesh handles (the TACSAssembler role),
// BCSR matrix handles (TACSSchurMat / BCSRMat role), the node-to-node
// pattern, the matrix ordering, element-slot maps and element colours.
#include <string.h>

#include <algorithm>
#include <cmath>
#include <mutex>
#include <numeric>
#include <string>
#include <vector>

#include "a2ds_internal.h"
#include "host_graph.h"
#include "kernels.h"
#include "runtime.h"

namespace a2ds {

static thread_local std::string g_last_error;

void set_error(int code, const std::string &msg) {
  (void)code;
  g_last_error = msg;
}
const char *last_error_cstr() { return g_last_error.c_str(); }

int fail(int code, const std::string &msg) {
  set_error(code, msg);
  return code;
}

int ensure_device() {
  static std::once_flag once;
  static int status = 0;
  static std::string msg;
  std::call_once(once, [] {
    int n = 0;
    cudaError_t e = cudaGetDeviceCount(&n);
    if (e != cudaSuccess || n == 0) {
      status = A2DS_ERR_CUDA;
      msg = std::string("no usable CUDA device: ") +
            (e != cudaSuccess ? cudaGetErrorString(e) : "device count is 0");
      return;
    }
    int rc = upload_shell_tables();
    if (rc) {
      status = rc;
      msg = g_last_error;
    }
  });
  if (status) return fail(status, msg);
  return 0;
}

// ------------------------------------------------------------ mesh setup
int Mesh::build_pattern() {
  // node -> node pattern with the diagonal, sorted and unique per row
  // (TACSAssembler::computeLocalNodeToNodeCSR + TacsSortAndUniquifyCSR)
  node_csr(nn, ne, npe, conn.data(), 0, node_rowp, node_cols);

  // TACSAssembler::createSchurMat(order_type) on one process (no coupling
  // nodes) -> computeMatReordering (src/TACSAssembler.cpp:1508-1600)
  perm.resize(nn);
  if (order_type == A2DS_TACS_AMD_ORDER || order_type == A2DS_AMD_ORDER) {
    // AMD_ORDER without the external AMD library is the same call
    std::vector<int> rp, cl;
    node_csr(nn, ne, npe, conn.data(), 1, rp, cl);
    amd_order(nn, rp, cl, perm);
  } else if (order_type == A2DS_RCM_ORDER || order_type == A2DS_MULTICOLOR_ORDER) {
    std::vector<int> new_vars, colors;
    if (order_type == A2DS_RCM_ORDER)
      rcm_order(nn, node_rowp, node_cols, 0, 1, new_vars);
    else
      multicolor_order(nn, node_rowp, node_cols, colors, new_vars);
    for (int k = 0; k < nn; k++) perm[new_vars[k]] = k;
  } else {
    std::iota(perm.begin(), perm.end(), 0);
  }
  iperm.assign(nn, -1);
  for (int i = 0; i < nn; i++) iperm[perm[i]] = i;

  // BCSR pattern in the row ordering: row i <-> node perm[i]
  rowp.assign(nn + 1, 0);
  for (int i = 0; i < nn; i++) {
    int node = perm[i];
    rowp[i + 1] = rowp[i] + (node_rowp[node + 1] - node_rowp[node]);
  }
  cols.resize(rowp[nn]);
  for (int i = 0; i < nn; i++) {
    int node = perm[i];
    int *c = &cols[rowp[i]];
    int k = 0;
    for (int jp = node_rowp[node]; jp < node_rowp[node + 1]; jp++) c[k++] = iperm[node_cols[jp]];
    std::sort(c, c + k);
  }
  nnzb = rowp[nn];

  // element connectivity in rows, and the element-slot map
  const int nn2 = npe * npe;
  conn_rows.resize((size_t)ne * npe);
  slots.resize((size_t)ne * nn2);
  for (int e = 0; e < ne; e++) {
    for (int a = 0; a < npe; a++) conn_rows[(size_t)e * npe + a] = iperm[conn[(size_t)e * npe + a]];
    for (int a = 0; a < npe; a++) {
      int r = conn_rows[(size_t)e * npe + a];
      const int *c0 = &cols[rowp[r]], *c1 = &cols[rowp[r + 1]];
      for (int b = 0; b < npe; b++) {
        int c = conn_rows[(size_t)e * npe + b];
        const int *f = std::lower_bound(c0, c1, c);
        if (f == c1 || *f != c)
          return fail(A2DS_ERR_STATE, "internal: element block missing from the pattern");
        slots[(size_t)e * nn2 + a * npe + b] = (int)(rowp[r] + (f - c0));
      }
    }
  }

  // element colours (no two elements of one colour share a node)
  greedy_element_colors(nn, ne, npe, conn.data(), color_ptr, color_elems);

  // Dirichlet rows
  bc_rows.resize(bc_nodes.size());
  for (size_t b = 0; b < bc_nodes.size(); b++) bc_rows[b] = iperm[bc_nodes[b]];
  return 0;
}

int Mesh::upload() {
  int rc;
  std::vector<double> Xr((size_t)nn * 3);
  for (int i = 0; i < nn; i++)
    for (int c = 0; c < 3; c++) Xr[(size_t)i * 3 + c] = X[(size_t)perm[i] * 3 + c];
  if ((rc = d_X.upload(Xr.data(), Xr.size(), stream))) return rc;
  if ((rc = d_conn.upload(conn_rows.data(), conn_rows.size(), stream))) return rc;
  if ((rc = d_slots.upload(slots.data(), slots.size(), stream))) return rc;
  if ((rc = d_rowp.upload(rowp.data(), rowp.size(), stream))) return rc;
  if ((rc = d_cols.upload(cols.data(), cols.size(), stream))) return rc;
  if ((rc = d_tvals.upload(tvals.data(), tvals.size(), stream))) return rc;
  if ((rc = d_tgroup.upload(tgroup.data(), tgroup.size(), stream))) return rc;
  if ((rc = d_bc_rows.upload(bc_rows.data(), bc_rows.size(), stream))) return rc;
  if ((rc = d_bc_masks.upload(bc_masks.data(), bc_masks.size(), stream))) return rc;
  if ((rc = d_color_elems.upload(color_elems.data(), color_elems.size(), stream))) return rc;
  if ((rc = d_state.alloc((size_t)nn * 6))) return rc;
  if ((rc = d_res.alloc((size_t)nn * 6))) return rc;
  A2DS_CUDA_TRY(cudaStreamSynchronize(stream));
  return 0;
}

// Node-ordered host vector -> row-ordered device vector
int Mesh::to_rows(const double *h, DBuf<double> &d) {
  const size_t n6 = (size_t)nn * 6;
  int rc = d.alloc(n6);
  if (rc) return rc;
  if ((rc = h_stage.reserve(n6))) return rc;
  double *st = h_stage.p;
  if (h) {
    for (int i = 0; i < nn; i++) memcpy(&st[(size_t)i * 6], &h[(size_t)perm[i] * 6], 6 * sizeof(double));
  } else {
    std::fill(st, st + n6, 0.0);
  }
  A2DS_CUDA_TRY(cudaMemcpyAsync(d.p, st, n6 * sizeof(double), cudaMemcpyHostToDevice, stream));
  A2DS_CUDA_TRY(cudaStreamSynchronize(stream));
  return 0;
}

// Row-ordered device vector -> node-ordered host vector
int Mesh::from_rows(const double *d, double *h) {
  const size_t n6 = (size_t)nn * 6;
  int rc;
  if ((rc = h_stage.reserve(n6))) return rc;
  double *st = h_stage.p;
  A2DS_CUDA_TRY(cudaMemcpyAsync(st, d, n6 * sizeof(double), cudaMemcpyDeviceToHost, stream));
  A2DS_CUDA_TRY(cudaStreamSynchronize(stream));
  for (int i = 0; i < nn; i++) memcpy(&h[(size_t)perm[i] * 6], &st[(size_t)i * 6], 6 * sizeof(double));
  return 0;
}

ElemLaunch Mesh::launch_params(int mode, const double *d_st, double *vals, double *res) const {
  ElemLaunch L;
  memset(&L, 0, sizeof(L));
  L.order = order;
  L.nonlinear = nonlinear;
  L.mode = mode;
  L.num_elements = ne;
  L.elem_list = nullptr;
  L.conn = d_conn.p;
  L.slots = d_slots.p;
  L.X = d_X.p;
  L.state = d_st;
  L.tvals = d_tvals.p;
  L.tgroup = d_tgroup.p;
  L.E = E;
  L.nu = nu;
  L.alpha = alpha;
  L.temperature = temperature;
  L.vals = vals;
  L.res = res;
  L.atomic_scatter = 1;
  return L;
}

int Mesh::element_output(const double *d_st, double *d_out) {
  ElemLaunch L = launch_params(MODE_OUT, d_st, nullptr, nullptr);
  L.out = d_out;
  int rc;
  if ((rc = launch_element_kernel(L, stream))) return rc;
  launches++;
  return 0;
}

// Element-by-element central differences (fdOrder 2) of the contractions
// that L describes, in each element coordinate (wrt_state = 0: the
// reference's TACSElement::addMatXptSensInnerProduct and addAdjResXptProduct,
// src/elements/TACSElement.cpp:434-507, 270-330) or each element state entry
// (wrt_state = 1: getMatSVSensInnerProduct, :509-581), step +/- dh.  Every
// element holds its own copy of its coordinates and state, so one launch
// steps entry k of all elements at once; the two launches of a step add
// +/- coef / (2 dh) times the contraction into ce[e][k].  The element rows
// are summed into the nodes on the host, element by element in order:
// out is num_nodes x 3 (coordinates) or num_nodes x 6 (state), caller
// numbering, added into.
int Mesh::fd_sens(ElemLaunch L, double dh, int wrt_state, double *out) {
  if (!(dh > 0.0) || !std::isfinite(dh)) return fail(A2DS_ERR_ARG, "finite-difference step must be > 0");
  const int per = wrt_state ? 6 : 3, nk = per * npe;
  DBuf<double> ce;
  int rc;
  if ((rc = ce.alloc((size_t)ne * nk))) return rc;
  A2DS_CUDA_TRY(cudaMemsetAsync(ce.p, 0, ce.n * sizeof(double), stream));
  const double c1 = L.ccoef, c2 = L.ccoef2;
  L.cout = ce.p;
  L.cstride = nk;
  L.xstate = wrt_state ? 1 : 0;
  for (int k = 0; k < nk; k++)
    for (int sgn = 1; sgn >= -1; sgn -= 2) {
      L.xk = k;
      L.xh = sgn * dh;
      L.ccoef = sgn * c1 / (2.0 * dh);
      L.ccoef2 = sgn * c2 / (2.0 * dh);
      if ((rc = launch_element_kernel(L, stream))) return rc;
      launches++;
    }
  std::vector<double> h;
  try {
    h.resize(ce.n);
  } catch (const std::bad_alloc &) {
    return fail(A2DS_ERR_NOMEM, "host allocation failed");
  }
  A2DS_CUDA_TRY(cudaMemcpyAsync(h.data(), ce.p, ce.n * sizeof(double), cudaMemcpyDeviceToHost, stream));
  A2DS_CUDA_TRY(cudaStreamSynchronize(stream));
  for (int e = 0; e < ne; e++)
    for (int k = 0; k < nk; k++)
      out[(size_t)conn[(size_t)e * npe + k / per] * per + k % per] += h[(size_t)e * nk + k];
  return 0;
}

// Element assembly into vals (zeroed first) and/or res, device state
int Mesh::assemble_device(int mode, const double *d_st, double *vals, double *res, int scatter) {
  int rc;
  if (vals) A2DS_CUDA_TRY(cudaMemsetAsync(vals, 0, (size_t)nnzb * 36 * sizeof(double), stream));
  if (res) A2DS_CUDA_TRY(cudaMemsetAsync(res, 0, (size_t)nn * 6 * sizeof(double), stream));
  ElemLaunch L = launch_params(mode, d_st, vals, res);
  if (scatter == A2DS_SCATTER_COLORED) {
    L.atomic_scatter = 0;
    const int ncol = (int)color_ptr.size() - 1;
    for (int c = 0; c < ncol; c++) {
      L.elem_list = d_color_elems.p + color_ptr[c];
      L.num_elements = color_ptr[c + 1] - color_ptr[c];
      if ((rc = launch_element_kernel(L, stream))) return rc;
      launches++;
    }
  } else {
    if ((rc = launch_element_kernel(L, stream))) return rc;
    launches++;
  }
  if (vals) {
    if ((rc = launch_apply_bc_rows(vals, d_rowp.p, d_cols.p, d_bc_rows.p, d_bc_masks.p,
                                   (int)bc_rows.size(), stream)))
      return rc;
    launches++;
  }
  return 0;
}

}  // namespace a2ds
