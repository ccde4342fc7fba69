// Handle types behind the opaque C ABI pointers.
#pragma once

#include <vector>

#include "a2ds_internal.h"

namespace a2ds {

int ensure_device();
struct Mesh;
void release_solver(Mesh &m);

struct Mesh {
  int nn = 0, ne = 0, npe = 0, order = 0, nonlinear = 0;
  std::vector<int> conn;    // ne x npe, caller's node numbering
  std::vector<double> X;    // nn x 3
  double E = 70e9, nu = 0.3, alpha = 0.0, temperature = 0.0;
  double ys = 0.0;  // yield stress for the failure output (0: not set)
  std::vector<double> tvals{1e-2};
  std::vector<int> tgroup;  // ne
  std::vector<int> bc_nodes, bc_masks;
  std::vector<double> bc_vals;  // nbc x 6

  bool planned = false;      // host pattern/ordering built
  bool initialized = false;  // uploaded to the device
  int order_type = A2DS_NATURAL_ORDER;
  std::vector<int> node_rowp, node_cols;  // node CSR with diagonal (caller numbering)
  std::vector<int> perm, iperm;           // row -> node, node -> row
  std::vector<int> rowp, cols;            // BCSR pattern (rows)
  int nnzb = 0;
  std::vector<int> conn_rows, slots;
  std::vector<int> color_ptr, color_elems;
  std::vector<int> bc_rows;

  cudaStream_t stream = nullptr;
  int device = -1;  // CUDA device current at initialize (the stream's device)
  DBuf<double> d_X, d_tvals, d_state, d_res;
  DBuf<int> d_conn, d_slots, d_rowp, d_cols, d_tgroup, d_bc_rows, d_bc_masks, d_color_elems;
  PinnedBuf<double> h_stage;  // pinned staging of node <-> row permuted vectors
  long long launches = 0;

  // buckling-solve state kept for sensitivities / stats
  std::vector<double> stats;
  void *solver = nullptr;   // BucklingState*
  void *preload = nullptr;  // PreloadState* (Newton load stepping)

  int build_pattern();
  int upload();
  int to_rows(const double *h, DBuf<double> &d);
  int from_rows(const double *d, double *h);
  ElemLaunch launch_params(int mode, const double *d_st, double *vals, double *res) const;
  int assemble_device(int mode, const double *d_st, double *vals, double *res, int scatter);
  // strain and stress at every element's node points (MODE_OUT), d_out
  // ne x npe x 18 on the device
  int element_output(const double *d_st, double *d_out);
  // Derivative of the element contractions that L describes (cx, cy, ccoef
  // and optionally cx2, cy2, ccoef2; or cx^T R_e for MODE_R) with respect to
  // every element coordinate (wrt_state = 0; out nn x 3) or state entry
  // (wrt_state = 1; out nn x 6), by second-order central differences with
  // step dh; added into out (caller numbering).
  int fd_sens(ElemLaunch L, double dh, int wrt_state, double *out);
  ~Mesh();
};

}  // namespace a2ds

struct a2ds_mesh_s {
  a2ds::Mesh m;
};

struct a2ds_bcsr_s {
  a2ds_mesh mesh = nullptr;
  a2ds::DBuf<double> vals;
};
