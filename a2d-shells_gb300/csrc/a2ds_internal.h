// Internal declarations shared by the a2ds translation units (host C++ and
// CUDA).  Not part of the public ABI (include/a2ds.h).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <string>
#include <vector>

#include "a2ds.h"

namespace a2ds {

// ------------------------------------------------------------------ errors
struct Error {
  int code;
  std::string msg;
};
void set_error(int code, const std::string &msg);
int fail(int code, const std::string &msg);  // sets and returns code
const char *last_error_cstr();

#define A2DS_CUDA_TRY(expr)                                                  \
  do {                                                                       \
    cudaError_t _e = (expr);                                                 \
    if (_e != cudaSuccess)                                                   \
      return ::a2ds::fail(A2DS_ERR_CUDA, std::string(#expr) + ": " +         \
                                             cudaGetErrorString(_e));        \
  } while (0)

// ----------------------------------------------------------- device buffer
template <typename T>
struct DBuf {
  T *p = nullptr;
  size_t n = 0;
  DBuf() = default;
  DBuf(const DBuf &) = delete;
  DBuf &operator=(const DBuf &) = delete;
  ~DBuf() { release(); }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    n = 0;
  }
  int alloc(size_t count) {
    if (count == n && p) return 0;
    release();
    if (count == 0) return 0;
    cudaError_t e = cudaMalloc((void **)&p, count * sizeof(T));
    if (e != cudaSuccess) {
      p = nullptr;
      return fail(A2DS_ERR_NOMEM, std::string("cudaMalloc of ") +
                                      std::to_string(count * sizeof(T)) + " bytes: " +
                                      cudaGetErrorString(e));
    }
    n = count;
    return 0;
  }
  int upload(const T *h, size_t count, cudaStream_t s) {
    int rc = alloc(count);
    if (rc) return rc;
    if (count) A2DS_CUDA_TRY(cudaMemcpyAsync(p, h, count * sizeof(T), cudaMemcpyHostToDevice, s));
    return 0;
  }
};

// Page-locked host staging buffer (grown on demand): host<->device copies at
// the C ABI run from pinned memory at full link rate.
template <typename T>
struct PinnedBuf {
  T *p = nullptr;
  size_t n = 0;
  PinnedBuf() = default;
  PinnedBuf(const PinnedBuf &) = delete;
  PinnedBuf &operator=(const PinnedBuf &) = delete;
  ~PinnedBuf() {
    if (p) cudaFreeHost(p);
  }
  int reserve(size_t count) {
    if (p && count <= n) return 0;
    if (p) cudaFreeHost(p);
    p = nullptr;
    n = 0;
    cudaError_t e = cudaMallocHost((void **)&p, count * sizeof(T));
    if (e != cudaSuccess) {
      p = nullptr;
      return fail(A2DS_ERR_NOMEM, std::string("cudaMallocHost of ") +
                                      std::to_string(count * sizeof(T)) + " bytes: " +
                                      cudaGetErrorString(e));
    }
    n = count;
    return 0;
  }
};

// --------------------------------------------------------- element kernel
// MODE_OUT: strain and stress of the state at each element's node points
// (TACSShellElement::getOutputData), written to out (element-major).
enum ElemMode { MODE_K = 0, MODE_G = 1, MODE_R = 2, MODE_KR = 3, MODE_OUT = 4 };

struct ElemLaunch {
  int order;             // 2 or 3
  int nonlinear;         // model: 0 linear, 1 nonlinear
  int mode;              // ElemMode
  int num_elements;      // elements in this launch (subset via elem_list)
  const int *elem_list;  // element ids for this launch (NULL = 0..num_elements-1)
  const int *conn;       // Ne x NN, node rows in matrix ordering
  const int *slots;      // Ne x NN*NN block indices
  const double *X;       // Nn x 3, matrix ordering
  const double *state;   // Nn x 6, matrix ordering (NULL = zero)
  const double *tvals;   // thickness per group
  const int *tgroup;     // group per element
  double E, nu, alpha, temperature;
  double *vals;          // BCSR values (36 per block) or NULL
  double *res;           // residual (Nn x 6) or NULL
  int atomic_scatter;    // 1 atomics, 0 plain adds (colour-ordered launch)
  // Design sensitivities: dconst = 1 evaluates the matrix with the thickness
  // derivative of the constitutive matrix (the element matrices are linear
  // in it); cout != NULL replaces the scatter by the contraction
  // cout[group(e)] += ccoef * cx_e^T M_e cy_e (cx, cy node-major, matrix ordering).
  int dconst;
  const double *cx, *cy;
  double *cout;
  double ccoef;
  // optional second contraction in the same launch (NULL = none)
  const double *cx2, *cy2;
  double ccoef2;
  // Finite-difference sensitivities: cstride != 0 adds xh to the element's
  // local coordinate xk (0..3*NN-1), or with xstate = 1 to its local state
  // entry xk (0..6*NN-1), and sends the contractions to cout[e * cstride + xk]
  // instead of the design group.  MODE_R with cout contracts the element
  // residual with cx instead of scattering it.
  int cstride, xk, xstate;
  double xh;
  // MODE_OUT: Ne x NN x 18 (strain e[9], stress C e[9] per node point)
  double *out;
};

int launch_element_kernel(const ElemLaunch &L, cudaStream_t s);
int upload_shell_tables();

// ---------------------------------------------------------- BCSR helpers
int launch_apply_bc_rows(double *vals, const int *rowp, const int *cols,
                         const int *bc_rows, const int *bc_masks, int nbc,
                         cudaStream_t s);

}  // namespace a2ds
