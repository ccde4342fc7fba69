// y = A x for callers that must not allocate device memory.
//
// a2ds_bcsr_mult_rows stages x and y through device buffers it allocates on
// every call.  Some callers cannot allow that: applications whose own
// memory manager has reserved the whole device up front (a framework with a
// caching pool leaves nothing for cudaMalloc), latency-critical loops that
// must not pay for cudaFree (it waits for the whole device, stalling work on
// every other stream), and runtimes that forbid allocator calls after start-up.
// This variant stages through a fixed file-scope device array instead and
// performs no allocation.
//
// The scratch array holds 2 x 6 x A2DS_NOALLOC_MAX_ROWS doubles (6.3 MB);
// every GPU that loads this library keeps it until the process exits.  Its
// device address is looked up once per device, on the first call made with
// that device current (cudaGetSymbolAddress); make that first call before
// any stream capture.  The cached address belongs to the device's current
// context: do not use this entry point across a device reset
// (cudaDeviceReset) in the same process.  The device current at the call
// must be the one the matrix's mesh was initialized on (the array of
// another device would be staged through otherwise); a mismatch is
// rejected.  All calls share the one array and it keeps the last call's
// contents: the leading 6 n entries of both halves are overwritten by every
// call (x by the host copy, y by the product) and nothing past them is
// read, so nothing needs clearing, but calls that overlap on the GPU race
// on it.
#include <mutex>

#include "a2ds_internal.h"
#include "kernels.h"
#include "runtime.h"

#define A2DS_NOALLOC_MAX_ROWS 65536

namespace a2ds {

static __device__ __align__(256) double g_noalloc_scratch[2 * 6 * A2DS_NOALLOC_MAX_ROWS];

static std::mutex g_noalloc_mu;
static double *g_noalloc_addr[64];  // per device ordinal

// Device address of the scratch array for the current device.
static int noalloc_scratch(double **out) {
  int dev = 0;
  A2DS_CUDA_TRY(cudaGetDevice(&dev));
  if (dev < 0 || dev >= 64) return fail(A2DS_ERR_CUDA, "device ordinal out of range");
  std::lock_guard<std::mutex> lk(g_noalloc_mu);
  if (!g_noalloc_addr[dev]) {
    void *p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p)
      return fail(A2DS_ERR_CUDA, std::string("cudaGetSymbolAddress(scratch): ") +
                                     cudaGetErrorString(e));
    g_noalloc_addr[dev] = (double *)p;
  }
  *out = g_noalloc_addr[dev];
  return 0;
}

}  // namespace a2ds

using namespace a2ds;

extern "C" int a2ds_bcsr_mult_rows_noalloc(a2ds_bcsr A, const double *x, double *y) try {
  if (!A || !x || !y) return fail(A2DS_ERR_ARG, "null argument");
  Mesh &m = A->mesh->m;
  if (!m.initialized || !m.d_rowp.p || !m.d_cols.p || !A->vals.p)
    return fail(A2DS_ERR_STATE, "matrix of an uninitialized mesh");
  int dev = -1;
  A2DS_CUDA_TRY(cudaGetDevice(&dev));
  if (dev != m.device)
    return fail(A2DS_ERR_ARG, "current device " + std::to_string(dev) +
                                  " is not the mesh's device " + std::to_string(m.device));
  if (m.nn > A2DS_NOALLOC_MAX_ROWS)
    return fail(A2DS_ERR_ARG, "a2ds_bcsr_mult_rows_noalloc supports at most " +
                                  std::to_string(A2DS_NOALLOC_MAX_ROWS) + " block rows (matrix has " +
                                  std::to_string(m.nn) + ")");
  double *scratch = nullptr;
  int rc = noalloc_scratch(&scratch);
  if (rc) return rc;
  const size_t n6 = (size_t)m.nn * 6;
  double *dx = scratch, *dy = scratch + 6 * (size_t)A2DS_NOALLOC_MAX_ROWS;
  A2DS_CUDA_TRY(cudaMemcpyAsync(dx, x, n6 * sizeof(double), cudaMemcpyHostToDevice, m.stream));
  if ((rc = launch_spmv_f64(m.nn, m.d_rowp.p, m.d_cols.p, A->vals.p, dx, dy, m.stream))) return rc;
  A2DS_CUDA_TRY(cudaMemcpyAsync(y, dy, n6 * sizeof(double), cudaMemcpyDeviceToHost, m.stream));
  A2DS_CUDA_TRY(cudaStreamSynchronize(m.stream));
  return 0;
} catch (...) {
  return fail(A2DS_ERR_STATE, "unexpected host exception");
}
