/*
  Reference timing: the reference's own buckling solve,
  TACSLinearBuckling::solve (src/TACSBuckling.cpp:197-273), compiled from the
  reference's sources by oracle/ref/Makefile, on a mesh written by
  oracle/ref/ref_timing.py.  Test infrastructure only: it times the
  reference, it ships nothing.

  The set-up is the reference cylinder example's
  (examples/cylinder-buckling/mechBuckling.cpp:104-160): one TACSAssembler of
  Quad4/Quad9 shells (one element object per thickness value), K, G and the
  shifted operator as TACSSchurMat (AMD row ordering), a TACSSchurPc on K with
  lev = params[3] (1e6: complete LU), GMRES(params[4], params[5]) on
  K + sigma G preconditioned by that factor, and TACSLinearBuckling with
  max_lanczos = params[6], num_eigvals = params[7] and eig_tol = params[12];
  the lowest params[13] loads are printed.  The reference's Lanczos
  (SEP::solve, src/bpmat/GSEP.cpp:480-570) stops as soon as it has
  num_eigvals vectors: its convergence test returns "converged" from
  n = num_eigvals on (SEP::checkConverged, src/bpmat/GSEP.cpp:754-789, the
  error estimate commented out), so num_eigvals sets the number of Lanczos
  vectors and therefore the accuracy, as the cylinder example's comment
  says (mechBuckling.cpp:147).
  Host threads: TACSAssembler::setNumThreads (src/TACSAssembler.cpp:306),
  which the factorization, products and triangular solves of BCSRMat use.

    cpu_ref_bench <in_dir> <threads> [verbose]

  (verbose: the GMRES residuals and the Lanczos table on stderr.)  Timed
  with std::chrono around solve() alone: assembly of K, its factor, the load
  path, G, the shifted operator, its factor and the Lanczos iteration.
  Prints one JSON line: threads, seconds, GMRES iterations (one factor
  application each) and cycles (restarts + solves), the eigenvalues and
  their error estimates.
*/
#include <math.h>
#include <stdio.h>

#include <algorithm>
#include <chrono>
#include <string>
#include <vector>

#include "KSM.h"
#include "TACSAssembler.h"
#include "TACSBuckling.h"
#include "TACSIsoShellConstitutive.h"
#include "TACSMaterialProperties.h"
#include "TACSSchurMat.h"
#include "TACSShellElementDefs.h"
#include "TACSShellElementTransform.h"
#include "npy_io.h"

// GMRES monitor that only counts: printResidual(0, .) opens every cycle
// (the start of a solve or a restart), printResidual(i > 0, .) follows every
// iteration (src/bpmat/KSM.cpp:800-880).
class CountingPrint : public KSMPrint {
 public:
  long iterations = 0, cycles = 0;
  bool echo = false;
  void printResidual(int iter, TacsScalar r) override {
    if (iter == 0)
      cycles++;
    else
      iterations++;
    if (echo) fprintf(stderr, "gmres %4d %.3e\n", iter, TacsRealPart(r));
  }
  void print(const char *s) override {
    if (echo) fputs(s, stderr);
  }
};

int main(int argc, char **argv) {
  if (argc < 3) {
    fprintf(stderr, "usage: cpu_ref_bench <in_dir> <threads> [verbose]\n");
    return 2;
  }
  MPI_Init(&argc, &argv);
  const std::string in = argv[1];
  const int threads = atoi(argv[2]);
  const bool verbose = argc > 3;
  std::vector<long> xs, cs;
  std::vector<double> X = read_npy<double>(in + "/X.npy", &xs);
  std::vector<int> conn = read_npy<int>(in + "/conn.npy", &cs);
  std::vector<int> bc_nodes = read_npy<int>(in + "/bc_nodes.npy");
  std::vector<int> bc_mask = read_npy<int>(in + "/bc_mask.npy");
  std::vector<double> bc_vals = read_npy<double>(in + "/bc_vals.npy");
  std::vector<double> rhs = read_npy<double>(in + "/rhs.npy");
  std::vector<double> prm = read_npy<double>(in + "/params.npy");
  std::vector<double> thick = read_npy<double>(in + "/elem_thickness.npy");
  const int nn = (int)xs[0], ne = (int)cs[0], npe = (int)cs[1];
  if (prm.size() < 13 || (npe != 4 && npe != 9)) {
    fprintf(stderr, "cpu_ref_bench: need 13 parameters and 4- or 9-node elements\n");
    return 2;
  }
  const double E = prm[0], nu = prm[1], sigma = prm[2];
  const int lev = (int)prm[3], gm_m = (int)prm[4], gm_restarts = (int)prm[5];
  const int max_lanczos = (int)prm[6], neig = (int)prm[7];
  const double gm_tol = prm[9], eig_tol = prm[12];
  const int nreport = prm.size() > 13 ? std::min((int)prm[13], neig) : neig;

  TACSShellTransform *tr = new TACSShellNaturalTransform();
  tr->incref();
  TACSMaterialProperties *props =
      new TACSMaterialProperties(2700.0, 921.0, E, nu, 270e6, 0.0, 230.0);
  props->incref();
  std::vector<TACSElement *> elems(ne), tobjs;
  std::vector<double> tvals;
  for (int e = 0; e < ne; e++) {
    int k = -1;
    for (size_t j = 0; j < tvals.size(); j++)
      if (tvals[j] == thick[e]) k = (int)j;
    if (k < 0) {
      TACSIsoShellConstitutive *con =
          new TACSIsoShellConstitutive(props, thick[e], (int)tvals.size());
      TACSElement *el;
      if (npe == 4)
        el = new TACSQuad4Shell(tr, con);
      else
        el = new TACSQuad9Shell(tr, con);
      el->incref();
      tvals.push_back(thick[e]);
      tobjs.push_back(el);
      k = (int)tvals.size() - 1;
    }
    elems[e] = tobjs[k];
  }

  TACSAssembler *assembler = new TACSAssembler(MPI_COMM_WORLD, 6, nn, ne);
  assembler->incref();
  std::vector<int> ptr(ne + 1);
  for (int e = 0; e <= ne; e++) ptr[e] = npe * e;
  assembler->setElementConnectivity(ptr.data(), conn.data());
  assembler->setElements(elems.data());
  for (size_t b = 0; b < bc_nodes.size(); b++) {
    int vars[6], nv = 0;
    TacsScalar vals[6];
    for (int k = 0; k < 6; k++)
      if (bc_mask[b] & (1 << k)) {
        vals[nv] = bc_vals[6 * b + k];
        vars[nv++] = k;
      }
    assembler->addBCs(1, &bc_nodes[b], nv, vars, vals);
  }
  assembler->initialize();
  assembler->setNumThreads(threads);
  TACSBVec *Xvec = assembler->createNodeVec();
  Xvec->incref();
  TacsScalar *xa;
  Xvec->getArray(&xa);
  for (int i = 0; i < 3 * nn; i++) xa[i] = X[i];
  assembler->setNodes(Xvec);

  // as the cylinder example builds them (symbolic factorization in the
  // TACSSchurPc constructor, outside the timed solve)
  TACSSchurMat *kmat = assembler->createSchurMat();
  TACSSchurMat *gmat = assembler->createSchurMat();
  TACSSchurMat *aux = assembler->createSchurMat();
  kmat->incref();
  gmat->incref();
  aux->incref();
  auto ts = std::chrono::steady_clock::now();
  TACSSchurPc *pc = new TACSSchurPc(kmat, lev, 10.0, 1);
  pc->incref();
  const double setup_s =
      std::chrono::duration<double>(std::chrono::steady_clock::now() - ts).count();
  GMRES *solver = new GMRES(aux, pc, gm_m, gm_restarts, 0);
  solver->incref();
  solver->setTolerances(gm_tol, gm_tol);
  CountingPrint *count = new CountingPrint();
  count->incref();
  count->echo = verbose;
  solver->setMonitor(count);
  TACSLinearBuckling *buck = new TACSLinearBuckling(assembler, sigma, gmat, kmat, aux, solver,
                                                    max_lanczos, neig, eig_tol);
  buck->incref();
  TACSBVec *f = assembler->createVec();
  f->incref();
  TacsScalar *fa;
  f->getArray(&fa);
  for (int i = 0; i < 6 * nn; i++) fa[i] = rhs[i];

  // With more than one thread, TACSAssembler::assembleRes runs
  // assembleRes_thread, which adds into the residual pointer of the shared
  // thread record (src/TACSAssembler_thread.cpp:52, 91), but assembleRes
  // never stores its argument there (src/TACSAssembler.cpp:4000-4012, unlike
  // assembleJacobian at :4099): the first threaded call dereferences an unset
  // pointer.  One threaded assembleJacobian beforehand leaves a live vector
  // in that record; solve() calls assembleRes only at the zero state, where
  // every element residual is zero, so the results are unchanged.
  TACSBVec *prime = assembler->createVec();
  prime->incref();
  if (threads > 1) assembler->assembleJacobian(1.0, 0.0, 0.0, prime, kmat);

  auto t0 = std::chrono::steady_clock::now();
  buck->solve(f, NULL, verbose ? count : NULL);
  const double secs =
      std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();

  printf("{\"threads\": %d, \"seconds\": %.6f, \"setup_s\": %.6f, \"gmres_iterations\": %ld, "
         "\"gmres_cycles\": %ld, \"nodes\": %d, \"elements\": %d, \"eigvals\": [",
         threads, secs, setup_s, count->iterations, count->cycles, nn, ne);
  for (int k = 0; k < nreport; k++) {
    TacsScalar err;
    TacsScalar lam = buck->extractEigenvalue(k, &err);
    printf("%s%.17g", k ? ", " : "", TacsRealPart(lam));
  }
  printf("], \"errors\": [");
  for (int k = 0; k < nreport; k++) {
    TacsScalar err;
    buck->extractEigenvalue(k, &err);
    printf("%s%.3e", k ? ", " : "", TacsRealPart(err));
  }
  printf("]}\n");
  fflush(stdout);
  return 0;
}
