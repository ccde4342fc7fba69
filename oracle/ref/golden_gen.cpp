/*
  Fixture generator: drives the reference implementation (compiled from the
  reference's own sources by oracle/ref/Makefile) and writes its outputs as
  .npy files.  Test infrastructure only; run by tests/golden/make_golden.py.

    golden_gen element  <out_dir>            element-level K, G, residual, J
    golden_gen assembly <in_dir> <out_dir>   assembled K/G, orderings, ILU,
                                             path and buckling eigenpairs

  The complex build (-DTACS_USE_COMPLEX) writes the same files with the
  suffix "_cs"; its G is the complex-step geometric stiffness
  (TACSShellElement.h:693-698, 754-762 in the reference).
*/
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <string>
#include <vector>

#include "AMDInterface.h"
#include "GSEP.h"
#include "KSM.h"
#include "TACSAssembler.h"
#include "TACSBuckling.h"
#include "TACSIsoShellConstitutive.h"
#include "TACSMaterialProperties.h"
#include "TACSSchurMat.h"
#include "TACSShellElementDefs.h"
#include "TACSShellElementTransform.h"
#include "TACSMeshLoader.h"
#include "TACSToFH5.h"
#include "TacsUtilities.h"

#ifdef TACS_USE_COMPLEX
static const char *SUFFIX = "_cs";
#else
static const char *SUFFIX = "";
#endif

#include "npy_io.h"

static void save_d(const std::string &dir, const std::string &name,
                   const TacsScalar *v, const std::vector<long> &shape) {
  size_t n = 1;
  for (long s : shape) n *= (size_t)s;
  std::vector<double> d(n);
  for (size_t i = 0; i < n; i++) d[i] = TacsRealPart(v[i]);
  write_npy(dir + "/" + name + SUFFIX + ".npy", "<f8", d.data(), 8, shape);
}

static void save_i(const std::string &dir, const std::string &name,
                   const int *v, const std::vector<long> &shape) {
  write_npy(dir + "/" + name + SUFFIX + ".npy", "<i4", v, 4, shape);
}

/* ------------------------------------------------------------- seeded rng */
struct SplitMix {
  uint64_t s;
  explicit SplitMix(uint64_t seed) : s(seed) {}
  uint64_t next() {
    uint64_t z = (s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
  }
  double uniform(double a, double b) {
    return a + (b - a) * ((next() >> 11) * (1.0 / 9007199254740992.0));
  }
};

/* ------------------------------------------------------- element fixtures */
static TACSElement *make_element(const char *name, TACSShellTransform *tr,
                                 TACSShellConstitutive *con) {
  return TacsCreateShellByName(name, tr, con);
}

/* A curved, skewed element patch of size h with the given node count per
   direction; nodes in tensor order (i fastest). */
static void element_geometry(SplitMix &rng, int order, double h, TacsScalar *X) {
  double R[9];
  // Random rotation from three random angles
  double a = rng.uniform(0, 6.283185307179586), b = rng.uniform(-1.2, 1.2),
         c = rng.uniform(0, 6.283185307179586);
  double ca = cos(a), sa = sin(a), cb = cos(b), sb = sin(b), cc = cos(c), sc = sin(c);
  double Rz1[9] = {ca, -sa, 0, sa, ca, 0, 0, 0, 1};
  double Ry[9] = {cb, 0, sb, 0, 1, 0, -sb, 0, cb};
  double Rz2[9] = {cc, -sc, 0, sc, cc, 0, 0, 0, 1};
  double T1[9];
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) {
      T1[3 * i + j] = 0;
      for (int k = 0; k < 3; k++) T1[3 * i + j] += Rz1[3 * i + k] * Ry[3 * k + j];
    }
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) {
      R[3 * i + j] = 0;
      for (int k = 0; k < 3; k++) R[3 * i + j] += T1[3 * i + k] * Rz2[3 * k + j];
    }
  double kx = rng.uniform(-1.0, 1.0) / h, ky = rng.uniform(-1.0, 1.0) / h;
  double skew = rng.uniform(-0.2, 0.2);
  double off[3] = {rng.uniform(-1, 1), rng.uniform(-1, 1), rng.uniform(-1, 1)};
  for (int j = 0; j < order; j++) {
    for (int i = 0; i < order; i++) {
      double u = h * (double)i / (order - 1), v = h * (double)j / (order - 1);
      u += skew * v;
      u += 0.08 * h * rng.uniform(-1, 1);
      v += 0.08 * h * rng.uniform(-1, 1);
      double w = 0.05 * (kx * u * u + ky * v * v) + 0.01 * h * rng.uniform(-1, 1);
      double p[3] = {u, v, w};
      for (int d = 0; d < 3; d++) {
        double s = off[d];
        for (int k = 0; k < 3; k++) s += R[3 * d + k] * p[k];
        X[3 * (i + order * j) + d] = s;
      }
    }
  }
}

static void run_elements(const std::string &out) {
  const char *names[4] = {"TACSQuad4Shell", "TACSQuad4NonlinearShell",
                          "TACSQuad9Shell", "TACSQuad9NonlinearShell"};
  const int orders[4] = {2, 2, 3, 3};
  const int nsamples = 6;
  TACSShellTransform *tr = new TACSShellNaturalTransform();
  tr->incref();
  for (int e = 0; e < 4; e++) {
    const int order = orders[e];
    const int nn = order * order;
    const int nv = 6 * nn;
    SplitMix rng(20261203ull + 7919ull * (uint64_t)e);
    std::vector<TacsScalar> Xall, Vall, Kall, Gall, Rall, Jall, JRall, params;
    std::vector<TacsScalar> PSall, PHall, KXall, GXall, KUall, GUall, RXall, KDall, GDall;
    SplitMix rng_x(977ull + 31ull * (uint64_t)e);  // psi, phi of the coordinate products
    for (int s = 0; s < nsamples; s++) {
      double h = rng.uniform(0.02, 0.6);
      double t = rng.uniform(1e-3, 2e-2);
      double E = rng.uniform(50e9, 210e9), nu = rng.uniform(0.2, 0.35);
      double alpha = 2.3e-5;
      double temp = (s == nsamples - 1) ? 25.0 : 0.0;
      std::vector<TacsScalar> X(3 * nn), vars(nv);
      element_geometry(rng, order, h, X.data());
      for (int i = 0; i < nn; i++) {
        for (int k = 0; k < 3; k++) vars[6 * i + k] = 1e-2 * h * rng.uniform(-1, 1);
        for (int k = 3; k < 6; k++) vars[6 * i + k] = 1e-2 * rng.uniform(-1, 1);
      }
      TACSMaterialProperties *props =
          new TACSMaterialProperties(2700.0, 921.0, E, nu, 270e6, alpha, 230.0);
      TACSIsoShellConstitutive *con = new TACSIsoShellConstitutive(props, t, 0);
      TACSElement *elem = make_element(names[e], tr, con);
      elem->incref();
      // setTemperature is not virtual: cast to the concrete instantiation.
      if (e == 0) ((TACSQuad4Shell *)elem)->setTemperature(temp);
      if (e == 1) ((TACSQuad4NonlinearShell *)elem)->setTemperature(temp);
      if (e == 2) ((TACSQuad9Shell *)elem)->setTemperature(temp);
      if (e == 3) ((TACSQuad9NonlinearShell *)elem)->setTemperature(temp);
#ifdef TACS_USE_COMPLEX
      if (e == 0) ((TACSQuad4Shell *)elem)->setComplexStepGmatrix(true);
      if (e == 1) ((TACSQuad4NonlinearShell *)elem)->setComplexStepGmatrix(true);
      if (e == 2) ((TACSQuad9Shell *)elem)->setComplexStepGmatrix(true);
      if (e == 3) ((TACSQuad9NonlinearShell *)elem)->setComplexStepGmatrix(true);
#endif
      std::vector<TacsScalar> K(nv * nv), G(nv * nv), R(nv, 0.0), J(nv * nv, 0.0),
          JR(nv, 0.0), zero(nv, 0.0);
      // G last: for the nonlinear instantiations getMatType(G) leaves the
      // element's own temperature perturbed (nlElem == this,
      // TACSShellElement.h:735-751), which would leak into later calls.
      elem->getMatType(TACS_STIFFNESS_MATRIX, 0, 0.0, X.data(), vars.data(), K.data());
      elem->addResidual(0, 0.0, X.data(), vars.data(), zero.data(), zero.data(), R.data());
      elem->addJacobian(0, 0.0, 1.0, 0.0, 0.0, X.data(), vars.data(), zero.data(),
                        zero.data(), JR.data(), J.data());
      elem->getMatType(TACS_GEOMETRIC_STIFFNESS_MATRIX, 0, 0.0, X.data(), vars.data(),
                       G.data());
      // Coordinate inner products d(psi^T M phi)/dX of K and G
      // (TACSElement::addMatXptSensInnerProduct, TACSElement.cpp:434-507:
      // central differences with dh = 1e-7 in the real build, complex step
      // in the complex build, where G is then the real-step central
      // difference).  Zero-temperature samples only: every G evaluation of
      // a nonlinear instantiation leaves its temperature stepped.
      std::vector<TacsScalar> psi(nv), phi(nv), KX(3 * nn, 0.0), GX(3 * nn, 0.0);
      std::vector<TacsScalar> KU(nv, 0.0), GU(nv, 0.0), RX(3 * nn, 0.0);
      for (int i = 0; i < nv; i++) {
        psi[i] = rng_x.uniform(-1, 1);
        phi[i] = rng_x.uniform(-1, 1);
      }
      if (temp == 0.0) {
#ifdef TACS_USE_COMPLEX
        if (e == 0) ((TACSQuad4Shell *)elem)->setComplexStepGmatrix(false);
        if (e == 1) ((TACSQuad4NonlinearShell *)elem)->setComplexStepGmatrix(false);
        if (e == 2) ((TACSQuad9Shell *)elem)->setComplexStepGmatrix(false);
        if (e == 3) ((TACSQuad9NonlinearShell *)elem)->setComplexStepGmatrix(false);
#endif
        elem->addMatXptSensInnerProduct(TACS_STIFFNESS_MATRIX, 0, 0.0, 1.0, psi.data(),
                                        phi.data(), X.data(), vars.data(), KX.data());
        elem->addMatXptSensInnerProduct(TACS_GEOMETRIC_STIFFNESS_MATRIX, 0, 0.0, 1.0,
                                        psi.data(), phi.data(), X.data(), vars.data(),
                                        GX.data());
        // state derivatives (getMatSVSensInnerProduct, :509-581) and the
        // adjoint-residual coordinate product (addAdjResXptProduct, :270)
        elem->getMatSVSensInnerProduct(TACS_STIFFNESS_MATRIX, 0, 0.0, psi.data(), phi.data(),
                                       X.data(), vars.data(), KU.data());
        elem->getMatSVSensInnerProduct(TACS_GEOMETRIC_STIFFNESS_MATRIX, 0, 0.0, psi.data(),
                                       phi.data(), X.data(), vars.data(), GU.data());
        elem->addAdjResXptProduct(0, 0.0, 1.0, psi.data(), X.data(), vars.data(), zero.data(),
                                  zero.data(), RX.data());
      }
      // Thickness inner products d(psi^T M phi)/dt of K and G
      // (TACSElement::addMatDVSensInnerProduct, TACSElement.cpp:355-432: the
      // element's one design variable, central differences with dh = 1e-7
      // in the real build, complex step in the complex build); last, since
      // the G evaluations of a nonlinear instantiation move its temperature
      TacsScalar kd = 0.0, gd = 0.0;
      if (temp == 0.0) {
        elem->addMatDVSensInnerProduct(TACS_STIFFNESS_MATRIX, 0, 0.0, 1.0, psi.data(),
                                       phi.data(), X.data(), vars.data(), 1, &kd);
        elem->addMatDVSensInnerProduct(TACS_GEOMETRIC_STIFFNESS_MATRIX, 0, 0.0, 1.0, psi.data(),
                                       phi.data(), X.data(), vars.data(), 1, &gd);
      }
      KDall.push_back(kd);
      GDall.push_back(gd);
      KUall.insert(KUall.end(), KU.begin(), KU.end());
      GUall.insert(GUall.end(), GU.begin(), GU.end());
      RXall.insert(RXall.end(), RX.begin(), RX.end());
      PSall.insert(PSall.end(), psi.begin(), psi.end());
      PHall.insert(PHall.end(), phi.begin(), phi.end());
      KXall.insert(KXall.end(), KX.begin(), KX.end());
      GXall.insert(GXall.end(), GX.begin(), GX.end());
      Xall.insert(Xall.end(), X.begin(), X.end());
      Vall.insert(Vall.end(), vars.begin(), vars.end());
      Kall.insert(Kall.end(), K.begin(), K.end());
      Gall.insert(Gall.end(), G.begin(), G.end());
      Rall.insert(Rall.end(), R.begin(), R.end());
      Jall.insert(Jall.end(), J.begin(), J.end());
      JRall.insert(JRall.end(), JR.begin(), JR.end());
      TacsScalar p[6] = {E, nu, t, alpha, temp, h};
      params.insert(params.end(), p, p + 6);
      elem->decref();
    }
    std::string pre = std::string(names[e]) + "_";
    save_d(out, pre + "X", Xall.data(), {nsamples, nn, 3});
    save_d(out, pre + "vars", Vall.data(), {nsamples, nv});
    save_d(out, pre + "params", params.data(), {nsamples, 6});
    save_d(out, pre + "K", Kall.data(), {nsamples, nv, nv});
    save_d(out, pre + "G", Gall.data(), {nsamples, nv, nv});
    save_d(out, pre + "res", Rall.data(), {nsamples, nv});
    save_d(out, pre + "J", Jall.data(), {nsamples, nv, nv});
    save_d(out, pre + "Jres", JRall.data(), {nsamples, nv});
    save_d(out, pre + "xs_psi", PSall.data(), {nsamples, nv});
    save_d(out, pre + "xs_phi", PHall.data(), {nsamples, nv});
    save_d(out, pre + "KX", KXall.data(), {nsamples, nn, 3});
    save_d(out, pre + "GX", GXall.data(), {nsamples, nn, 3});
    save_d(out, pre + "KU", KUall.data(), {nsamples, nv});
    save_d(out, pre + "GU", GUall.data(), {nsamples, nv});
    save_d(out, pre + "RX", RXall.data(), {nsamples, nn, 3});
    save_d(out, pre + "KD", KDall.data(), {nsamples});
    save_d(out, pre + "GD", GDall.data(), {nsamples});
  }
  tr->decref();
}

/* ------------------------------------------------------ assembly fixtures */
static void run_assembly(const std::string &in, const std::string &out) {
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
  const double E = prm[0], nu = prm[1], sigma = prm[2];
  const int lev = (int)prm[3], gm_m = (int)prm[4], gm_restarts = (int)prm[5];
  const int max_lanczos = (int)prm[6], neig = (int)prm[7];
  const int nonlinear = (int)prm[8];
  const double gm_tol = prm[9], temperature = prm[10], alpha_t = prm[11];

  const char *name = NULL;
  if (npe == 4) name = nonlinear ? "TACSQuad4NonlinearShell" : "TACSQuad4Shell";
  if (npe == 9) name = nonlinear ? "TACSQuad9NonlinearShell" : "TACSQuad9Shell";
  if (!name) {
    fprintf(stderr, "unsupported element size %d\n", npe);
    exit(1);
  }

  TACSShellTransform *tr = new TACSShellNaturalTransform();
  tr->incref();
  TACSMaterialProperties *props =
      new TACSMaterialProperties(2700.0, 921.0, E, nu, 270e6, alpha_t, 230.0);
  props->incref();

  // One constitutive object (and element object) per distinct thickness
  // value, as a component-per-thickness model would build them.
  std::vector<TACSElement *> elems(ne);
  std::vector<double> tvals;
  std::vector<TACSElement *> tobjs;
  for (int e = 0; e < ne; e++) {
    int k = -1;
    for (size_t j = 0; j < tvals.size(); j++)
      if (tvals[j] == thick[e]) k = (int)j;
    if (k < 0) {
      TACSIsoShellConstitutive *con =
          new TACSIsoShellConstitutive(props, thick[e], (int)tvals.size());
      TACSElement *el = make_element(name, tr, con);
      el->incref();
      tvals.push_back(thick[e]);
      tobjs.push_back(el);
      k = (int)tvals.size() - 1;
    }
    elems[e] = tobjs[k];
  }
  for (TACSElement *el : tobjs) {
    if (npe == 4 && !nonlinear) ((TACSQuad4Shell *)el)->setTemperature(temperature);
    if (npe == 4 && nonlinear) ((TACSQuad4NonlinearShell *)el)->setTemperature(temperature);
    if (npe == 9 && !nonlinear) ((TACSQuad9Shell *)el)->setTemperature(temperature);
    if (npe == 9 && nonlinear) ((TACSQuad9NonlinearShell *)el)->setTemperature(temperature);
#ifdef TACS_USE_COMPLEX
    if (npe == 4 && !nonlinear) ((TACSQuad4Shell *)el)->setComplexStepGmatrix(true);
    if (npe == 4 && nonlinear) ((TACSQuad4NonlinearShell *)el)->setComplexStepGmatrix(true);
    if (npe == 9 && !nonlinear) ((TACSQuad9Shell *)el)->setComplexStepGmatrix(true);
    if (npe == 9 && nonlinear) ((TACSQuad9NonlinearShell *)el)->setComplexStepGmatrix(true);
#endif
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
    for (int k = 0; k < 6; k++) {
      if (bc_mask[b] & (1 << k)) {
        vals[nv] = bc_vals[6 * b + k];
        vars[nv++] = k;
      }
    }
    assembler->addBCs(1, &bc_nodes[b], nv, vars, vals);
  }
  assembler->initialize();
  TACSBVec *Xvec = assembler->createNodeVec();
  Xvec->incref();
  TacsScalar *xa;
  Xvec->getArray(&xa);
  for (int i = 0; i < 3 * nn; i++) xa[i] = X[i];
  assembler->setNodes(Xvec);

  // Node-to-node CSR (with and without the diagonal)
  int *rowp, *cols;
  assembler->computeLocalNodeToNodeCSR(&rowp, &cols, 0);
  save_i(out, "csr_rowp", rowp, {nn + 1});
  save_i(out, "csr_cols", cols, {rowp[nn]});
  delete[] rowp;
  delete[] cols;
  assembler->computeLocalNodeToNodeCSR(&rowp, &cols, 1);
  {
    std::vector<int> perm(nn);
    amd_order_interface(nn, rowp, cols, perm.data(), NULL, 0, 0, NULL, NULL, NULL, 0);
    save_i(out, "amd_perm", perm.data(), {nn});
  }
  delete[] rowp;
  delete[] cols;

  TACSSchurMat *kmat = assembler->createSchurMat();
  TACSSchurMat *gmat = assembler->createSchurMat();
  TACSSchurMat *aux = assembler->createSchurMat();
  kmat->incref();
  gmat->incref();
  aux->incref();

  // Assembled stiffness at the zero state (with BC rows applied)
  assembler->zeroVariables();
  assembler->assembleMatType(TACS_STIFFNESS_MATRIX, kmat);
  BCSRMat *B, *Em, *Fm, *Cm;
  kmat->getBCSRMat(&B, &Em, &Fm, &Cm);
  int bsize, nrows, ncols;
  const int *browp, *bcols;
  TacsScalar *bA;
  B->getArrays(&bsize, &nrows, &ncols, &browp, &bcols, &bA);
  save_i(out, "bcsr_rowp", browp, {nrows + 1});
  save_i(out, "bcsr_cols", bcols, {browp[nrows]});
  save_d(out, "K", bA, {browp[nrows], 6, 6});

  // ILU(lev) pattern and numeric factor of K
  {
    BCSRMat *fac = new BCSRMat(MPI_COMM_WORLD, B, lev, 10.0);
    fac->incref();
    fac->copyValues(B);
    fac->factor();
    const int *frowp, *fcols;
    TacsScalar *fA;
    int fb, fnr, fnc;
    fac->getArrays(&fb, &fnr, &fnc, &frowp, &fcols, &fA);
    save_i(out, "ilu_rowp", frowp, {fnr + 1});
    save_i(out, "ilu_cols", fcols, {frowp[fnr]});
    save_d(out, "ilu_K", fA, {frowp[fnr], 6, 6});
    // Apply the factor to a fixed vector (x_i = sin(i+1))
    std::vector<TacsScalar> xv(6 * nrows), yv(6 * nrows), yv2(6 * nrows);
    for (int i = 0; i < 6 * nrows; i++) xv[i] = sin(1.0 + i);
    fac->applyFactor(xv.data(), yv.data());
    save_d(out, "ilu_apply_x", xv.data(), {6 * nrows});
    save_d(out, "ilu_apply_y", yv.data(), {6 * nrows});
    B->mult(xv.data(), yv2.data());
    save_d(out, "K_mult_y", yv2.data(), {6 * nrows});
    fac->decref();
  }

  // Buckling solve exactly as the cylinder example drives it
  TACSSchurPc *pc = new TACSSchurPc(kmat, lev, 10.0, 1);
  pc->incref();
  GMRES *solver = new GMRES(aux, pc, gm_m, gm_restarts, 0);
  solver->incref();
  solver->setTolerances(gm_tol, gm_tol);
  TACSLinearBuckling *buck = new TACSLinearBuckling(assembler, sigma, gmat, kmat, aux,
                                                    solver, max_lanczos, neig, 1e-12);
  buck->incref();
  TACSBVec *f = assembler->createVec();
  f->incref();
  TacsScalar *fa;
  f->getArray(&fa);
  for (int i = 0; i < 6 * nn; i++) fa[i] = rhs[i];
  buck->solve(f, NULL, NULL);

  // Path = the variables the assembler holds after solve()
  TACSBVec *path = assembler->createVec();
  path->incref();
  assembler->getVariables(path);
  TacsScalar *pa;
  path->getArray(&pa);
  save_d(out, "path", pa, {nn, 6});

  gmat->getBCSRMat(&B, &Em, &Fm, &Cm);
  B->getArrays(&bsize, &nrows, &ncols, &browp, &bcols, &bA);
  save_d(out, "G", bA, {browp[nrows], 6, 6});
  kmat->getBCSRMat(&B, &Em, &Fm, &Cm);
  B->getArrays(&bsize, &nrows, &ncols, &browp, &bcols, &bA);
  save_d(out, "K_after", bA, {browp[nrows], 6, 6});

  std::vector<TacsScalar> lam(neig), err(neig), vecs((size_t)neig * 6 * nn);
  TACSBVec *phi = assembler->createVec();
  phi->incref();
  for (int k = 0; k < neig; k++) {
    TacsScalar e;
    lam[k] = buck->extractEigenvector(k, phi, &e);
    err[k] = e;
    TacsScalar *ph;
    phi->getArray(&ph);
    memcpy(&vecs[(size_t)k * 6 * nn], ph, sizeof(TacsScalar) * 6 * nn);
  }
  save_d(out, "eigvals", lam.data(), {neig});
  save_d(out, "eigerr", err.data(), {neig});
  save_d(out, "eigvecs", vecs.data(), {neig, nn, 6});

  // Residual at the path state
  TACSBVec *res = assembler->createVec();
  res->incref();
  assembler->setVariables(path);
  assembler->assembleRes(res);
  TacsScalar *ra;
  res->getArray(&ra);
  save_d(out, "res_path", ra, {nn, 6});
  printf("assembly fixture: nn=%d ne=%d nnzb=%d\n", nn, ne, browp[nrows]);
}

// Orderings of the node graph (TACSAssembler::computeMatReordering,
// src/TACSAssembler.cpp:1508-1600): RCM from root 0 with one pass and the
// serial greedy multicolouring, on the node-to-node CSR with the diagonal.
static void run_orderings(const std::string &in, const std::string &out) {
  std::vector<long> xs, cs;
  std::vector<double> X = read_npy<double>(in + "/X.npy", &xs);
  std::vector<int> conn = read_npy<int>(in + "/conn.npy", &cs);
  const int nn = (int)xs[0], ne = (int)cs[0], npe = (int)cs[1];
  TACSShellTransform *tr = new TACSShellNaturalTransform();
  tr->incref();
  TACSMaterialProperties *props =
      new TACSMaterialProperties(2700.0, 921.0, 70e9, 0.3, 270e6, 0.0, 230.0);
  props->incref();
  TACSIsoShellConstitutive *con = new TACSIsoShellConstitutive(props, 1e-2, 0);
  TACSElement *el = make_element(npe == 4 ? "TACSQuad4Shell" : "TACSQuad9Shell", tr, con);
  el->incref();
  std::vector<TACSElement *> elems(ne, el);
  TACSAssembler *assembler = new TACSAssembler(MPI_COMM_WORLD, 6, nn, ne);
  assembler->incref();
  std::vector<int> ptr(ne + 1);
  for (int e = 0; e <= ne; e++) ptr[e] = npe * e;
  assembler->setElementConnectivity(ptr.data(), conn.data());
  assembler->setElements(elems.data());
  assembler->initialize();
  int *rowp, *cols;
  assembler->computeLocalNodeToNodeCSR(&rowp, &cols, 0);
  std::vector<int> rcm(nn), colors(nn), mc(nn);
  TacsComputeRCMOrder(nn, rowp, cols, rcm.data(), 0, 1);
  int ncolors = TacsComputeSerialMultiColor(nn, rowp, cols, colors.data(), mc.data());
  save_i(out, "rcm_new_vars", rcm.data(), {nn});
  save_i(out, "mc_colors", colors.data(), {nn});
  save_i(out, "mc_new_vars", mc.data(), {nn});
  save_i(out, "mc_ncolors", &ncolors, {1});
  delete[] rowp;
  delete[] cols;
  assembler->decref();
}

// The reference's BDF loader (TACSMeshLoader::scanBDFFile,
// src/io/TACSMeshLoader.cpp:569-1098) on one file: connectivity, nodes,
// SPC entries and the per-component names, as the loader returns them.
static void run_bdf(const std::string &file, const std::string &out) {
  TACSMeshLoader *loader = new TACSMeshLoader(MPI_COMM_WORLD);
  loader->incref();
  const int fail = loader->scanBDFFile(file.c_str());
  int nn = 0, ne = 0, nbcs = 0;
  const int *ptr, *conn, *comp, *bc_nodes, *bc_vars, *bc_ptr;
  const TacsScalar *X, *bc_vals;
  loader->getConnectivity(&nn, &ne, &ptr, &conn, &comp, &X);
  loader->getBCs(&nbcs, &bc_nodes, &bc_vars, &bc_ptr, &bc_vals);
  const int ncomp = loader->getNumComponents();
  int sizes[5] = {fail, nn, ne, nbcs, ncomp};
  save_i(out, "sizes", sizes, {5});
  save_i(out, "elem_node_ptr", ptr, {ne + 1});
  save_i(out, "elem_node_conn", conn, {ptr[ne]});
  save_i(out, "elem_component", comp, {ne});
  save_d(out, "Xpts", X, {nn, 3});
  save_i(out, "bc_nodes", bc_nodes, {nbcs});
  save_i(out, "bc_ptr", bc_ptr, {nbcs + 1});
  save_i(out, "bc_vars", bc_vars, {bc_ptr[nbcs]});
  save_d(out, "bc_vals", bc_vals, {bc_ptr[nbcs]});
  // component names, NUL-padded to 40 characters each
  std::vector<char> names((size_t)2 * ncomp * 40, 0);
  for (int c = 0; c < ncomp; c++) {
    strncpy(&names[(size_t)c * 40], loader->getElementDescript(c), 39);
    strncpy(&names[(size_t)(ncomp + c) * 40], loader->getComponentDescript(c), 39);
  }
  write_npy(out + "/names" + SUFFIX + ".npy", "|u1", names.data(), 1, {2 * ncomp, 40});
  printf("bdf fixture: nn=%d ne=%d nbcs=%d ncomp=%d\n", nn, ne, nbcs, ncomp);
  loader->decref();
}

// TACSToFH5::writeToFile (src/io/TACSToFH5.cpp:126) for a shell mesh with
// per-element components, named components 0 and 1, the given variables
// and each of nine output-class flags: in/X, conn, comp, vars ->
// out/f5_<flag>.f5.
static void run_f5(const std::string &in, const std::string &out) {
  std::vector<long> xs, cs;
  std::vector<double> X = read_npy<double>(in + "/X.npy", &xs);
  std::vector<int> conn = read_npy<int>(in + "/conn.npy", &cs);
  std::vector<int> comp = read_npy<int>(in + "/comp.npy");
  std::vector<double> vars = read_npy<double>(in + "/vars.npy");
  const int nn = (int)xs[0], ne = (int)cs[0], npe = (int)cs[1];
  int ncomp = 0;
  for (int e = 0; e < ne; e++) ncomp = comp[e] + 1 > ncomp ? comp[e] + 1 : ncomp;
  TACSShellTransform *tr = new TACSShellNaturalTransform();
  tr->incref();
  TACSMaterialProperties *props =
      new TACSMaterialProperties(2700.0, 921.0, 70e9, 0.3, 270e6, 0.0, 230.0);
  props->incref();
  std::vector<TACSElement *> per_comp(ncomp);
  for (int c = 0; c < ncomp; c++) {
    TACSIsoShellConstitutive *con = new TACSIsoShellConstitutive(props, 1e-2, c);
    per_comp[c] = make_element(npe == 4 ? "TACSQuad4Shell" : "TACSQuad9Shell", tr, con);
    per_comp[c]->incref();
    per_comp[c]->setComponentNum(c);
  }
  std::vector<TACSElement *> elems(ne);
  for (int e = 0; e < ne; e++) elems[e] = per_comp[comp[e]];
  TACSAssembler *assembler = new TACSAssembler(MPI_COMM_WORLD, 6, nn, ne);
  assembler->incref();
  std::vector<int> ptr(ne + 1);
  for (int e = 0; e <= ne; e++) ptr[e] = npe * e;
  assembler->setElementConnectivity(ptr.data(), conn.data());
  assembler->setElements(elems.data());
  assembler->initialize();
  TACSBVec *Xv = assembler->createNodeVec();
  Xv->incref();
  TacsScalar *xa;
  Xv->getArray(&xa);
  for (int i = 0; i < 3 * nn; i++) xa[i] = X[i];
  assembler->setNodes(Xv);
  TACSBVec *q = assembler->createVec();
  q->incref();
  TacsScalar *qa;
  q->getArray(&qa);
  for (int i = 0; i < 6 * nn; i++) qa[i] = vars[i];
  assembler->setVariables(q);
  const int all = TACS_OUTPUT_CONNECTIVITY | TACS_OUTPUT_NODES | TACS_OUTPUT_DISPLACEMENTS |
                  TACS_OUTPUT_STRAINS | TACS_OUTPUT_STRESSES | TACS_OUTPUT_EXTRAS |
                  TACS_OUTPUT_LOADS;
  const int flags[9] = {TACS_OUTPUT_CONNECTIVITY | TACS_OUTPUT_NODES | TACS_OUTPUT_DISPLACEMENTS,
                        TACS_OUTPUT_NODES, TACS_OUTPUT_DISPLACEMENTS, TACS_OUTPUT_CONNECTIVITY,
                        TACS_OUTPUT_LOADS,
                        TACS_OUTPUT_CONNECTIVITY | TACS_OUTPUT_NODES | TACS_OUTPUT_DISPLACEMENTS |
                            TACS_OUTPUT_LOADS,
                        TACS_OUTPUT_STRAINS | TACS_OUTPUT_STRESSES, TACS_OUTPUT_EXTRAS, all};
  for (int f = 0; f < 9; f++) {
    TACSToFH5 *f5 = new TACSToFH5(assembler, TACS_BEAM_OR_SHELL_ELEMENT, flags[f]);
    f5->incref();
    f5->setComponentName(0, "skin");
    if (ncomp > 1) f5->setComponentName(1, "stiffener panel");
    const std::string path = out + "/f5_" + std::to_string(flags[f]) + ".f5";
    remove(path.c_str());
    f5->writeToFile(path.c_str());
    f5->decref();
  }
  printf("f5 fixture: nn=%d ne=%d ncomp=%d\n", nn, ne, ncomp);
  assembler->decref();
}

int main(int argc, char **argv) {
  MPI_Init(&argc, &argv);
  TacsInitialize();
  if (argc >= 3 && strcmp(argv[1], "element") == 0) {
    run_elements(argv[2]);
  } else if (argc >= 4 && strcmp(argv[1], "orderings") == 0) {
    run_orderings(argv[2], argv[3]);
  } else if (argc >= 4 && strcmp(argv[1], "assembly") == 0) {
    run_assembly(argv[2], argv[3]);
  } else if (argc >= 4 && strcmp(argv[1], "bdf") == 0) {
    run_bdf(argv[2], argv[3]);
  } else if (argc >= 4 && strcmp(argv[1], "f5") == 0) {
    run_f5(argv[2], argv[3]);
  } else {
    fprintf(stderr, "usage: golden_gen element <out> | assembly <in> <out>\n");
    return 2;
  }
  TacsFinalize();
  MPI_Finalize();
  return 0;
}
