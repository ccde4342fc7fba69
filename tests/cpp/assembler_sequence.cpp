// The reference's own construction sequence of an assembler
// (TACSAssembler(comm, 6, numOwnedNodes, numElements), setElementConnectivity,
// setElements, addBCs, initialize, createNodeVec + setNodes) and the
// BCSRMat / checkEigenvector / assembleJacobian(alpha) calls of the
// reference's surface, through include/a2ds_tacs.hpp.
//
// usage: assembler_sequence dir sigma num_eigvals
//   dir holds raw little-endian arrays written by the test: sizes.i32
//   (num_nodes, num_elements, nodes_per_elem, num_bcs, E, nu bits as
//   doubles follow in params.f64), X.f64, conn.i32, bc_nodes.i32,
//   rhs.f64, params.f64 (E, nu, t)
// prints: "eig k lambda residual" lines, "check rel" (checkEigenvector),
//   "apply rel" (||B y - x|| / ||x|| with y = (LU)^-1 x through BCSRMat),
//   "jac rel" (alpha = 2 Jacobian against 2 K off the Dirichlet rows)
#include <math.h>
#include <stdio.h>
#include <stdlib.h>

#include <string>
#include <vector>

#include "a2ds_tacs.hpp"

using namespace a2ds_tacs;

template <typename T>
static std::vector<T> read_raw(const std::string &path) {
  std::vector<T> v;
  FILE *fp = fopen(path.c_str(), "rb");
  if (!fp) return v;
  fseek(fp, 0, SEEK_END);
  long n = ftell(fp);
  fseek(fp, 0, SEEK_SET);
  v.resize((size_t)n / sizeof(T));
  if (fread(v.data(), sizeof(T), v.size(), fp) != v.size()) v.clear();
  fclose(fp);
  return v;
}

int main(int argc, char **argv) {
  if (argc < 4) {
    fprintf(stderr, "usage: %s dir sigma num_eigvals\n", argv[0]);
    return 2;
  }
  const std::string dir = argv[1];
  const double sigma = atof(argv[2]);
  const int nev = atoi(argv[3]);
  std::vector<int> sz = read_raw<int>(dir + "/sizes.i32");
  std::vector<double> X = read_raw<double>(dir + "/X.f64");
  std::vector<int> conn = read_raw<int>(dir + "/conn.i32");
  std::vector<int> bcn = read_raw<int>(dir + "/bc_nodes.i32");
  std::vector<double> rhs = read_raw<double>(dir + "/rhs.f64");
  std::vector<double> prm = read_raw<double>(dir + "/params.f64");
  if (sz.size() != 4 || prm.size() != 3) return 1;
  const int nn = sz[0], ne = sz[1], npe = sz[2], nbc = sz[3];

  TACSShellTransform *transform = new TACSShellNaturalTransform();
  TACSMaterialProperties *mat =
      new TACSMaterialProperties(2700.0, 921.0, prm[0], prm[1], 270e6, 0.0, 230.0);
  TACSIsoShellConstitutive *con = new TACSIsoShellConstitutive(mat, prm[2]);
  TACSElement *shell = new TACSQuad4Shell(transform, con);
  shell->incref();
  std::vector<TACSElement *> elems(ne, shell);
  std::vector<int> ptr(ne + 1);
  for (int e = 0; e <= ne; e++) ptr[e] = npe * e;

  // the reference's sequence
  TACSAssembler *assembler = new TACSAssembler(MPI_COMM_WORLD, 6, nn, ne);
  assembler->incref();
  if (assembler->setElementConnectivity(ptr.data(), conn.data())) return 1;
  if (assembler->setElements(elems.data())) return 1;
  if (assembler->addBCs(nbc, bcn.data())) return 1;
  TACSBVec *Xvec = assembler->createNodeVec();
  Xvec->incref();
  TacsScalar *xa;
  Xvec->getArray(&xa);
  for (int i = 0; i < 3 * nn; i++) xa[i] = X[i];
  if (assembler->setNodes(Xvec)) return 1;
  if (assembler->initialize()) return 1;

  TACSSchurMat *kmat = assembler->createSchurMat();
  TACSSchurMat *gmat = assembler->createSchurMat();
  TACSSchurMat *aux = assembler->createSchurMat();
  kmat->incref();
  gmat->incref();
  aux->incref();
  TACSSchurPc *pc = new TACSSchurPc(kmat, 1000000, 10.0, 1);
  pc->incref();
  GMRES *solver = new GMRES(aux, pc, 10, 15, 0);
  solver->incref();
  solver->setTolerances(1e-12, 1e-12);
  TACSLinearBuckling *buck =
      new TACSLinearBuckling(assembler, sigma, gmat, kmat, aux, solver, 120, nev, 1e-12);
  buck->incref();
  TACSBVec *f = assembler->createVec();
  f->incref();
  f->values() = rhs;
  if (buck->solve(f)) return 1;
  for (int k = 0; k < nev; k++) {
    TacsScalar err = 0.0;
    TacsScalar lam = buck->extractEigenvalue(k, &err);
    printf("eig %d %.17g %.3e\n", k, lam, err);
  }
  const double check = buck->checkEigenvector(0);
  printf("check %.3e\n", check);

  // BCSRMat of K: arrays, and a complete-LU factor object applied to a vector
  BCSRMat *B = nullptr;
  kmat->getBCSRMat(&B, nullptr, nullptr, nullptr);
  int bsize, nrows, ncols;
  const int *rowp, *cols;
  TacsScalar *A;
  B->getArrays(&bsize, &nrows, &ncols, &rowp, &cols, &A);
  if (bsize != 6 || nrows != nn || ncols != nn) return 1;
  BCSRMat *fac = new BCSRMat(MPI_COMM_WORLD, B, 1000000, 10.0);
  fac->incref();
  fac->copyValues(B);
  if (fac->factor()) return 1;
  std::vector<double> x(6 * nn), y(6 * nn), z(6 * nn);
  for (int i = 0; i < 6 * nn; i++) x[i] = sin(1.0 + i);
  fac->applyFactor(x.data(), y.data());
  B->mult(y.data(), z.data());
  double num = 0.0, den = 0.0;
  for (int i = 0; i < 6 * nn; i++) {
    num += (z[i] - x[i]) * (z[i] - x[i]);
    den += x[i] * x[i];
  }
  printf("apply %.3e\n", sqrt(num / den));

  // assembleJacobian(alpha = 2) at the zero state against 2 K
  TACSSchurMat *J = assembler->createSchurMat();
  J->incref();
  assembler->zeroVariables();
  TACSBVec *res = assembler->createVec();
  res->incref();
  if (assembler->assembleJacobian(2.0, 0.0, 0.0, res, J)) return 1;
  assembler->assembleMatType(TACS_STIFFNESS_MATRIX, kmat);
  BCSRMat *BJ = nullptr;
  J->getBCSRMat(&BJ, nullptr, nullptr, nullptr);
  const int *jrowp, *jcols;
  TacsScalar *JA;
  BJ->getArrays(&bsize, &nrows, &ncols, &jrowp, &jcols, &JA);
  B->getArrays(&bsize, &nrows, &ncols, &rowp, &cols, &A);
  double dmax = 0.0, amax = 0.0;
  std::vector<char> bcrow(nn, 0);
  std::vector<int> perm(nn);
  a2ds_mesh_get_ordering(assembler->handle(), perm.data());
  std::vector<int> iperm(nn);
  for (int r = 0; r < nn; r++) iperm[perm[r]] = r;
  for (int b = 0; b < nbc; b++) bcrow[iperm[bcn[b]]] = 1;
  for (int r = 0; r < nn; r++) {
    if (bcrow[r]) continue;
    for (int k = rowp[r]; k < rowp[r + 1]; k++)
      for (int e = 0; e < 36; e++) {
        dmax = fmax(dmax, fabs(JA[(size_t)k * 36 + e] - 2.0 * A[(size_t)k * 36 + e]));
        amax = fmax(amax, fabs(2.0 * A[(size_t)k * 36 + e]));
      }
  }
  printf("jac %.3e\n", dmax / amax);

  res->decref();
  J->decref();
  fac->decref();
  f->decref();
  buck->decref();
  solver->decref();
  pc->decref();
  aux->decref();
  gmat->decref();
  kmat->decref();
  Xvec->decref();
  assembler->decref();
  shell->decref();
  return 0;
}
