// The call sequence of the reference's examples/cylinder-buckling/
// mechBuckling.cpp (BDF deck -> one shell element object per component ->
// createTACS -> Schur matrices, TACSSchurPc, GMRES -> TACSLinearBuckling ->
// eigenvalues and eigenvector .f5 files) through the C++ classes of
// include/a2ds_tacs.hpp.
//
// usage: mech_buckling deck.bdf E nu thickness sigma num_eigvals out.f5
// prints one line per eigenvalue: index, value, residual error
#include <stdio.h>
#include <stdlib.h>

#include "a2ds_tacs.hpp"

using namespace a2ds_tacs;

int main(int argc, char **argv) {
  if (argc < 8) {
    fprintf(stderr, "usage: %s deck.bdf E nu thickness sigma num_eigvals out.f5\n", argv[0]);
    return 2;
  }
  const double E = atof(argv[2]), nu = atof(argv[3]), thick = atof(argv[4]);
  const double sigma = atof(argv[5]);
  const int num_eigvals = atoi(argv[6]);

  TACSMeshLoader *mesh = new TACSMeshLoader(MPI_COMM_WORLD);
  mesh->incref();
  if (mesh->scanBDFFile(argv[1])) return 1;
  int num_components = mesh->getNumComponents();

  TACSShellTransform *transform = new TACSShellNaturalTransform();
  transform->incref();
  TACSMaterialProperties *mat = new TACSMaterialProperties(2718.0, 0.0, E, nu, 1e11, 10e-6, 0.0);
  mat->incref();
  for (int icomp = 0; icomp < num_components; icomp++) {
    const char *descriptor = mesh->getElementDescript(icomp);
    TACSIsoShellConstitutive *con = new TACSIsoShellConstitutive(mat, thick);
    TACSElement *shell = TacsCreateShellByName(descriptor, transform, con);
    if (!shell) {
      fprintf(stderr, "no shell element for %s\n", descriptor);
      return 1;
    }
    mesh->setElement(icomp, shell);
  }
  mat->decref();
  transform->decref();

  TACSAssembler *assembler = mesh->createTACS(6);
  if (!assembler) return 1;
  assembler->incref();
  mesh->decref();

  for (int ielem = 0; ielem < assembler->getNumElements(); ielem++) {
    TACSQuad4Shell *elem = dynamic_cast<TACSQuad4Shell *>(assembler->getElement(ielem));
    if (elem) elem->setTemperature(0.0);
  }

  TACSBVec *u0 = assembler->createVec();
  TACSBVec *f = assembler->createVec();
  u0->incref();
  f->incref();
  TACSSchurMat *kmat = assembler->createSchurMat(TACSAssembler::TACS_AMD_ORDER);
  TACSSchurMat *gmat = assembler->createSchurMat();
  TACSSchurMat *aux_mat = assembler->createSchurMat();
  if (!kmat || !gmat || !aux_mat) return 1;

  int lev = 1000000;
  double fill = 10.0;
  TACSSchurPc *pc = new TACSSchurPc(kmat, lev, fill, 1);
  pc->incref();
  GMRES *solver = new GMRES(aux_mat, pc, 10, 15, 0);
  solver->incref();
  solver->setTolerances(1e-12, 1e-12);

  TACSLinearBuckling *buckling = new TACSLinearBuckling(assembler, sigma, gmat, kmat, aux_mat,
                                                        solver, 120, num_eigvals, 1e-12);
  buckling->incref();
  KSMPrint *ksm_print = new KSMPrintStdout("BucklingAnalysis", 0, 10);
  ksm_print->incref();
  // the deck's enforced end displacement drives the load path (no nodal loads)
  if (buckling->solve(NULL, u0, ksm_print)) return 1;

  int write_flag = (TACS_OUTPUT_CONNECTIVITY | TACS_OUTPUT_NODES | TACS_OUTPUT_DISPLACEMENTS |
                    TACS_OUTPUT_STRAINS | TACS_OUTPUT_STRESSES | TACS_OUTPUT_EXTRAS);
  TACSToFH5 *f5 = new TACSToFH5(assembler, TACS_BEAM_OR_SHELL_ELEMENT, write_flag);
  f5->incref();
  TACSBVec *phi = assembler->createVec();
  phi->incref();
  for (int imode = 0; imode < num_eigvals; imode++) {
    TacsScalar error = 0.0;
    TacsScalar lam = buckling->extractEigenvector(imode, phi, &error);
    printf("%d %.17g %.3e\n", imode, lam, error);
    if (imode == 0) {
      assembler->setVariables(phi);
      if (f5->writeToFile(argv[7])) return 1;
    }
  }

  phi->decref();
  f5->decref();
  ksm_print->decref();
  buckling->decref();
  solver->decref();
  pc->decref();
  u0->decref();
  f->decref();
  assembler->decref();
  return 0;
}
