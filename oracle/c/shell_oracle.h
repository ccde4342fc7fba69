/*
  CPU restatement of the reference's buckling hot path (sean-engelstad/
  a2d-shells).  TEST INFRASTRUCTURE ONLY: the checker that the GB300 path is
  compared against, and the timed CPU baseline.  Nothing shipped links it.

  Parity pinning: the element routines are checked against fixtures written
  by the reference itself (tests/golden/elements_*.npz, made by
  oracle/ref/golden_gen.cpp from the reference's own sources), the assembly
  and solver routines against tests/golden/cyl_*.npz.

  Conventions (as in the reference):
    * element variables: 6 per node (u, v, w, q1, q2, q3), node-major;
    * element matrices: row-major (6*nn) x (6*nn);
    * nodes in tensor order, order = nodes per direction (2: Quad4, 3: Quad9).
*/
#ifndef A2DS_SHELL_ORACLE_H
#define A2DS_SHELL_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

/* Matrix kinds, numbered as ElementMatrixType (src/elements/TACSElementTypes.h:101-107) */
enum { ORC_STIFFNESS = 0, ORC_MASS = 1, ORC_GEOMETRIC = 2 };

typedef struct {
  double E, nu, t, alpha, temperature;
  double kcorr;       /* 5/6 */
  double drill_reg;   /* DRILLING_REGULARIZATION = 10 */
  double t_offset;    /* 0 */
} orc_material;

/* TACSShellElement::addResidual (TACSShellElement.h:303-449) */
void orc_add_residual(int order, int nonlinear, const orc_material *m,
                      const double *X, const double *vars, double *res);

/* TACSShellElement::addJacobian with beta = gamma = 0
   (TACSShellElement.h:455-672): res += R, mat += alpha*J */
void orc_add_jacobian(int order, int nonlinear, const orc_material *m,
                      double alpha, const double *X, const double *vars,
                      double *res, double *mat);

/* TACSShellElement::getMatType (TACSShellElement.h:675-771); the geometric
   stiffness is the central difference of the nonlinear tangent used there. */
void orc_get_mat_type(int order, int nonlinear, int kind, const orc_material *m,
                      const double *X, const double *vars, double *mat);

#ifdef __cplusplus
}
#endif
#endif
