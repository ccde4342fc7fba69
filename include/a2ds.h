/*
  a2ds -- GB300 (sm_103a) buckling hot path of the a2d-shells director-MITC
  shell code, behind a plain C ABI.

  Every entry point returns 0 on success or a positive A2DS_ERR_* code; the
  message of the last failure on the calling thread is a2ds_last_error().
  All pointers are caller-owned HOST buffers (copied in or out during the
  call; nothing is retained).  Device memory is owned by the handles.  Calls
  on one handle must not overlap; distinct handles may be used from
  different threads.  There is no CPU fallback: without a usable CUDA device
  every call that needs one fails with A2DS_ERR_CUDA.

  Vectors are node-major with 6 DOF per node (u, v, w, q1, q2, q3) in the
  caller's node numbering, as TACSBVec stores them (src/bpmat/TACSBVec.h:67).
  Element connectivity is in tensor order (xi fastest), as TACSAssembler
  expects after TACSMeshLoader's CQUAD4 reorder (src/io/TACSMeshLoader.cpp:
  932-937).  Block-CSR arrays use the reference layout BCSRMatData
  (src/bpmat/BCSRMatImpl.h:27-45): row-major 6x6 blocks, rows in the matrix
  ordering (see a2ds_mesh_get_ordering), sorted column indices.
*/
#ifndef A2DS_H
#define A2DS_H

#ifdef __cplusplus
extern "C" {
#endif

#define A2DS_OK 0
#define A2DS_ERR_ARG 1        /* invalid argument or size */
#define A2DS_ERR_STATE 2      /* call out of order (e.g. before initialize) */
#define A2DS_ERR_CUDA 3       /* CUDA runtime error / no device */
#define A2DS_ERR_NOMEM 4      /* device or host allocation failed */
#define A2DS_ERR_SINGULAR 5   /* zero pivot block in a factorization */
#define A2DS_ERR_NOCONV 6     /* iterative solve did not reach its tolerance */
#define A2DS_ERR_BREAKDOWN 7  /* Lanczos breakdown (beta ~ 0) */
#define A2DS_ERR_NUMERIC 8    /* NaN/Inf detected on the device */

/* Element matrix kinds, numbered as ElementMatrixType
   (src/elements/TACSElementTypes.h:101-107). */
#define A2DS_STIFFNESS_MATRIX 0
#define A2DS_GEOMETRIC_STIFFNESS_MATRIX 2

/* Node orderings for the matrix, numbered as TACSAssembler::OrderingType
   (src/TACSAssembler.h:64-71).  RCM: TacsComputeRCMOrder from node 0, one
   pass; AMD and TACS_AMD: amd_order_interface (one process, no coupling
   nodes); MULTICOLOR: TacsComputeSerialMultiColor.  ND needs METIS, which is
   not available (a2ds_mesh_plan returns A2DS_ERR_ARG). */
#define A2DS_NATURAL_ORDER 0
#define A2DS_RCM_ORDER 1
#define A2DS_AMD_ORDER 2
#define A2DS_ND_ORDER 3
#define A2DS_TACS_AMD_ORDER 4
#define A2DS_MULTICOLOR_ORDER 5

/* Scatter strategies for element-to-BCSR assembly. */
#define A2DS_SCATTER_ATOMIC 0   /* FP64 atomic adds (fastest, order-dependent rounding) */
#define A2DS_SCATTER_COLORED 1  /* element colours, plain adds (bitwise reproducible) */

typedef struct a2ds_mesh_s *a2ds_mesh;
typedef struct a2ds_bcsr_s *a2ds_bcsr;
typedef struct a2ds_pc_s *a2ds_pc;

/* Message for the last failed call on this thread ("" if none). */
const char *a2ds_last_error(void);

/* Number of CUDA devices visible (0 if none); never fails. */
int a2ds_device_count(void);

/* ------------------------------------------------------------------ mesh
   Replaces: TACSAssembler(comm, 6, numOwnedNodes, numElements)
   (src/TACSAssembler.h:81), setElementConnectivity (:88), setElements (:90)
   with one TACSQuad{4,9}[Nonlinear]Shell type for all elements
   (src/elements/shell/TACSShellElementDefs.h:12-33), and setNodes (:156).
   nodes_per_elem is 4 (Quad4) or 9 (Quad9); conn is num_elements x
   nodes_per_elem; X is num_nodes x 3. */
int a2ds_mesh_create(int num_nodes, int num_elements, int nodes_per_elem,
                     const int *conn, const double *X, int nonlinear,
                     a2ds_mesh *out);
int a2ds_mesh_destroy(a2ds_mesh mesh);

/* Isotropic material (TACSMaterialProperties iso ctor,
   src/constitutive/TACSMaterialProperties.cpp:24-63) shared by all
   elements, plus the element temperature (TACSShellElement::setTemperature,
   src/elements/shell/TACSShellElement.h:76).  Shear correction 5/6 and
   drilling regularisation 10 as in TACSIsoShellConstitutive /
   TACSShellConstitutive (src/constitutive/TACSShellConstitutive.cpp:59). */
int a2ds_mesh_set_material(a2ds_mesh mesh, double E, double nu, double alpha,
                           double temperature);

/* Yield stress of the material (the ys argument of TACSMaterialProperties,
   src/constitutive/TACSMaterialProperties.h); used only by the failure
   values of the .f5 element output. */
int a2ds_mesh_set_yield_stress(a2ds_mesh mesh, double ys);

/* Thickness design variables: one TACSIsoShellConstitutive per group
   (src/constitutive/TACSIsoShellConstitutive.cpp:28-43, design variable
   tNum); elem_group[e] in [0, num_groups).  Default: one group, t = 1e-2. */
int a2ds_mesh_set_thickness(a2ds_mesh mesh, int num_groups, const double *t,
                            const int *elem_group);

/* Dirichlet conditions: TACSAssembler::addBCs(1, &node, nbcs, vars, vals)
   per entry (src/TACSAssembler.h:104); mask bit k fixes DOF k; vals is
   num_bcs x 6 (entries whose bit is clear are ignored).  May be NULL. */
int a2ds_mesh_add_bcs(a2ds_mesh mesh, int num_bcs, const int *nodes,
                      const int *masks, const double *vals);

/* Host-only half of a2ds_mesh_initialize (no GPU needed): the node-to-node
   pattern, the matrix ordering of createSchurMat(order_type), the BCSR
   pattern, the element-slot map and element colours.  After it,
   a2ds_mesh_get_ordering / get_pattern / ilu_pattern can be queried. */
int a2ds_mesh_plan(a2ds_mesh mesh, int order_type);

/* The BCSR pattern of every matrix of this mesh (rows in the matrix
   ordering): sizes first with rowp = cols = NULL. */
int a2ds_mesh_get_pattern(a2ds_mesh mesh, int *nnzb, int *rowp, int *cols);

/* The ILU(lev_fill) pattern of that matrix, as BCSRMat(comm, mat, levFill,
   fill) builds it (BCSRMat::computeILUk, src/bpmat/BCSRMat.cpp:625-754). */
int a2ds_mesh_ilu_pattern(a2ds_mesh mesh, int lev_fill, int *nnzb, int *rowp, int *cols);

/* TACSAssembler::initialize (src/TACSAssembler.cpp:2459) plus the matrix
   ordering of createSchurMat(order_type) (src/TACSAssembler.cpp:3453):
   builds the node-to-node pattern, the ordering, the element-slot map and
   uploads everything.  order_type: one of the A2DS_*_ORDER values above. */
int a2ds_mesh_initialize(a2ds_mesh mesh, int order_type);

/* perm[i] = node in row i of every matrix of this mesh (the reference's
   schurBIndices / b_map, src/TACSAssembler.cpp:3593-3600). */
int a2ds_mesh_get_ordering(a2ds_mesh mesh, int *perm);

/* TACSAssembler::computeLocalNodeToNodeCSR(&rowp, &cols, nodiag)
   (src/TACSAssembler.cpp:1839): rowp[num_nodes+1]; pass cols = NULL to get
   the size in *nnz first. */
int a2ds_mesh_node_csr(a2ds_mesh mesh, int nodiag, int *nnz, int *rowp, int *cols);

/* ------------------------------------------------------------ matrices
   Replaces TACSAssembler::createSchurMat (src/TACSAssembler.cpp:3453) with a
   single-GPU BCSR matrix in the mesh ordering. */
int a2ds_bcsr_create(a2ds_mesh mesh, a2ds_bcsr *out);
int a2ds_bcsr_destroy(a2ds_bcsr mat);

/* BCSRMat::getArrays (src/bpmat/BCSRMat.h:82): sizes first (pointers may be
   NULL), then rowp[nrows+1], cols[nnzb], vals[36*nnzb]. */
int a2ds_bcsr_get(a2ds_bcsr mat, int *nrows, int *nnzb, int *rowp, int *cols,
                  double *vals);

/* Overwrite the values (36*nnzb, the layout a2ds_bcsr_get returns). */
int a2ds_bcsr_set_values(a2ds_bcsr mat, const double *vals);

/* TACSAssembler::assembleMatType(matType, A) (src/TACSAssembler.cpp:4186)
   at the element state vars (num_nodes x 6, NULL = zero), including the
   row-only Dirichlet treatment of TACSSchurMat::applyBCs
   (src/bpmat/TACSSchurMat.cpp:662).  For the geometric stiffness vars is the
   load path (TACSShellElement::getMatType, TACSShellElement.h:675-771). */
int a2ds_assemble_mat(a2ds_mesh mesh, int mat_type, const double *vars,
                      a2ds_bcsr A);

/* Same, selecting the scatter strategy (A2DS_SCATTER_*). */
int a2ds_assemble_mat_ex(a2ds_mesh mesh, int mat_type, const double *vars,
                         a2ds_bcsr A, int scatter);

/* The assembler-level element inner product that the reference's (commented)
   TACSLinearBuckling::evalEigenXptSens calls (src/TACSBuckling.cpp:471-476),
   element by element TACSElement::addMatXptSensInnerProduct
   (src/elements/TACSElement.cpp:434-507): dfdX += scale *
   d(psi^T M(X, vars) phi)/dX for M = K (mat_type A2DS_STIFFNESS_MATRIX, at
   vars) or G (A2DS_GEOMETRIC_STIFFNESS_MATRIX, along vars), by second-order
   central differences with step dh in every element coordinate (dh = 0: the
   reference's real-mode step 1e-7).  psi, phi, vars: num_nodes x 6 (vars
   NULL = zero); dfdX: num_nodes x 3, added into.  Element matrices without
   the Dirichlet rows. */
int a2ds_add_mat_xpt_sens_inner_product(a2ds_mesh mesh, int mat_type, double scale,
                                        const double *psi, const double *phi,
                                        const double *vars, double dh, double *dfdX);

/* The assembler-level thickness inner product of the reference's
   (commented) TACSLinearBuckling::evalEigenDVSens (src/TACSBuckling.cpp:
   397-403, assembler->addMatDVSensInnerProduct), element by element
   TACSElement::addMatDVSensInnerProduct (src/elements/TACSElement.cpp:
   355-432): dfdx[g] += scale * sum over the elements of thickness group g of
   d(psi^T M(vars) phi)/dt for M = K (at vars) or G (along vars).  Exact:
   the element matrices are linear in the constitutive matrix, so the
   derivative is the element matrix with dC/dt (the reference takes central
   differences with step 1e-7).  psi, phi, vars: num_nodes x 6 (vars NULL =
   zero); dfdx: num_groups values (a2ds_mesh_set_thickness), added into. */
int a2ds_add_mat_dv_sens_inner_product(a2ds_mesh mesh, int mat_type, double scale,
                                       const double *psi, const double *phi,
                                       const double *vars, double *dfdx);

/* The adjoint-residual coordinate product of the same body
   (addAdjointResXptSensProducts, src/TACSBuckling.cpp:486), element by
   element TACSElement::addAdjResXptProduct (src/elements/TACSElement.cpp:
   270-330): dfdX += scale * psi^T dR(X, vars)/dX, central differences with
   step dh (0 = 1e-7).  psi, vars: num_nodes x 6 (vars NULL = zero); dfdX
   num_nodes x 3, added into.  The element residuals only (no Dirichlet
   rows). */
int a2ds_add_adjoint_res_xpt_sens_product(a2ds_mesh mesh, double scale, const double *psi,
                                          const double *vars, double dh, double *dfdX);

/* The state derivative of the same body (evalMatSVSensInnerProduct,
   src/TACSBuckling.cpp:481), element by element
   TACSElement::getMatSVSensInnerProduct (src/elements/TACSElement.cpp:
   509-581): dfdu = d(psi^T M(vars) phi)/d(vars) for M = K (the tangent at
   vars) or G (along vars), central differences with step dh (0 = 1e-7) in
   every element state entry.  dfdu: num_nodes x 6, overwritten, Dirichlet
   entries zero (the right-hand side of a load-path adjoint). */
int a2ds_eval_mat_sv_sens_inner_product(a2ds_mesh mesh, int mat_type, const double *psi,
                                        const double *phi, const double *vars, double dh,
                                        double *dfdu);

/* TACSAssembler::assembleRes (src/TACSAssembler.cpp:4000) at vars (NULL =
   zero); res is num_nodes x 6, BC DOFs set to vars - bcval as in
   TACSBVec::applyBCs / the assembler's BC residual. */
int a2ds_assemble_res(a2ds_mesh mesh, const double *vars, double *res);

/* TACSAssembler::assembleJacobian(1, 0, 0, res, A) (src/TACSAssembler.cpp:
   4084): the tangent and residual at vars in one pass (res may be NULL). */
int a2ds_assemble_jacobian(a2ds_mesh mesh, const double *vars, double *res,
                           a2ds_bcsr A);

/* BCSRMat::mult / TACSSchurMat::mult (src/bpmat/BCSRMat.cpp:1212,
   TACSSchurMat.cpp:866): y = A x, x and y num_nodes x 6 in node order. */
int a2ds_bcsr_mult(a2ds_bcsr A, const double *x, double *y);

/* y = A x with both vectors already in the matrix (row) ordering. */
int a2ds_bcsr_mult_rows(a2ds_bcsr A, const double *x, double *y);

/* a2ds_bcsr_mult_rows without any device allocation.  No counterpart in the
   reference: it exists for callers that cannot call cudaMalloc/cudaFree
   (their memory manager owns the device, or cudaFree's device-wide wait is
   not acceptable).  x and y are staged through a fixed device array of at
   most 65536 block rows (6.3 MB, kept by every GPU that loads the library
   until exit); larger matrices are rejected with A2DS_ERR_ARG.  The first
   call on a device resolves that array's address (make it before any stream
   capture).  All calls share the array: calls that overlap on the GPU race. */
int a2ds_bcsr_mult_rows_noalloc(a2ds_bcsr A, const double *x, double *y);

/* BCSRMat::copyValues (src/bpmat/BCSRMat.cpp:2375): Y <- X;
   BCSRMat::axpy (:2430): Y <- Y + alpha X; same pattern required. */
/* Device time of the matrix product on device-resident vectors: y = A x
   (nvec = 1, BCSRMatVecMult6, src/bpmat/BCSRMatMult6.cpp:82-122) or A times
   nvec stacked vectors (2, 4, 8, 16; the block Lanczos product), averaged
   over iters launches after 3 warm-up launches, CUDA events on the mesh's
   stream.  No counterpart in the reference (a measurement entry). */
int a2ds_bcsr_time_mult(a2ds_bcsr A, int nvec, int iters, double *ms_per_mult);
/* The same for the double-float product of the mixed-precision GMRES-IR
   inner loop: A converted once to double-float pairs (8 bytes per value),
   times nvec (1, 2, 4, 8, 16) stacked FP32 vectors, double-float result. */
int a2ds_bcsr_time_mult_df(a2ds_bcsr A, int nvec, int iters, double *ms_per_mult);

int a2ds_bcsr_copy(a2ds_bcsr Y, a2ds_bcsr X);
int a2ds_bcsr_axpy(a2ds_bcsr Y, double alpha, a2ds_bcsr X);

/* TACSSchurMat::applyBCs (src/bpmat/TACSSchurMat.cpp:662-700) with the
   mesh's Dirichlet set: zero BC rows, identity on the diagonal. */
int a2ds_bcsr_apply_bcs(a2ds_bcsr A);

/* ------------------------------------------------ factorization (ILU(k))
   Replaces TACSSchurPc(kmat, levFill, fill, 1) (src/bpmat/TACSSchurMat.cpp:
   944): symbolic ILU(levFill) of A's pattern (BCSRMat::computeILUk,
   src/bpmat/BCSRMat.cpp:625); levFill >= num_nodes gives the complete LU.
   precision: 64 (FP64 factor), 48 (factored in double-float arithmetic on
   the FP32 pipe, ~48-bit mantissa, then stored as FP64) or 32 (FP32
   factor). */
int a2ds_pc_create(a2ds_bcsr A, int lev_fill, int precision, a2ds_pc *out);
int a2ds_pc_destroy(a2ds_pc pc);

/* TACSSchurPc::factor (src/bpmat/TACSSchurMat.cpp:1430) of the current
   values of the matrix given at creation (or of `from`, same pattern, when
   not NULL). */
int a2ds_pc_factor(a2ds_pc pc, a2ds_bcsr from);

/* TACSSchurPc::applyFactor (src/bpmat/TACSSchurMat.cpp:1549): y = (LU)^-1 x,
   node-ordered num_nodes x 6 host vectors. */
int a2ds_pc_apply(a2ds_pc pc, const double *x, double *y);

/* applyFactor for nrhs right-hand sides at once (nrhs in {1, 2, 4, 8, 16};
   the reference applies one vector per call): x and y hold nrhs node-ordered
   num_nodes x 6 vectors one after another.  Each factor block is read once
   for all of them. */
int a2ds_pc_apply_multi(a2ds_pc pc, int nrhs, const double *x, double *y);

/* BCSRMat::getArrays on the factor: the ILU(k) pattern (bit-exact with the
   reference's) and the factored values (diagonal blocks stored inverted,
   as BCSRMatFactor6 leaves them). */
int a2ds_pc_get(a2ds_pc pc, int *nrows, int *nnzb, int *rowp, int *cols,
                double *vals);

/* GMRES(mat, pc, msub, nrestart, isFlexible = 0) with setTolerances(rtol,
   atol) and solve(b, x, zero_guess = 1) (src/bpmat/KSM.cpp:547-645,
   785-970): right-preconditioned restarted GMRES on A with the factor of pc
   (NULL: no preconditioner).  b and x are node-ordered num_nodes x 6 host
   vectors.  *iters receives the total inner iterations and *res_norm the
   final residual estimate; A2DS_ERR_NOCONV if the tolerance was not met
   (x then holds the last iterate). */
int a2ds_gmres_solve(a2ds_bcsr A, a2ds_pc pc, int msub, int nrestart, double rtol,
                     double atol, const double *b, double *x, int *iters,
                     double *res_norm);

/* GMRES(mat, pc, msub, nrestart, isFlexible = 1) (src/bpmat/KSM.h:391-419,
   flexible variant of GMRES::solve, src/bpmat/KSM.cpp:785-970) run as GMRES-IR
   for nrhs in {1, 2, 4, 8, 16} right-hand sides at once: one Krylov space per
   right-hand side, FP64 Arnoldi vectors and products with A, the factor of
   pc (FP32, double-float or FP64) applied to every Arnoldi vector, and the
   true FP64 residual b - A x evaluated after every cycle of msub (<= 63)
   steps.  Stops when ||b_k - A x_k|| <= rtol ||b_k|| for every k (zero
   initial guess); A2DS_ERR_NOCONV after nrestart + 1 cycles (x then holds
   the last iterate).  b and x hold nrhs node-ordered num_nodes x 6 vectors
   one after another; *iters receives the Arnoldi steps (= preconditioner
   applications). */
int a2ds_fgmres_solve(a2ds_bcsr A, a2ds_pc pc, int msub, int nrestart, double rtol, int nrhs,
                      const double *b, double *x, int *iters);

/* --------------------------------------------------------- buckling solve */
typedef struct {
  double sigma;          /* spectral shift (TACSLinearBuckling ctor) */
  int max_lanczos;       /* maximum Lanczos vectors */
  int num_eigvals;       /* eigenvalues wanted (lowest magnitude) */
  double eig_tol;        /* relative eigenvalue residual tolerance */
  int lev_fill;          /* ILU level of fill for the preconditioner */
  int gmres_m;           /* GMRES subspace size */
  int gmres_restarts;    /* GMRES restarts */
  double gmres_rtol;     /* GMRES relative tolerance */
  double gmres_atol;     /* GMRES absolute tolerance */
  int precision;         /* 64: all-FP64; 48: double-float factors + FP64
                            solves and refinement; 32: FP32 factors and
                            FP32 triangular solves as the preconditioner of
                            FP64 flexible GMRES (GMRES-IR) for the load
                            path and every shift-invert solve */
  int seed;              /* Lanczos start vector seed */
  int block_size;        /* Lanczos block size p in {1, 2, 4, 8, 16}: p vectors
                            per shift-invert solve (1 = the reference's
                            single-vector Lanczos) */
} a2ds_buckling_opts;

/* Fills opts with the defaults (sigma = 0, 100 vectors, 10 eigenvalues,
   tol 1e-10, complete LU, GMRES(30, 15) at 1e-12, FP64, block size 4). */
void a2ds_buckling_default_opts(a2ds_buckling_opts *opts);

/* TACSLinearBuckling::solve(rhs, NULL) (src/TACSBuckling.cpp:197-278) and
   extractEigenvector (:288): K at zero state, load path K u = rhs,
   G at u, shift-invert Lanczos for the num_eigvals buckling loads lambda of
   K x + lambda G x = 0 with the smallest magnitude.  Outputs (host):
   eigvals[num_eigvals], errors[num_eigvals] (||K x + lambda G x|| / ||K x||),
   eigvecs (num_eigvals x num_nodes x 6, may be NULL), path (num_nodes x 6,
   may be NULL). */
int a2ds_buckling_solve(a2ds_mesh mesh, const a2ds_buckling_opts *opts,
                        const double *rhs, double *eigvals, double *errors,
                        double *eigvecs, double *path);

/* SEP::solve with EPBucklingShiftInvert(sigma, K, G)
   (src/bpmat/GSEP.cpp:200-244, 485-596) on matrices the caller assembled:
   the num_eigvals smallest-magnitude lambda of K x + lambda G x = 0 by the
   same block shift-invert Lanczos as a2ds_buckling_solve (K and G in this
   mesh's pattern, Dirichlet rows applied).  Used, for example, for
   buckling about a nonlinear preloaded state with K = K_T(u) from
   a2ds_assemble_jacobian and G from a2ds_assemble_mat along u.  Outputs as
   a2ds_buckling_solve (no path). */
int a2ds_eigen_shift_invert(a2ds_mesh mesh, const a2ds_buckling_opts *opts, a2ds_bcsr K,
                            a2ds_bcsr G, double *eigvals, double *errors,
                            double *eigvecs);

/* Timings and counters of the last a2ds_buckling_solve on this mesh:
   fills up to n doubles {total_s, assemble_k_s, assemble_g_s, factor_s,
   path_s, lanczos_s, lanczos_vectors, inner_iters, kernel_launches,
   solve_event_ms, factor_a_event_ms, factor_k_event_ms, factor_nnzb,
   factor_levels, factor_flops, block_size, block_iters, trisolve_ms,
   trisolve_calls, gmres_ir_iters, gmres_ir_cycles} (the last two: Arnoldi
   steps and restart cycles of the GMRES-IR solves with FP32 factors). */
int a2ds_buckling_stats(a2ds_mesh mesh, int n, double *out);

/* ------------------------------------------------ nonlinear preload
   The reference has the building blocks of buckling about a nonlinear
   preloaded state -- TACSAssembler::assembleRes / assembleJacobian
   (src/TACSAssembler.cpp:4000, 4084), TACSSchurPc and the nonlinear shell
   elements (TACSQuad{4,9}NonlinearShell, src/elements/shell/
   TACSShellElementDefs.h:27-33) -- but no driver (its continuation and
   integrator classes are not built).  These entries are that driver.

   Newton load stepping: equal increments s_k = load k / nsteps of the
   nodal load vector rhs (num_nodes x 6; Dirichlet entries ignored), at each
   full Newton on R(u) = s_k rhs with the exact tangent K_T(u) (complete LU
   in `precision` 64, 48 or 32 on the GPU, FP64 GMRES-IR solves to 1e-12)
   until ||R(u) - s_k rhs|| <= rtol ||s_k rhs|| (Dirichlet rows u - u_bc).
   u_out: num_nodes x 6; iters: nsteps values (Newton steps per increment,
   may be NULL); *rel_out: the final relative residual (may be NULL).
   A2DS_ERR_NOCONV if an increment needs more than max_newton steps. */
int a2ds_newton_preload(a2ds_mesh mesh, const double *rhs, double load, int nsteps, double rtol,
                        int max_newton, int precision, double *u_out, int *iters,
                        double *rel_out);

/* Buckling about the preloaded state u (num_nodes x 6): the num_eigvals
   smallest-magnitude lambda of K_T(u) x + lambda G(u) x = 0, G(u) the
   geometric stiffness along u, by the same block shift-invert Lanczos as
   a2ds_buckling_solve (EPBucklingShiftInvert + SEP::solve,
   src/bpmat/GSEP.cpp:200-244, 485-596).  Outputs as a2ds_buckling_solve. */
int a2ds_preload_buckling(a2ds_mesh mesh, const a2ds_buckling_opts *opts, const double *u,
                          double *eigvals, double *errors, double *eigvecs);

/* dlambda_n/dX (num_nodes x 3) of a2ds_preload_buckling's n-th load, the
   formula of the reference's (commented) evalEigenXptSens
   (src/TACSBuckling.cpp:457-497) with the preload's Newton system:
     dlambda/dX = -[phi^T K_T' phi + lambda phi^T G' phi - psi^T R'] / phi^T G phi,
     K_T(u) psi = d/du [phi^T (K_T(u) + lambda G(u)) phi],
   ' = d/dX at fixed u (R' the residual's coordinate derivative at fixed
   loads); element derivatives by central differences with step dh (0 =
   1e-7), element states recomputed from u and X on the GPU. */
int a2ds_preload_xpt_sens(a2ds_mesh mesh, int n, double dh, double *dlam_dX);

/* ---------------------------------------------- eigenvalue sensitivities
   The derivative of buckling load lambda_n with respect to each thickness
   group, dlambda/dt_g = -phi^T (dK/dt_g + lambda dG/dt_g) phi / (phi^T G phi)
   plus the load-path adjoint term (the formula documented at
   src/TACSBuckling.cpp:359-382; the reference's evalEigenDVSens body is
   commented out).  Needs a preceding a2ds_buckling_solve on this mesh. */
int a2ds_eig_sens_thickness(a2ds_mesh mesh, int n, double *dlam_dt);

/* TACSLinearBuckling::evalEigenXptSens (src/TACSBuckling.cpp:457-497, body
   commented out in the reference; the same formula):
   dlambda/dX = -[phi^T K' phi + lambda phi^T G'(path) phi
                  - lambda psi^T K' path] / (phi^T G phi),
   ' = d/dX at fixed states, K psi = d(phi^T G(path) phi)/d(path), the
   element derivatives by central differences with step dh (0 = 1e-7, the
   reference's element default).  dlam_dX: num_nodes x 3.  Needs a
   preceding a2ds_buckling_solve on this mesh; loads are fixed nodal forces
   (no thermal load). */
int a2ds_eig_sens_xpts(a2ds_mesh mesh, int n, double dh, double *dlam_dX);

/* ------------------------------------------------------ BDF mesh input
   Replaces: TACSMeshLoader::scanBDFFile (src/io/TACSMeshLoader.cpp:569-1098),
   getConnectivity (:1247), getBCs (:1272), getElementDescript and
   getComponentDescript (src/io/TACSMeshLoader.h:73-74) on one process.
   Reads GRID / GRID*, SPC / SPC* and the element cards CBAR, CQUADR,
   CQUAD4, CQUAD9, CQUAD, CHEXA (8 nodes), CTRIA3 and CTETRA, with the same
   field widths, continuation rules, Nastran real formats, node-order
   conversion (CQUAD4/CQUADR, CQUAD9/CQUAD, CHEXA) and renumbering (nodes by
   sorted file node number, elements by sorted file element number).  Where
   the reference aborts (unreadable file, empty bulk line, bad element
   card, undefined node) the scan fails with A2DS_ERR_ARG.  Arrays:
   elem_node_ptr num_elements + 1, elem_node_conn conn_size,
   elem_component num_elements (0-based), Xpts num_nodes x 3; bc_nodes
   num_bcs, bc_ptr num_bcs + 1, bc_vars / bc_vals bc_vars_size (variable
   0..7 per entry).  Host only: no GPU needed. */
typedef struct a2ds_bdf_s *a2ds_bdf;
int a2ds_bdf_scan(const char *file_name, a2ds_bdf *out);
int a2ds_bdf_destroy(a2ds_bdf bdf);
int a2ds_bdf_get_sizes(a2ds_bdf bdf, int *num_nodes, int *num_elements, int *conn_size,
                       int *num_bcs, int *bc_vars_size, int *num_components);
int a2ds_bdf_get_connectivity(a2ds_bdf bdf, int *elem_node_ptr, int *elem_node_conn,
                              int *elem_component, double *Xpts);
int a2ds_bdf_get_bcs(a2ds_bdf bdf, int *bc_nodes, int *bc_vars, int *bc_ptr, double *bc_vals);
/* Element type name of a component (first card seen for it, "CTETRA10" for
   10-node tetrahedra) and its "$       Shell" comment name ("" if none),
   copied into name[len] with a terminating NUL. */
int a2ds_bdf_get_element_descript(a2ds_bdf bdf, int comp, char *name, int len);
int a2ds_bdf_get_component_descript(a2ds_bdf bdf, int comp, char *descript, int len);

/* ------------------------------------------------------------ .f5 output
   Replaces: TACSToFH5(assembler, TACS_BEAM_OR_SHELL_ELEMENT, write_flag)
   with setComponentName and writeToFile (src/io/TACSToFH5.cpp:35-358;
   file layout of TACSFH5File, src/io/TACSFH5.cpp:64-210) on one process,
   for the connectivity, node, displacement and load output classes: the
   same layout as the reference for the same mesh, names and variables,
   and the element output classes.
   write_flag: A2DS_F5_* bits.  Loads are the residual at vars without
   external loads (assembleRes(F, 0.0)); the element classes (strains,
   stresses, extras: failure0-5 and dv1-7 as getOutputData) are evaluated
   at every element's node points on the GPU (an "element data" zone).
   Both need an initialized mesh and a GPU; extras need
   a2ds_mesh_set_yield_stress.  component_names: NULL or
   num_components entries (NULL entries give "Component k");
   num_components is raised to 1 + the largest elem_component value;
   elem_component: NULL (all 0) or num_elements values; vars: NULL (zeros)
   or num_nodes x 6 in the caller's node numbering (a load path or an
   eigenvector); time: the zone time stamp (getSimulationTime). */
#define A2DS_F5_CONNECTIVITY 1
#define A2DS_F5_NODES 2
#define A2DS_F5_DISPLACEMENTS 4
#define A2DS_F5_STRAINS 8
#define A2DS_F5_STRESSES 16
#define A2DS_F5_EXTRAS 32
#define A2DS_F5_LOADS 64
int a2ds_write_f5(a2ds_mesh mesh, const char *file_name, int write_flag, int num_components,
                  const char *const *component_names, const int *elem_component,
                  const double *vars, double time);

#ifdef __cplusplus
}
#endif
#endif
