/* C++ classes with the reference's names and call sequence on the buckling
   path, forwarding to the C ABI of a2ds.h (header only).

   A driver written against the reference's classes (the sequence of
   examples/cylinder-buckling/mechBuckling.cpp: TACSMeshLoader::scanBDFFile,
   TacsCreateShellByName per component, createTACS, createSchurMat,
   TACSSchurPc, GMRES, TACSLinearBuckling::solve, extractEigenvector,
   TACSToFH5::writeToFile) compiles against these with `using namespace
   a2ds_tacs;` in place of the reference's headers and without MPI.  What
   the GB300 path covers and how the classes map:

   TACSMeshLoader      TACSMeshLoader (src/io/TACSMeshLoader.h): BDF input,
                       one element object per component, createTACS
   TACSAssembler       TACSAssembler (src/TACSAssembler.h): one a2ds_mesh;
                       all elements one shell type (TACSQuad4/9[Nonlinear]
                       Shell) and one material; thickness design groups =
                       the distinct constitutive objects
   TACSSchurMat        TACSSchurMat: one a2ds_bcsr in the assembler's
                       ordering (the first createSchurMat fixes it)
   TACSSchurPc, GMRES  TACSSchurPc / GMRES (src/bpmat/TACSSchurMat.h,
                       src/bpmat/KSM.h): settings read by TACSLinearBuckling
                       and direct factor / apply / solve calls
   TACSLinearBuckling  TACSLinearBuckling (src/TACSBuckling.h:43-107)
   TACSToFH5           TACSToFH5 (src/io/TACSToFH5.h)

   Errors follow the reference: a message on stderr (with a2ds_last_error())
   and, where the reference returns an int, a nonzero code.  Objects are
   reference counted like TACSObject (src/TACSObject.h:112-146). */
#ifndef A2DS_TACS_HPP
#define A2DS_TACS_HPP

#include <math.h>
#include <stdio.h>
#include <string.h>

#include <string>
#include <vector>

#include "a2ds.h"

namespace a2ds_tacs {

typedef double TacsScalar;
#ifndef MPI_COMM_WORLD
typedef int MPI_Comm;  // single process: the communicator argument is ignored
static const MPI_Comm MPI_COMM_WORLD = 0;
#endif

enum ElementMatrixType {
  TACS_STIFFNESS_MATRIX = A2DS_STIFFNESS_MATRIX,
  TACS_GEOMETRIC_STIFFNESS_MATRIX = A2DS_GEOMETRIC_STIFFNESS_MATRIX
};
enum ElementType { TACS_BEAM_OR_SHELL_ELEMENT = 1 };
static const int TACS_OUTPUT_CONNECTIVITY = A2DS_F5_CONNECTIVITY;
static const int TACS_OUTPUT_NODES = A2DS_F5_NODES;
static const int TACS_OUTPUT_DISPLACEMENTS = A2DS_F5_DISPLACEMENTS;
static const int TACS_OUTPUT_STRAINS = A2DS_F5_STRAINS;
static const int TACS_OUTPUT_STRESSES = A2DS_F5_STRESSES;
static const int TACS_OUTPUT_EXTRAS = A2DS_F5_EXTRAS;
static const int TACS_OUTPUT_LOADS = A2DS_F5_LOADS;

inline int a2ds_report(const char *where, int rc) {
  if (rc) fprintf(stderr, "%s: %s\n", where, a2ds_last_error());
  return rc;
}

class TACSObject {
 public:
  TACSObject() : ref_count_(0) {}
  virtual ~TACSObject() {}
  void incref() { ref_count_++; }
  void decref() {
    if (--ref_count_ <= 0) delete this;
  }

 private:
  TACSObject(const TACSObject &);
  TACSObject &operator=(const TACSObject &);
  int ref_count_;
};

// Holds o with one reference; releases the previous one.
template <class T>
inline void a2ds_hold(T *&slot, T *o) {
  if (o) o->incref();
  if (slot) slot->decref();
  slot = o;
}

/* ------------------------------------------------------------ materials */
class TACSMaterialProperties : public TACSObject {
 public:
  // isotropic (src/constitutive/TACSMaterialProperties.cpp:24-63)
  TACSMaterialProperties(TacsScalar rho, TacsScalar specific_heat, TacsScalar E, TacsScalar nu,
                         TacsScalar ys, TacsScalar alpha, TacsScalar kappa)
      : rho(rho), specific_heat(specific_heat), E(E), nu(nu), ys(ys), alpha(alpha),
        kappa(kappa) {}
  TacsScalar rho, specific_heat, E, nu, ys, alpha, kappa;
};

class TACSShellTransform : public TACSObject {};
class TACSShellNaturalTransform : public TACSShellTransform {};

class TACSShellConstitutive : public TACSObject {
 public:
  virtual TACSMaterialProperties *getMaterialProperties() = 0;
  virtual TacsScalar getThickness() const = 0;
};

// TACSIsoShellConstitutive (src/constitutive/TACSIsoShellConstitutive.h):
// thickness t, design variable tNum (-1: none), no offset
class TACSIsoShellConstitutive : public TACSShellConstitutive {
 public:
  TACSIsoShellConstitutive(TACSMaterialProperties *props, TacsScalar t = 1.0, int tNum = -1)
      : props_(nullptr), t_(t), tNum_(tNum) {
    a2ds_hold(props_, props);
  }
  ~TACSIsoShellConstitutive() {
    if (props_) props_->decref();
  }
  TACSMaterialProperties *getMaterialProperties() { return props_; }
  TacsScalar getThickness() const { return t_; }
  void setThickness(TacsScalar t) { t_ = t; }
  int getThicknessDVNum() const { return tNum_; }

 private:
  TACSMaterialProperties *props_;
  TacsScalar t_;
  int tNum_;
};

/* ------------------------------------------------------------- elements */
class TACSElement : public TACSObject {
 public:
  TACSElement(int order, int nonlinear, TACSShellTransform *transform,
              TACSShellConstitutive *con)
      : order_(order), nonlinear_(nonlinear), transform_(nullptr), con_(nullptr),
        temperature_(0.0) {
    a2ds_hold(transform_, transform);
    a2ds_hold(con_, con);
  }
  ~TACSElement() {
    if (con_) con_->decref();
    if (transform_) transform_->decref();
  }
  int getNumNodes() const { return order_ * order_; }
  int getVarsPerNode() const { return 6; }
  int order() const { return order_; }
  int nonlinear() const { return nonlinear_; }
  TACSShellConstitutive *getConstitutive() { return con_; }
  // TACSShellElement::setTemperature (TACSShellElement.h:76)
  void setTemperature(TacsScalar T) { temperature_ = T; }
  TacsScalar getTemperature() const { return temperature_; }

 private:
  int order_, nonlinear_;
  TACSShellTransform *transform_;
  TACSShellConstitutive *con_;
  TacsScalar temperature_;
};

// The instantiations the GB300 path implements (TACSShellElementDefs.h:12-33)
class TACSQuad4Shell : public TACSElement {
 public:
  TACSQuad4Shell(TACSShellTransform *tr, TACSShellConstitutive *con)
      : TACSElement(2, 0, tr, con) {}
};
class TACSQuad9Shell : public TACSElement {
 public:
  TACSQuad9Shell(TACSShellTransform *tr, TACSShellConstitutive *con)
      : TACSElement(3, 0, tr, con) {}
};
class TACSQuad4NonlinearShell : public TACSElement {
 public:
  TACSQuad4NonlinearShell(TACSShellTransform *tr, TACSShellConstitutive *con)
      : TACSElement(2, 1, tr, con) {}
};
class TACSQuad9NonlinearShell : public TACSElement {
 public:
  TACSQuad9NonlinearShell(TACSShellTransform *tr, TACSShellConstitutive *con)
      : TACSElement(3, 1, tr, con) {}
};

// TacsCreateShellByName (TACSShellElementDefs.h:77-105); names of element
// types the GB300 path does not implement (Quad16, ModRot) give NULL
inline TACSElement *TacsCreateShellByName(const char *name, TACSShellTransform *transform,
                                          TACSShellConstitutive *con) {
  if (!strcmp(name, "TACSQuad4Shell") || !strcmp(name, "CQUAD") || !strcmp(name, "CQUAD4") ||
      !strcmp(name, "CQUADR"))
    return new TACSQuad4Shell(transform, con);
  if (!strcmp(name, "TACSQuad9Shell") || !strcmp(name, "CQUAD9"))
    return new TACSQuad9Shell(transform, con);
  if (!strcmp(name, "TACSQuad4NonlinearShell")) return new TACSQuad4NonlinearShell(transform, con);
  if (!strcmp(name, "TACSQuad9NonlinearShell")) return new TACSQuad9NonlinearShell(transform, con);
  return nullptr;
}

/* -------------------------------------------------------------- vectors */
// TACSBVec on one process: node-major, vars_per_node interleaved values
class TACSVec : public TACSObject {};
class TACSBVec : public TACSVec {
 public:
  TACSBVec(int num_nodes, int vars_per_node) : v_((size_t)num_nodes * vars_per_node, 0.0) {}
  int getArray(TacsScalar **array) {
    *array = v_.data();
    return (int)v_.size();
  }
  int getSize() const { return (int)v_.size(); }
  void zeroEntries() { v_.assign(v_.size(), 0.0); }
  void set(TacsScalar a) { v_.assign(v_.size(), a); }
  void scale(TacsScalar a) {
    for (double &x : v_) x *= a;
  }
  void axpy(TacsScalar a, TACSBVec *x) {
    for (size_t i = 0; i < v_.size(); i++) v_[i] += a * x->v_[i];
  }
  void copyValues(TACSBVec *x) { v_ = x->v_; }
  TacsScalar dot(TACSBVec *x) const {
    double s = 0.0;
    for (size_t i = 0; i < v_.size(); i++) s += v_[i] * x->v_[i];
    return s;
  }
  TacsScalar norm() const;
  std::vector<double> &values() { return v_; }

 private:
  std::vector<double> v_;
};
inline TacsScalar TACSBVec::norm() const {
  double s = 0.0;
  for (double x : v_) s += x * x;
  return sqrt(s);
}

class TACSAssembler;

/* ------------------------------------------------------------- matrices */
// BCSRMat (src/bpmat/BCSRMat.h:34-204) on one process, 6x6 blocks, rows in
// the assembler's matrix ordering.  Two kinds, as in the reference: a view
// of an assembled matrix (TACSSchurMat::getBCSRMat), and a factor built as
// BCSRMat(comm, A, levFill, fill) (the ILU(levFill) pattern of A; copyValues
// then factor, applyFactor).  Raw vectors (mult, applyFactor) are in the
// row ordering, 6 values per row, as the reference's BCSRMat takes them.
class BCSRMat : public TACSObject {
 public:
  // a view of an a2ds_bcsr (the handle stays owned by its TACSSchurMat)
  BCSRMat(a2ds_mesh mesh, a2ds_bcsr A) : mesh_(mesh), A_(A) {}
  // BCSRMat(comm, A, levFill, fill): the factor object of A's pattern
  BCSRMat(MPI_Comm, BCSRMat *A, int levFill, double fill)
      : mesh_(A->mesh_), A_(A->A_), factor_(true) {
    (void)fill;
    a2ds_report("BCSRMat", a2ds_pc_create(A_, levFill, 64, &pc_));
  }
  ~BCSRMat() {
    if (pc_) a2ds_pc_destroy(pc_);
  }
  // getArrays(&bsize, &nrows, &ncols, &rowp, &cols, &A): host copies kept
  // by this object until the next call
  void getArrays(int *bsize, int *nrows, int *ncols, const int **rowp, const int **cols,
                 TacsScalar **A) {
    int n = 0, nz = 0;
    int rc = factor_ ? a2ds_pc_get(pc_, &n, &nz, nullptr, nullptr, nullptr)
                     : a2ds_bcsr_get(A_, &n, &nz, nullptr, nullptr, nullptr);
    rowp_.assign(n + 1, 0);
    cols_.assign(nz, 0);
    vals_.assign((size_t)nz * 36, 0.0);
    if (!rc)
      rc = factor_ ? a2ds_pc_get(pc_, nullptr, nullptr, rowp_.data(), cols_.data(), vals_.data())
                   : a2ds_bcsr_get(A_, nullptr, nullptr, rowp_.data(), cols_.data(),
                                   vals_.data());
    a2ds_report("BCSRMat::getArrays", rc);
    if (bsize) *bsize = 6;
    if (nrows) *nrows = n;
    if (ncols) *ncols = n;
    if (rowp) *rowp = rowp_.data();
    if (cols) *cols = cols_.data();
    if (A) *A = vals_.data();
  }
  // y = A x (BCSRMatVecMult6)
  void mult(TacsScalar *x, TacsScalar *y) {
    a2ds_report("BCSRMat::mult", a2ds_bcsr_mult_rows(A_, x, y));
  }
  // factor object: the values to factor next (BCSRMat::copyValues)
  void copyValues(BCSRMat *B) { from_ = B->A_; }
  // BCSRMatFactor6 of the copied values (the matrix it was built from if none)
  int factor() {
    if (!factor_) return a2ds_report("BCSRMat::factor", A2DS_ERR_STATE);
    return a2ds_report("BCSRMat::factor", a2ds_pc_factor(pc_, from_));
  }
  // y = (LU)^-1 x, BCSRMatApplyLower6 / Upper6 on row-ordered vectors
  void applyFactor(TacsScalar *x, TacsScalar *y) {
    if (!factor_) {
      a2ds_report("BCSRMat::applyFactor", A2DS_ERR_STATE);
      return;
    }
    int n = 0;
    a2ds_bcsr_get(A_, &n, nullptr, nullptr, nullptr, nullptr);
    std::vector<int> perm(n);
    a2ds_mesh_get_ordering(mesh_, perm.data());
    std::vector<double> xn((size_t)n * 6), yn((size_t)n * 6);
    for (int r = 0; r < n; r++)
      for (int k = 0; k < 6; k++) xn[(size_t)perm[r] * 6 + k] = x[(size_t)r * 6 + k];
    a2ds_report("BCSRMat::applyFactor", a2ds_pc_apply(pc_, xn.data(), yn.data()));
    for (int r = 0; r < n; r++)
      for (int k = 0; k < 6; k++) y[(size_t)r * 6 + k] = yn[(size_t)perm[r] * 6 + k];
  }
  a2ds_bcsr handle() const { return A_; }

 private:
  a2ds_mesh mesh_;
  a2ds_bcsr A_;
  a2ds_bcsr from_ = nullptr;
  a2ds_pc pc_ = nullptr;
  bool factor_ = false;
  std::vector<int> rowp_, cols_;
  std::vector<double> vals_;
};

class TACSMat : public TACSObject {};
class TACSSchurMat : public TACSMat {
 public:
  explicit TACSSchurMat(TACSAssembler *assembler);
  ~TACSSchurMat() {
    if (B_) B_->decref();
    if (h_) a2ds_bcsr_destroy(h_);
  }
  a2ds_bcsr handle() const { return h_; }
  // TACSSchurMat::getBCSRMat(&B, &E, &F, &C): on one process B is the whole
  // matrix and E, F, C are empty (NULL here)
  void getBCSRMat(BCSRMat **B, BCSRMat **E, BCSRMat **F, BCSRMat **C) {
    if (!B_) {
      B_ = new BCSRMat(mesh_, h_);
      B_->incref();
    }
    if (B) *B = B_;
    if (E) *E = nullptr;
    if (F) *F = nullptr;
    if (C) *C = nullptr;
  }
  // BCSRMat::mult through TACSSchurMat::mult, node-major vectors
  void mult(TACSBVec *x, TACSBVec *y) {
    a2ds_report("TACSSchurMat::mult",
                a2ds_bcsr_mult(h_, x->values().data(), y->values().data()));
  }
  void copyValues(TACSSchurMat *x) {
    a2ds_report("TACSSchurMat::copyValues", a2ds_bcsr_copy(h_, x->h_));
  }
  void axpy(TacsScalar alpha, TACSSchurMat *x) {
    a2ds_report("TACSSchurMat::axpy", a2ds_bcsr_axpy(h_, alpha, x->h_));
  }
  void applyBCs() { a2ds_report("TACSSchurMat::applyBCs", a2ds_bcsr_apply_bcs(h_)); }

 private:
  a2ds_bcsr h_ = nullptr;
  a2ds_mesh mesh_ = nullptr;
  BCSRMat *B_ = nullptr;
};

/* ------------------------------------------------- preconditioner, KSM */
class KSMPrint : public TACSObject {};
class KSMPrintStdout : public KSMPrint {
 public:
  KSMPrintStdout(const char *, int, int) {}
};

// TACSSchurPc(mat, levFill, fill, reorder) (src/bpmat/TACSSchurMat.h):
// ILU(levFill) of mat (levFill >= num_nodes: complete LU), FP64 values
// unless setPrecision is called (48: double-float, 32: FP32)
class TACSPc : public TACSObject {};
class TACSSchurPc : public TACSPc {
 public:
  TACSSchurPc(TACSSchurMat *mat, int levFill, double fill, int reorder_schur = 0)
      : mat_(nullptr), lev_(levFill), precision_(64) {
    a2ds_hold(mat_, mat);
    (void)fill;
    (void)reorder_schur;
  }
  ~TACSSchurPc() {
    if (pc_) a2ds_pc_destroy(pc_);
    if (mat_) mat_->decref();
  }
  void setPrecision(int p) { precision_ = p; }
  int getLevFill() const { return lev_; }
  int getPrecision() const { return precision_; }
  TACSSchurMat *getMat() { return mat_; }
  int factor() {
    int rc = 0;
    if (!pc_) rc = a2ds_pc_create(mat_->handle(), lev_, precision_, &pc_);
    if (!rc) rc = a2ds_pc_factor(pc_, nullptr);
    return a2ds_report("TACSSchurPc::factor", rc);
  }
  int applyFactor(TACSBVec *x, TACSBVec *y) {
    if (!pc_) {
      fprintf(stderr, "TACSSchurPc::applyFactor: call factor() first\n");
      return A2DS_ERR_STATE;
    }
    return a2ds_report("TACSSchurPc::applyFactor",
                       a2ds_pc_apply(pc_, x->values().data(), y->values().data()));
  }
  a2ds_pc handle() const { return pc_; }

 private:
  TACSSchurMat *mat_;
  a2ds_pc pc_ = nullptr;
  int lev_, precision_;
};

class TACSKsm : public TACSObject {};
// GMRES(mat, pc, m, nrestart, isFlexible) (src/bpmat/KSM.cpp:547-645)
class GMRES : public TACSKsm {
 public:
  GMRES(TACSSchurMat *mat, TACSSchurPc *pc, int m, int nrestart, int isFlexible)
      : mat_(nullptr), pc_(nullptr), m_(m), nrestart_(nrestart), rtol_(1e-8), atol_(1e-30) {
    a2ds_hold(mat_, mat);
    a2ds_hold(pc_, pc);
    (void)isFlexible;
  }
  ~GMRES() {
    if (mat_) mat_->decref();
    if (pc_) pc_->decref();
  }
  void setTolerances(double rtol, double atol) {
    rtol_ = rtol;
    atol_ = atol;
  }
  // right-preconditioned restarted GMRES with the factor pc holds
  int solve(TACSBVec *b, TACSBVec *x, int zero_guess = 1) {
    (void)zero_guess;
    int iters = 0;
    double res = 0.0;
    return a2ds_report("GMRES::solve",
                       a2ds_gmres_solve(mat_->handle(), pc_->handle(), m_, nrestart_, rtol_,
                                        atol_, b->values().data(), x->values().data(), &iters,
                                        &res));
  }
  TACSSchurPc *getPc() { return pc_; }
  int m() const { return m_; }
  int nrestart() const { return nrestart_; }
  double rtol() const { return rtol_; }
  double atol() const { return atol_; }

 private:
  TACSSchurMat *mat_;
  TACSSchurPc *pc_;
  int m_, nrestart_;
  double rtol_, atol_;
};

/* ------------------------------------------------------------ assembler */
class TACSAssembler : public TACSObject {
 public:
  enum OrderingType {
    NATURAL_ORDER = A2DS_NATURAL_ORDER,
    RCM_ORDER = A2DS_RCM_ORDER,
    AMD_ORDER = A2DS_AMD_ORDER,
    ND_ORDER = A2DS_ND_ORDER,
    TACS_AMD_ORDER = A2DS_TACS_AMD_ORDER,
    MULTICOLOR_ORDER = A2DS_MULTICOLOR_ORDER
  };

  // TACSAssembler(comm, varsPerNode, numOwnedNodes, numElements,
  // numDependentNodes) (src/TACSAssembler.h:81), then setElementConnectivity,
  // setElements and setNodes as the reference's drivers call them; the
  // device mesh is created when all three are given (at the latest by
  // initialize).  One process: 6 variables per node, no dependent nodes.
  TACSAssembler(MPI_Comm, int varsPerNode, int numOwnedNodes, int numElements,
                int numDependentNodes = 0)
      : nn_(numOwnedNodes), ne_(numElements), npe_(0), vars_((size_t)numOwnedNodes * 6, 0.0) {
    if (varsPerNode != 6 || numDependentNodes != 0) {
      fprintf(stderr, "TACSAssembler: 6 variables per node and no dependent nodes\n");
      fail_ = A2DS_ERR_ARG;
    }
  }
  // Mesh with one element object per element (elems[e], shared objects
  // allowed), node-major X, tensor-order connectivity, 0-based component
  // ids (for .f5 output; may be NULL): the sequence above in one call.
  TACSAssembler(int num_nodes, int num_elements, int nodes_per_elem, const int *conn,
                const double *X, TACSElement *const *elems, const int *elem_component)
      : nn_(num_nodes), ne_(num_elements), npe_(nodes_per_elem),
        conn_(conn, conn + (size_t)num_elements * nodes_per_elem), vars_(num_nodes * 6, 0.0),
        comp_(elem_component ? elem_component : nullptr,
              elem_component ? elem_component + num_elements : nullptr),
        X_(X, X + (size_t)num_nodes * 3) {
    elems_.assign(elems, elems + num_elements);
    for (TACSElement *e : elems_) e->incref();
    fail_ = create_mesh();
  }
  ~TACSAssembler() {
    for (TACSElement *e : elems_) e->decref();
    if (mesh_) a2ds_mesh_destroy(mesh_);
  }
  // setElementConnectivity(ptr, conn) (TACSAssembler.h:88): ptr[e+1] -
  // ptr[e] nodes per element, all 4 (Quad4) or all 9 (Quad9)
  int setElementConnectivity(const int *ptr, const int *conn) {
    if (mesh_) return a2ds_report("TACSAssembler::setElementConnectivity", A2DS_ERR_STATE);
    const int npe = ne_ > 0 ? ptr[1] - ptr[0] : 0;
    for (int e = 0; e < ne_; e++)
      if (ptr[e + 1] - ptr[e] != npe || (npe != 4 && npe != 9))
        return a2ds_report("TACSAssembler::setElementConnectivity", A2DS_ERR_ARG);
    npe_ = npe;
    conn_.assign(conn + ptr[0], conn + ptr[ne_]);
    return maybe_create();
  }
  // setElements(elements) (TACSAssembler.h:90)
  int setElements(TACSElement **elements) {
    if (mesh_) return a2ds_report("TACSAssembler::setElements", A2DS_ERR_STATE);
    for (TACSElement *e : elems_) e->decref();
    elems_.assign(elements, elements + ne_);
    for (TACSElement *e : elems_) e->incref();
    return maybe_create();
  }
  // setNodes(X) (TACSAssembler.h:156): node-major coordinates, before the
  // mesh exists (the device mesh keeps its coordinates)
  int setNodes(TACSBVec *X) {
    if (mesh_) return a2ds_report("TACSAssembler::setNodes", A2DS_ERR_STATE);
    X_ = X->values();
    return maybe_create();
  }
  int getNumNodes() const { return nn_; }
  int getNumElements() const { return ne_; }
  int getVarsPerNode() const { return 6; }
  TACSElement *getElement(int e) { return elems_[e]; }
  a2ds_mesh handle() const { return mesh_; }
  const std::vector<int> &components() const { return comp_; }

  // TACSAssembler::addBCs(nnodes, nodes, nbcs, vars, vals) (TACSAssembler.h:104)
  int addBCs(int nnodes, const int *nodes, int nbcs = -1, const int *vars = nullptr,
             const TacsScalar *vals = nullptr) {
    std::vector<int> masks(nnodes, 0);
    std::vector<double> v6((size_t)nnodes * 6, 0.0);
    for (int i = 0; i < nnodes; i++) {
      if (nbcs < 0 || !vars) {
        masks[i] = 0x3f;
      } else {
        for (int k = 0; k < nbcs; k++)
          if (vars[k] >= 0 && vars[k] < 6) {
            masks[i] |= 1 << vars[k];
            if (vals) v6[(size_t)i * 6 + vars[k]] = vals[k];
          }
      }
    }
    return addBCsMasked(nnodes, nodes, masks.data(), v6.data());
  }
  // one a2ds_mesh_add_bcs entry per (node, mask, values): the loader's form;
  // kept until the device mesh exists
  int addBCsMasked(int n, const int *nodes, const int *masks, const double *vals6) {
    if (!mesh_) {
      bc_nodes_.insert(bc_nodes_.end(), nodes, nodes + n);
      bc_masks_.insert(bc_masks_.end(), masks, masks + n);
      bc_vals_.insert(bc_vals_.end(), vals6, vals6 + (size_t)n * 6);
      return 0;
    }
    return a2ds_report("TACSAssembler::addBCs", a2ds_mesh_add_bcs(mesh_, n, nodes, masks, vals6));
  }
  int initialize(OrderingType order = TACS_AMD_ORDER) {
    if (initialized_) return 0;
    if (fail_) return fail_;
    if (!mesh_ && (fail_ = create_mesh())) return fail_;
    int rc = a2ds_report("TACSAssembler::initialize", a2ds_mesh_initialize(mesh_, (int)order));
    if (!rc) initialized_ = true;
    return rc;
  }

  TACSBVec *createVec() { return new TACSBVec(nn_, 6); }
  TACSBVec *createNodeVec() { return new TACSBVec(nn_, 3); }
  void getNodes(TACSBVec *X) { X->values().assign(X_.begin(), X_.end()); }
  // the first call fixes the matrix ordering (createSchurMat(order))
  TACSSchurMat *createSchurMat(OrderingType order = TACS_AMD_ORDER) {
    if (fail_ || initialize(order)) return nullptr;
    return new TACSSchurMat(this);
  }
  void setVariables(TACSBVec *u) { vars_ = u->values(); }
  void getVariables(TACSBVec *u) { u->values() = vars_; }
  void zeroVariables() { vars_.assign(vars_.size(), 0.0); }
  const std::vector<double> &variables() const { return vars_; }

  // thickness design variables: one per distinct constitutive object
  TACSBVec *createDesignVec() { return new TACSBVec((int)cons_.size(), 1); }
  void getDesignVars(TACSBVec *x) {
    for (size_t g = 0; g < cons_.size(); g++) x->values()[g] = cons_[g]->getThickness();
  }
  int setDesignVars(TACSBVec *x) {
    for (size_t g = 0; g < cons_.size(); g++)
      ((TACSIsoShellConstitutive *)cons_[g])->setThickness(x->values()[g]);
    return set_material_and_thickness();
  }

  // assembleMatType(type, mat) at the current variables (G: along them)
  int assembleMatType(ElementMatrixType type, TACSMat *A) {
    int rc = sync_temperature();
    if (!rc) rc = a2ds_assemble_mat(mesh_, (int)type, vars_.data(), mat_handle(A));
    return a2ds_report("TACSAssembler::assembleMatType", rc);
  }
  // assembleRes(res) at the current variables (no external loads)
  int assembleRes(TACSBVec *res) {
    int rc = sync_temperature();
    if (!rc) rc = a2ds_assemble_res(mesh_, vars_.data(), res->values().data());
    return a2ds_report("TACSAssembler::assembleRes", rc);
  }
  // assembleJacobian(alpha, beta, gamma, res, A, matOr, lambda)
  // (TACSAssembler.cpp:4084): res = R(u) and A = alpha dR/du at the current
  // variables, Dirichlet rows the identity.  The static shell path has no
  // velocity or acceleration variables, so beta and gamma (damping and
  // mass terms) must be 0; lambda scales auxiliary element loads, of which
  // this path has none; matOr: the normal orientation only.
  int assembleJacobian(TacsScalar alpha, TacsScalar beta, TacsScalar gamma, TACSBVec *res,
                       TACSMat *A, int matOr = 0, TacsScalar lambda = 1.0) {
    (void)lambda;
    if (beta != 0.0 || gamma != 0.0 || matOr != 0) {
      fprintf(stderr, "TACSAssembler::assembleJacobian: beta = gamma = 0 and the normal "
                      "orientation only (static shells)\n");
      return A2DS_ERR_ARG;
    }
    int rc = sync_temperature();
    a2ds_bcsr h = mat_handle(A);
    if (!rc)
      rc = a2ds_assemble_jacobian(mesh_, vars_.data(), res ? res->values().data() : nullptr, h);
    if (!rc && alpha != 1.0) {
      rc = a2ds_bcsr_axpy(h, alpha - 1.0, h);     // A <- alpha A
      if (!rc) rc = a2ds_bcsr_apply_bcs(h);         // identity Dirichlet rows again
    }
    return a2ds_report("TACSAssembler::assembleJacobian", rc);
  }

  int sync_temperature() {
    double T = elems_.empty() ? 0.0 : elems_[0]->getTemperature();
    for (TACSElement *e : elems_)
      if (e->getTemperature() != T) {
        fprintf(stderr, "TACSAssembler: elements must share one temperature\n");
        return A2DS_ERR_ARG;
      }
    if (T == temperature_) return 0;
    temperature_ = T;
    return set_material_and_thickness();
  }

 private:
  static a2ds_bcsr mat_handle(TACSMat *A) {
    TACSSchurMat *s = dynamic_cast<TACSSchurMat *>(A);
    return s ? s->handle() : nullptr;
  }
  int set_material_and_thickness() {
    if (elems_.empty()) return a2ds_report("TACSAssembler", A2DS_ERR_ARG);
    TACSMaterialProperties *p = elems_[0]->getConstitutive()->getMaterialProperties();
    std::vector<int> group(ne_);
    cons_.clear();
    for (int e = 0; e < ne_; e++) {
      TACSShellConstitutive *c = elems_[e]->getConstitutive();
      TACSMaterialProperties *q = c->getMaterialProperties();
      if (q->E != p->E || q->nu != p->nu || q->alpha != p->alpha) {
        fprintf(stderr, "TACSAssembler: elements must share one material\n");
        return A2DS_ERR_ARG;
      }
      size_t g = 0;
      while (g < cons_.size() && cons_[g] != c) g++;
      if (g == cons_.size()) cons_.push_back(c);
      group[e] = (int)g;
    }
    std::vector<double> t(cons_.size());
    for (size_t g = 0; g < cons_.size(); g++) t[g] = cons_[g]->getThickness();
    int rc = a2ds_mesh_set_material(mesh_, p->E, p->nu, p->alpha, temperature_);
    if (!rc) rc = a2ds_mesh_set_yield_stress(mesh_, p->ys);
    if (!rc) rc = a2ds_mesh_set_thickness(mesh_, (int)t.size(), t.data(), group.data());
    return a2ds_report("TACSAssembler", rc);
  }

  int maybe_create() {
    if (fail_) return fail_;
    if (npe_ && !elems_.empty() && X_.size() == (size_t)nn_ * 3) fail_ = create_mesh();
    return fail_;
  }
  int create_mesh() {
    if (mesh_) return 0;
    if (!npe_ || elems_.size() != (size_t)ne_ || X_.size() != (size_t)nn_ * 3) {
      fprintf(stderr, "TACSAssembler: connectivity, elements and nodes must all be set\n");
      return A2DS_ERR_STATE;
    }
    const int nl = elems_[0]->nonlinear();
    int rc = a2ds_report("TACSAssembler",
                         a2ds_mesh_create(nn_, ne_, npe_, conn_.data(), X_.data(), nl, &mesh_));
    if (!rc) rc = set_material_and_thickness();
    if (!rc && !bc_nodes_.empty()) {
      rc = a2ds_report("TACSAssembler::addBCs",
                       a2ds_mesh_add_bcs(mesh_, (int)bc_nodes_.size(), bc_nodes_.data(),
                                         bc_masks_.data(), bc_vals_.data()));
      bc_nodes_.clear();
      bc_masks_.clear();
      bc_vals_.clear();
    }
    return rc;
  }

  int nn_, ne_, npe_;
  a2ds_mesh mesh_ = nullptr;
  std::vector<int> conn_, bc_nodes_, bc_masks_;
  std::vector<double> bc_vals_;
  int fail_ = 0;
  bool initialized_ = false;
  double temperature_ = 0.0;
  std::vector<double> vars_;
  std::vector<int> comp_;
  std::vector<double> X_;
  std::vector<TACSElement *> elems_;
  std::vector<TACSShellConstitutive *> cons_;
};

inline TACSSchurMat::TACSSchurMat(TACSAssembler *assembler) : mesh_(assembler->handle()) {
  a2ds_report("TACSSchurMat", a2ds_bcsr_create(assembler->handle(), &h_));
}

/* -------------------------------------------------------------- buckling */
// TACSLinearBuckling(assembler, sigma, gmat, kmat, aux_mat, solver,
// max_lanczos, num_eigvals, eig_tol) (src/TACSBuckling.cpp:51-134): the
// solver's GMRES settings and its TACSSchurPc's level of fill and precision
// select the solve (complete fill: direct factors of K + sigma G with FP64
// refinement; ILU(k): GMRES preconditioned by the factor of K)
class TACSLinearBuckling : public TACSObject {
 public:
  TACSLinearBuckling(TACSAssembler *assembler, TacsScalar sigma, TACSMat *gmat, TACSMat *kmat,
                     TACSMat *aux_mat, TACSKsm *ksm, int max_lanczos, int num_eigvals,
                     double eig_tol)
      : assembler_(nullptr) {
    GMRES *solver = dynamic_cast<GMRES *>(ksm);
    a2ds_hold(assembler_, assembler);
    a2ds_hold(gmat_, dynamic_cast<TACSSchurMat *>(gmat));
    a2ds_hold(kmat_, dynamic_cast<TACSSchurMat *>(kmat));
    a2ds_hold(aux_, dynamic_cast<TACSSchurMat *>(aux_mat));
    a2ds_buckling_default_opts(&opts_);
    opts_.sigma = sigma;
    opts_.max_lanczos = max_lanczos;
    opts_.num_eigvals = num_eigvals;
    opts_.eig_tol = eig_tol;
    if (solver) {
      opts_.gmres_m = solver->m();
      opts_.gmres_restarts = solver->nrestart();
      opts_.gmres_rtol = solver->rtol();
      opts_.gmres_atol = solver->atol();
      if (solver->getPc()) {
        opts_.lev_fill = solver->getPc()->getLevFill();
        opts_.precision = solver->getPc()->getPrecision();
      }
    }
  }
  ~TACSLinearBuckling() {
    if (assembler_) assembler_->decref();
    if (gmat_) gmat_->decref();
    if (kmat_) kmat_->decref();
    if (aux_) aux_->decref();
  }
  // GB300 settings without a counterpart in the reference
  void setBlockSize(int p) { opts_.block_size = p; }
  void setPrecision(int precision) { opts_.precision = precision; }
  TacsScalar getSigma() const { return opts_.sigma; }
  void setSigma(TacsScalar sigma) { opts_.sigma = sigma; }

  // solve(rhs, u0, print) (src/TACSBuckling.cpp:197-278): rhs NULL = the
  // load path from the prescribed Dirichlet values alone
  int solve(TACSVec *rhs = nullptr, TACSVec *u0 = nullptr, KSMPrint *print = nullptr) {
    (void)u0;
    (void)print;
    int rc = assembler_->sync_temperature();
    if (rc) return rc;
    const int n = opts_.num_eigvals, nn = assembler_->getNumNodes();
    eig_.assign(n, 0.0);
    err_.assign(n, 0.0);
    vecs_.assign((size_t)n * nn * 6, 0.0);
    path_.assign((size_t)nn * 6, 0.0);
    TACSBVec *f = dynamic_cast<TACSBVec *>(rhs);
    rc = a2ds_buckling_solve(assembler_->handle(), &opts_, f ? f->values().data() : nullptr,
                             eig_.data(), err_.data(), vecs_.data(), path_.data());
    // as the reference leaves them: kmat = K at the zero state, gmat = G
    // along the load path, aux_mat = K + sigma G (Dirichlet rows applied);
    // the assembler's variables hold the path
    a2ds_mesh h = assembler_->handle();
    if ((!rc || rc == A2DS_ERR_NOCONV) && kmat_)
      rc = keep_rc(rc, a2ds_assemble_mat(h, A2DS_STIFFNESS_MATRIX, nullptr, kmat_->handle()));
    if ((!rc || rc == A2DS_ERR_NOCONV) && gmat_)
      rc = keep_rc(rc, a2ds_assemble_mat(h, A2DS_GEOMETRIC_STIFFNESS_MATRIX, path_.data(),
                                         gmat_->handle()));
    if ((!rc || rc == A2DS_ERR_NOCONV) && aux_ && kmat_ && gmat_) {
      rc = keep_rc(rc, a2ds_bcsr_copy(aux_->handle(), kmat_->handle()));
      rc = keep_rc(rc, a2ds_bcsr_axpy(aux_->handle(), opts_.sigma, gmat_->handle()));
      rc = keep_rc(rc, a2ds_bcsr_apply_bcs(aux_->handle()));
    }
    TACSBVec path(assembler_->getNumNodes(), 6);
    path.values() = path_;
    assembler_->setVariables(&path);
    return a2ds_report("TACSLinearBuckling::solve", rc);
  }
  // checkEigenvector(n) (src/TACSBuckling.cpp:310-349): prints ||K e||,
  // ||G e|| and ||K e + lambda G e|| with the kmat and gmat of the last
  // solve (given to the constructor); returns the relative residual
  // ||K e + lambda G e|| / ||K e|| (the reference returns nothing)
  double checkEigenvector(int n) {
    if (!kmat_ || !gmat_ || n < 0 || n >= (int)eig_.size()) {
      fprintf(stderr, "TACSLinearBuckling::checkEigenvector: needs kmat, gmat and a solve\n");
      return -1.0;
    }
    const int nn = assembler_->getNumNodes();
    TACSBVec e(nn, 6), t1(nn, 6), t2(nn, 6);
    TacsScalar err = 0.0;
    TacsScalar eig = extractEigenvector(n, &e, &err);
    kmat_->mult(&e, &t1);
    gmat_->mult(&e, &t2);
    const double t1n = t1.norm(), t2n = t2.norm();
    printf("|K*e| = %15.5e  \n|G*e| = %15.5e \n", t1n, t2n);
    t1.axpy(eig, &t2);
    const double rn = t1.norm();
    printf("||K*e + lambda*G*e|| = %15.5e \n", rn);
    return t1n > 0.0 ? rn / t1n : rn;
  }
  TacsScalar extractEigenvalue(int n, TacsScalar *error) {
    if (n < 0 || n >= (int)eig_.size()) return 0.0;
    if (error) *error = err_[n];
    return eig_[n];
  }
  TacsScalar extractEigenvector(int n, TACSBVec *ans, TacsScalar *error) {
    if (n < 0 || n >= (int)eig_.size()) return 0.0;
    const size_t nv = path_.size();
    ans->values().assign(vecs_.begin() + n * nv, vecs_.begin() + (n + 1) * nv);
    if (error) *error = err_[n];
    return eig_[n];
  }
  // the load path of the last solve
  void getPath(TACSBVec *u) { u->values() = path_; }
  // evalEigenDVSens / evalEigenXptSens (bodies commented out in the
  // reference, src/TACSBuckling.cpp:359-497): thickness groups / nodes x 3
  int evalEigenDVSens(int n, TACSBVec *dfdx) {
    return a2ds_report("TACSLinearBuckling::evalEigenDVSens",
                       a2ds_eig_sens_thickness(assembler_->handle(), n, dfdx->values().data()));
  }
  int evalEigenXptSens(int n, TACSBVec *dfdX) {
    return a2ds_report("TACSLinearBuckling::evalEigenXptSens",
                       a2ds_eig_sens_xpts(assembler_->handle(), n, 0.0, dfdX->values().data()));
  }

 private:
  static int keep_rc(int rc, int next) { return rc ? rc : next; }
  TACSAssembler *assembler_;
  TACSSchurMat *gmat_ = nullptr, *kmat_ = nullptr, *aux_ = nullptr;
  a2ds_buckling_opts opts_;
  std::vector<double> eig_, err_, vecs_, path_;
};

/* ---------------------------------------------------------- mesh loader */
class TACSMeshLoader : public TACSObject {
 public:
  explicit TACSMeshLoader(MPI_Comm comm = MPI_COMM_WORLD) { (void)comm; }
  ~TACSMeshLoader() {
    for (TACSElement *e : elems_)
      if (e) e->decref();
    if (bdf_) a2ds_bdf_destroy(bdf_);
  }
  // scanBDFFile (src/io/TACSMeshLoader.cpp:569-1098)
  int scanBDFFile(const char *file_name) {
    int rc = a2ds_bdf_scan(file_name, &bdf_);
    if (!rc) rc = a2ds_bdf_get_sizes(bdf_, &nn_, &ne_, &conn_size_, &nbcs_, &bcv_size_, &ncomp_);
    if (rc) return a2ds_report("TACSMeshLoader::scanBDFFile", rc);
    elems_.assign(ncomp_, nullptr);
    names_.assign(ncomp_, std::string());
    descripts_.assign(ncomp_, std::string());
    char buf[256];
    for (int c = 0; c < ncomp_; c++) {
      if (!a2ds_bdf_get_element_descript(bdf_, c, buf, sizeof(buf))) names_[c] = buf;
      if (!a2ds_bdf_get_component_descript(bdf_, c, buf, sizeof(buf))) descripts_[c] = buf;
    }
    return 0;
  }
  int getNumComponents() const { return ncomp_; }
  int getNumNodes() const { return nn_; }
  int getNumElements() const { return ne_; }
  const char *getElementDescript(int c) const { return names_[c].c_str(); }
  const char *getComponentDescript(int c) const { return descripts_[c].c_str(); }
  void setElement(int c, TACSElement *elem) {
    if (c >= 0 && c < ncomp_) a2ds_hold(elems_[c], elem);
  }
  // createTACS(vars_per_node) with the SPC entries as boundary conditions
  TACSAssembler *createTACS(int vars_per_node,
                            TACSAssembler::OrderingType order = TACSAssembler::NATURAL_ORDER) {
    (void)order;  // the matrix ordering is chosen by createSchurMat
    if (vars_per_node != 6 || !bdf_) {
      fprintf(stderr, "TACSMeshLoader::createTACS: needs a scanned BDF and 6 vars per node\n");
      return nullptr;
    }
    std::vector<int> ptr(ne_ + 1), conn(conn_size_), comp(ne_);
    std::vector<double> X((size_t)nn_ * 3);
    if (a2ds_report("TACSMeshLoader::createTACS",
                    a2ds_bdf_get_connectivity(bdf_, ptr.data(), conn.data(), comp.data(),
                                              X.data())))
      return nullptr;
    const int npe = ne_ ? ptr[1] - ptr[0] : 0;
    std::vector<TACSElement *> elems(ne_);
    for (int e = 0; e < ne_; e++) {
      TACSElement *el = elems_[comp[e]];
      if (!el || ptr[e + 1] - ptr[e] != npe || el->getNumNodes() != npe ||
          el->nonlinear() != elems_[comp[0]]->nonlinear()) {
        fprintf(stderr, "TACSMeshLoader::createTACS: every component needs a shell element "
                        "object of one type matching its cards\n");
        return nullptr;
      }
      elems[e] = el;
    }
    TACSAssembler *a =
        new TACSAssembler(nn_, ne_, npe, conn.data(), X.data(), elems.data(), comp.data());
    std::vector<int> bnodes(nbcs_), bvars(bcv_size_), bptr(nbcs_ + 1);
    std::vector<double> bvals(bcv_size_);
    if (nbcs_ && !a2ds_report("TACSMeshLoader::createTACS",
                              a2ds_bdf_get_bcs(bdf_, bnodes.data(), bvars.data(), bptr.data(),
                                               bvals.data()))) {
      std::vector<int> masks(nbcs_, 0);
      std::vector<double> v6((size_t)nbcs_ * 6, 0.0);
      for (int b = 0; b < nbcs_; b++)
        for (int q = bptr[b]; q < bptr[b + 1]; q++)
          if (bvars[q] >= 0 && bvars[q] < 6) {
            masks[b] |= 1 << bvars[q];
            v6[(size_t)b * 6 + bvars[q]] = bvals[q];
          }
      a->addBCsMasked(nbcs_, bnodes.data(), masks.data(), v6.data());
    }
    return a;
  }

 private:
  a2ds_bdf bdf_ = nullptr;
  int nn_ = 0, ne_ = 0, conn_size_ = 0, nbcs_ = 0, bcv_size_ = 0, ncomp_ = 0;
  std::vector<TACSElement *> elems_;
  std::vector<std::string> names_, descripts_;
};

/* ------------------------------------------------------------ .f5 output */
// TACSToFH5(assembler, TACS_BEAM_OR_SHELL_ELEMENT, write_flag)
// (src/io/TACSToFH5.cpp:35-358): writes the assembler's current variables
class TACSToFH5 : public TACSObject {
 public:
  TACSToFH5(TACSAssembler *assembler, ElementType type, int write_flag)
      : assembler_(nullptr), flag_(write_flag) {
    a2ds_hold(assembler_, assembler);
    (void)type;
  }
  ~TACSToFH5() {
    if (assembler_) assembler_->decref();
  }
  void setComponentName(int comp, const char *name) {
    if (comp < 0) return;
    if ((int)names_.size() <= comp) names_.resize(comp + 1);
    names_[comp] = name ? name : "";
  }
  int writeToFile(const char *file_name) {
    const std::vector<int> &comp = assembler_->components();
    int ncomp = (int)names_.size();
    for (int c : comp) ncomp = c + 1 > ncomp ? c + 1 : ncomp;
    std::vector<const char *> ptrs(ncomp, nullptr);
    for (int c = 0; c < (int)names_.size(); c++) ptrs[c] = names_[c].c_str();
    int rc = assembler_->sync_temperature();
    if (!rc)
      rc = a2ds_write_f5(assembler_->handle(), file_name, flag_, ncomp, ptrs.data(),
                         comp.empty() ? nullptr : comp.data(),
                         assembler_->variables().data(), 0.0);
    return a2ds_report("TACSToFH5::writeToFile", rc);
  }

 private:
  TACSAssembler *assembler_;
  int flag_;
  std::vector<std::string> names_;
};

}  // namespace a2ds_tacs

#endif
