"""Regenerate the golden fixtures in this directory from the reference itself.

Builds the reference's own C++ sources into oracle/_ref (oracle/ref/Makefile),
runs its fixture generator (oracle/ref/golden_gen.cpp, real and complex-step
builds) and packs inputs and outputs into small .npz files:

  elements_<TYPE>.npz   per-element K, G (finite-difference and complex-step),
                        residual and Jacobian for 6 seeded elements of each of
                        TACSQuad4Shell, TACSQuad4NonlinearShell,
                        TACSQuad9Shell, TACSQuad9NonlinearShell
  <case>.npz            a seeded cylinder or stiffened panel: mesh and loads (inputs), the
                        reference's node CSR, AMD permutation, BCSR pattern,
                        assembled K and G, ILU pattern and factor, load path
                        and buckling eigenpairs
  bdf_*.bdf, bdf.npz    synthetic Nastran decks (bdf_cases.py) and the
                        reference loader's arrays for each
  f5.npz                .f5 files of the reference's TACSToFH5 (raw bytes)
                        for two seeded meshes and nine output-class flags

Only a machine with the reference sources can run it; the fixtures are committed so
the tests never need them.  Run:  python tests/golden/make_golden.py [part ...]
(parts: the make_* names without the prefix, e.g. config1; default all).
"""
from __future__ import annotations

import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(REPO, "a2d-shells_gb300"))
sys.path.insert(0, HERE)

from a2ds import mesh as meshgen  # noqa: E402

REF_OUT = os.path.join(REPO, "oracle", "_ref")
ELEMENT_TYPES = ["TACSQuad4Shell", "TACSQuad4NonlinearShell",
                 "TACSQuad9Shell", "TACSQuad9NonlinearShell"]


def build_reference():
    subprocess.run(["make", "-s", "-j8", "-C", os.path.join(REPO, "oracle", "ref"),
                    f"OUT={REF_OUT}", os.path.join(REF_OUT, "golden_gen"),
                    os.path.join(REF_OUT, "golden_gen_cplx")], check=True)


def load_dir(d):
    return {f[:-4]: np.load(os.path.join(d, f)) for f in os.listdir(d) if f.endswith(".npy")}


def make_elements():
    with tempfile.TemporaryDirectory() as d:
        subprocess.run([os.path.join(REF_OUT, "golden_gen"), "element", d], check=True)
        subprocess.run([os.path.join(REF_OUT, "golden_gen_cplx"), "element", d], check=True)
        arrs = load_dir(d)
    for name in ELEMENT_TYPES:
        pre = name + "_"
        out = {k[len(pre):]: v for k, v in arrs.items() if k.startswith(pre)}
        np.savez_compressed(os.path.join(HERE, f"elements_{name}.npz"), **out)
        print("wrote", f"elements_{name}.npz", sorted(out))


def write_inputs(d, m: meshgen.ShellMesh, sigma, lev, gm_m, gm_restarts, lanczos, neig,
                 nonlinear=0, gm_tol=1e-12, temperature=0.0, alpha_t=0.0):
    np.save(os.path.join(d, "X.npy"), np.ascontiguousarray(m.X, dtype=np.float64))
    np.save(os.path.join(d, "conn.npy"), np.ascontiguousarray(m.conn, dtype=np.int32))
    np.save(os.path.join(d, "bc_nodes.npy"), m.bc_nodes.astype(np.int32))
    np.save(os.path.join(d, "bc_mask.npy"), m.bc_mask.astype(np.int32))
    np.save(os.path.join(d, "bc_vals.npy"), np.ascontiguousarray(m.bc_vals, dtype=np.float64))
    np.save(os.path.join(d, "rhs.npy"), np.ascontiguousarray(m.rhs, dtype=np.float64))
    np.save(os.path.join(d, "elem_thickness.npy"), m.thickness.astype(np.float64))
    prm = np.array([m.E, m.nu, sigma, lev, gm_m, gm_restarts, lanczos, neig, nonlinear,
                    gm_tol, temperature, alpha_t], dtype=np.float64)
    np.save(os.path.join(d, "params.npy"), prm)


def dense_eigs(fx, neig):
    """Lowest buckling loads of K x + lam G x = 0 on the free DOFs (dense)."""
    import scipy.linalg as sla
    n = fx["bcsr_rowp"].size - 1
    rowp, cols = fx["bcsr_rowp"], fx["bcsr_cols"]

    def dense(vals):
        A = np.zeros((6 * n, 6 * n))
        for i in range(n):
            for jp in range(rowp[i], rowp[i + 1]):
                j = cols[jp]
                A[6 * i:6 * i + 6, 6 * j:6 * j + 6] = vals[jp]
        return A
    K, G = dense(fx["K_after"]), dense(fx["G"])
    perm = fx["amd_perm"]
    bcdof = np.zeros(6 * n, bool)
    inv = np.empty(n, np.int64)
    inv[perm] = np.arange(n)
    for node, mask in zip(fx["bc_nodes"], fx["bc_mask"]):
        for k in range(6):
            if mask >> k & 1:
                bcdof[6 * inv[node] + k] = True
    free = ~bcdof
    Kf = 0.5 * (K[np.ix_(free, free)] + K[np.ix_(free, free)].T)
    Gf = 0.5 * (G[np.ix_(free, free)] + G[np.ix_(free, free)].T)
    mu = sla.eigh(-Gf, Kf, eigvals_only=True)      # mu = 1/lambda
    lam = 1.0 / mu[mu > 0]
    lam = np.sort(lam)
    return lam[:neig]


def run_case(name, m, lev, gm_m, gm_restarts, lanczos, neig, sigma=None, nonlinear=0,
             temperature=0.0, alpha_t=0.0, drop=()):
    with tempfile.TemporaryDirectory() as d:
        ind, outd = os.path.join(d, "in"), os.path.join(d, "out")
        os.makedirs(ind)
        os.makedirs(outd)
        s0 = sigma if sigma is not None else 1e4
        write_inputs(ind, m, s0, lev, gm_m, gm_restarts, lanczos, neig, nonlinear,
                     temperature=temperature, alpha_t=alpha_t)
        subprocess.run([os.path.join(REF_OUT, "golden_gen"), "assembly", ind, outd], check=True)
        fx = load_dir(outd)
        fx.update(bc_nodes=m.bc_nodes, bc_mask=m.bc_mask)
        lam_dense = dense_eigs(fx, neig)
        if sigma is None:
            # Second pass with the shift just below the lowest dense eigenvalue
            sigma = 0.95 * lam_dense[0]
            write_inputs(ind, m, sigma, lev, gm_m, gm_restarts, lanczos, neig, nonlinear,
                         temperature=temperature, alpha_t=alpha_t)
            subprocess.run([os.path.join(REF_OUT, "golden_gen"), "assembly", ind, outd],
                           check=True)
        subprocess.run([os.path.join(REF_OUT, "golden_gen_cplx"), "assembly", ind, outd],
                       check=True)
        fx = load_dir(outd)
    out = dict(fx)
    out.update(X=m.X, conn=m.conn, bc_nodes=m.bc_nodes, bc_mask=m.bc_mask, bc_vals=m.bc_vals,
               rhs=m.rhs, thickness=m.thickness, E=np.float64(m.E), nu=np.float64(m.nu),
               sigma=np.float64(sigma), lev=np.int32(lev), gm_m=np.int32(gm_m),
               gm_restarts=np.int32(gm_restarts), lanczos=np.int32(lanczos),
               neig=np.int32(neig), nonlinear=np.int32(nonlinear),
               temperature=np.float64(temperature), alpha_t=np.float64(alpha_t),
               eigvals_dense=lam_dense)
    for k in drop:
        out.pop(k, None)
    np.savez_compressed(os.path.join(HERE, f"{name}.npz"), **out)
    rel = np.abs(out["eigvals"][:3] - lam_dense[:3]) / lam_dense[:3]
    print("wrote", f"{name}.npz", "nnzb", out["bcsr_cols"].size, "eig", out["eigvals"][:3],
          "dense", lam_dense[:3], "rel", rel)


def make_orderings():
    """Orderings of the three fixture meshes' node graphs by the reference's
    own routines (RCM, serial multicolouring, AMD with the diagonal)."""
    cases = {"cyl_q4_4x8": meshgen.cylinder(4, 8, order=2),
             "cyl_q4_8x16": meshgen.cylinder(8, 16, order=2),
             "cyl_q9_2x4": meshgen.cylinder(2, 4, order=3),
             "cyl_q4_16x32": meshgen.cylinder(16, 32, order=2)}
    out = {}
    for name, m in cases.items():
        with tempfile.TemporaryDirectory() as d:
            ind, outd = os.path.join(d, "in"), os.path.join(d, "out")
            os.makedirs(ind)
            os.makedirs(outd)
            np.save(os.path.join(ind, "X.npy"), np.ascontiguousarray(m.X, np.float64))
            np.save(os.path.join(ind, "conn.npy"), np.ascontiguousarray(m.conn, np.int32))
            subprocess.run([os.path.join(REF_OUT, "golden_gen"), "orderings", ind, outd],
                           check=True)
            for k, v in load_dir(outd).items():
                out[f"{name}__{k}"] = v
            out[f"{name}__X"] = m.X
            out[f"{name}__conn"] = m.conn
    np.savez_compressed(os.path.join(HERE, "orderings.npz"), **out)
    print("wrote orderings.npz")


def thermal_cylinder(nx, ny):
    """Both ends clamped, no mechanical load: uniform heating (temperature
    with a thermal expansion coefficient) compresses the shell axially, as in
    the reference's thermal buckling example."""
    m = meshgen.cylinder(nx, ny, order=2)
    x = m.X[:, 0]
    ends = np.where((np.abs(x) < 1e-12) | (np.abs(x - x.max()) < 1e-12))[0].astype(np.int32)
    m.bc_nodes = ends
    m.bc_mask = np.full(ends.size, 63, np.int32)
    m.bc_vals = np.zeros((ends.size, 6))
    m.rhs = np.zeros_like(m.rhs)
    return m


def make_thermal():
    run_case("cyl_q4_4x8_thermal", thermal_cylinder(4, 8), lev=1000000, gm_m=10,
             gm_restarts=15, lanczos=100, neig=50, temperature=10.0, alpha_t=1e-5)


def parse_bdf_reference(path):
    """The reference loader's arrays for one deck (golden_gen bdf)."""
    with tempfile.TemporaryDirectory() as d:
        subprocess.run([os.path.join(REF_OUT, "golden_gen"), "bdf", path, d], check=True)
        return load_dir(d)


def make_bdf():
    """Synthetic decks (bdf_cases.py) written here, the reference loader's
    arrays for each in bdf.npz, and a buckling case on the cylinder deck's
    parsed mesh (displacement control through nonzero SPC values)."""
    import bdf_cases
    decks = {"bdf_mixed": bdf_cases.mixed_deck(), "bdf_plain": bdf_cases.plain_deck(),
             "bdf_cyl_q4_8x16": bdf_cases.cylinder_deck(meshgen.cylinder(8, 16, order=2))}
    out = {}
    for name, text in decks.items():
        path = os.path.join(HERE, name + ".bdf")
        with open(path, "w", newline="") as f:
            f.write(text)
        for k, v in parse_bdf_reference(path).items():
            out[f"{name}__{k}"] = v
    np.savez_compressed(os.path.join(HERE, "bdf.npz"), **out)
    print("wrote bdf.npz")
    # the cylinder deck's mesh as the reference loader returns it
    pre = "bdf_cyl_q4_8x16__"
    ptr, conn = out[pre + "elem_node_ptr"], out[pre + "elem_node_conn"]
    X = out[pre + "Xpts"]
    nodes, var, bptr, vals = (out[pre + "bc_nodes"], out[pre + "bc_vars"], out[pre + "bc_ptr"],
                              out[pre + "bc_vals"])
    mask = np.zeros(nodes.size, np.int32)
    v6 = np.zeros((nodes.size, 6))
    for b in range(nodes.size):
        for q in range(bptr[b], bptr[b + 1]):
            if var[q] < 6:
                mask[b] |= 1 << int(var[q])
                v6[b, var[q]] = vals[q]
    ne = ptr.size - 1
    m = meshgen.ShellMesh(X=X, conn=conn.reshape(ne, 4), bc_nodes=nodes.astype(np.int32),
                          bc_mask=mask, bc_vals=v6, rhs=np.zeros((X.shape[0], 6)),
                          thickness=np.full(ne, 2e-3), dv_group=np.zeros(ne, np.int32))
    run_case("bdf_cyl_q4_8x16_lu", m, lev=1000000, gm_m=10, gm_restarts=15, lanczos=100,
             neig=20)


def make_f5():
    """.f5 files written by the reference's TACSToFH5 for a Quad4 and a Quad9
    cylinder and a Quad9 stiffened panel (skin and webs), each with two
    components and a seeded variable vector, for nine
    output-class flags (node, element and load classes); stored as raw
    bytes in f5.npz with the inputs."""
    rng = np.random.default_rng(11)
    out = {}
    for name, m in {"q4": meshgen.cylinder(4, 8, order=2),
                    "q9": meshgen.cylinder(2, 4, order=3),
                    "panel": meshgen.stiffened_panel(2, 8, 1)}.items():
        if name == "panel":  # skin and webs as the two components
            comp = (np.arange(m.num_elements) >= 2 * 8).astype(np.int32)
        else:
            comp = (np.arange(m.num_elements) % 3 == 1).astype(np.int32)
        vars_ = rng.standard_normal((m.num_nodes, 6)) * 1e-3
        with tempfile.TemporaryDirectory() as d:
            ind, outd = os.path.join(d, "in"), os.path.join(d, "out")
            os.makedirs(ind)
            os.makedirs(outd)
            np.save(os.path.join(ind, "X.npy"), np.ascontiguousarray(m.X, np.float64))
            np.save(os.path.join(ind, "conn.npy"), np.ascontiguousarray(m.conn, np.int32))
            np.save(os.path.join(ind, "comp.npy"), comp)
            np.save(os.path.join(ind, "vars.npy"), vars_)
            subprocess.run([os.path.join(REF_OUT, "golden_gen"), "f5", ind, outd], check=True)
            for f in sorted(os.listdir(outd)):
                with open(os.path.join(outd, f), "rb") as fh:
                    out[f"{name}__{f[:-3]}"] = np.frombuffer(fh.read(), np.uint8)
        out.update({f"{name}__X": m.X, f"{name}__conn": m.conn, f"{name}__comp": comp,
                    f"{name}__vars": vars_})
    np.savez_compressed(os.path.join(HERE, "f5.npz"), **out)
    print("wrote f5.npz", sorted(k for k in out if "f5_" in k))


def sparse_eigs(fx, neig, sigma):
    """Lowest buckling loads of K x + lam G x = 0 on the free DOFs by a
    sparse shift-invert eigensolve (scipy ARPACK, tolerance 1e-14) of the
    reference's own assembled K and G: the dense solve's role for meshes too
    large for dense FP64 (the symmetric parts, as in dense_eigs)."""
    import scipy.sparse as sp
    import scipy.sparse.linalg as sla
    n = fx["bcsr_rowp"].size - 1
    rowp, cols = fx["bcsr_rowp"], fx["bcsr_cols"]
    K = sp.bsr_matrix((fx["K_after"], cols, rowp), shape=(6 * n, 6 * n)).tocsr()
    G = sp.bsr_matrix((fx["G"], cols, rowp), shape=(6 * n, 6 * n)).tocsr()
    perm = fx["amd_perm"]
    inv = np.empty(n, np.int64)
    inv[perm] = np.arange(n)
    bcdof = np.zeros(6 * n, bool)
    for node, mask in zip(fx["bc_nodes"], fx["bc_mask"]):
        for k in range(6):
            if mask >> k & 1:
                bcdof[6 * inv[node] + k] = True
    free = np.where(~bcdof)[0]
    Kf = K[free][:, free]
    Gf = G[free][:, free]
    Kf = (0.5 * (Kf + Kf.T)).tocsc()
    Gf = (0.5 * (Gf + Gf.T)).tocsc()
    # K x = lam (-G) x, shift-invert about sigma (K - sigma (-G)) = K + sigma G
    vals = sla.eigsh(Kf, k=2 * neig, M=-Gf, sigma=sigma, which="LM", tol=1e-14,
                     return_eigenvectors=False, mode="buckling")
    vals = np.sort(vals[vals > 0])
    return vals[:neig]


def make_config1():
    """The reference's CPU-runnable workload: the 32 x 64 Quad4 cylinder (2,112
    nodes, 12,672 DOF).  The reference solves it as its cylinder example does
    (complete LU of K, GMRES(10, 15, 1e-12) on K + sigma G, 100 Lanczos
    vectors for 50 eigenvalues), with sigma = 0.95 x the lowest load.  Kept:
    inputs, the AMD permutation and BCSR pattern, the load path, the
    reference's eigenvalues and, for each, the residual
    ||K phi + lambda G phi|| / ||K phi|| of its eigenvector computed as
    TACSLinearBuckling::checkEigenvector does (src/TACSBuckling.cpp:310-349,
    the reference's own K, G and eigenvectors), and a sparse shift-invert
    solve of the reference's K and G (eigvals_sparse).  Matrices, factors
    and eigenvectors are left out to keep the file small."""
    m = meshgen.cylinder(32, 64, order=2)
    neig = 10
    with tempfile.TemporaryDirectory() as d:
        ind, outd = os.path.join(d, "in"), os.path.join(d, "out")
        os.makedirs(ind)
        os.makedirs(outd)
        lam_cl = meshgen.classical_cylinder_load(m.E, m.nu, m.meta["t"], 1.0)
        write_inputs(ind, m, 0.3 * lam_cl, 1000000, 10, 15, 100, 50)
        subprocess.run([os.path.join(REF_OUT, "golden_gen"), "assembly", ind, outd], check=True)
        fx = load_dir(outd)
        fx.update(bc_nodes=m.bc_nodes, bc_mask=m.bc_mask)
        lam0 = sparse_eigs(fx, neig, 0.3 * lam_cl)
        sigma = 0.95 * lam0[0]
        write_inputs(ind, m, sigma, 1000000, 10, 15, 100, 50)
        subprocess.run([os.path.join(REF_OUT, "golden_gen"), "assembly", ind, outd], check=True)
        fx = load_dir(outd)
        fx.update(bc_nodes=m.bc_nodes, bc_mask=m.bc_mask)
    lam_sparse = sparse_eigs(fx, neig, sigma)
    # checkEigenvector on the reference's own matrices (row ordering) and vectors
    import scipy.sparse as sp
    n = fx["bcsr_rowp"].size - 1
    rowp, cols = fx["bcsr_rowp"], fx["bcsr_cols"]
    K = sp.bsr_matrix((fx["K_after"], cols, rowp), shape=(6 * n, 6 * n)).tocsr()
    G = sp.bsr_matrix((fx["G"], cols, rowp), shape=(6 * n, 6 * n)).tocsr()
    perm = fx["amd_perm"]
    check = []
    for k in range(neig):
        phi = fx["eigvecs"][k][perm].ravel()      # node order -> row order
        kp, gp = K @ phi, G @ phi
        check.append(np.linalg.norm(kp + fx["eigvals"][k] * gp) / np.linalg.norm(kp))
    out = dict(X=m.X, conn=m.conn, bc_nodes=m.bc_nodes, bc_mask=m.bc_mask, bc_vals=m.bc_vals,
               rhs=m.rhs, thickness=m.thickness, E=np.float64(m.E), nu=np.float64(m.nu),
               sigma=np.float64(sigma), lev=np.int32(1000000), gm_m=np.int32(10),
               gm_restarts=np.int32(15), lanczos=np.int32(100), neig=np.int32(50),
               amd_perm=fx["amd_perm"], bcsr_rowp=rowp, bcsr_cols=cols, path=fx["path"],
               eigvals=fx["eigvals"][:neig], eigerr=fx["eigerr"][:neig],
               check_res=np.array(check), eigvals_sparse=lam_sparse)
    np.savez_compressed(os.path.join(HERE, "cyl_q4_32x64_lu.npz"), **out)
    rel = np.abs(out["eigvals"] - lam_sparse) / lam_sparse
    print("wrote cyl_q4_32x64_lu.npz: reference", out["eigvals"][:5], "sparse", lam_sparse[:5],
          "rel", rel[:5], "checkEigenvector", out["check_res"][:5])


def main():
    if len(sys.argv) > 1:
        build_reference()
        for part in sys.argv[1:]:
            globals()["make_" + part]()
        return
    build_reference()
    make_f5()
    make_bdf()
    make_thermal()
    make_orderings()
    make_elements()
    run_case("cyl_q4_4x8_lu", meshgen.cylinder(4, 8, order=2), lev=1000000, gm_m=10,
             gm_restarts=15, lanczos=100, neig=50)
    run_case("cyl_q4_8x16_ilu1", meshgen.cylinder(8, 16, order=2), lev=1, gm_m=30,
             gm_restarts=15, lanczos=100, neig=50)
    run_case("cyl_q9_2x4_lu", meshgen.cylinder(2, 4, order=3), lev=1000000, gm_m=10,
             gm_restarts=15, lanczos=100, neig=50)
    # stiffened panel (Quad9 skin and blade webs, one thickness group per
    # element cell of 20 axial segments x 20 lanes); the complex-step copies
    # and unused matrices are left out to keep the file small
    make_config1()
    run_case("panel_q9_4x8x1_lu", meshgen.stiffened_panel(4, 8, 1), lev=1000000, gm_m=10,
             gm_restarts=15, lanczos=100, neig=10,
             drop=("K", "K_cs", "K_after_cs", "G_cs", "ilu_K_cs", "eigvecs", "eigvecs_cs",
                   "path_cs", "res_path_cs", "K_mult_y_cs", "ilu_apply_x_cs",
                   "ilu_apply_y_cs", "ilu_rowp_cs", "ilu_cols_cs", "csr_rowp_cs",
                   "csr_cols_cs", "bcsr_rowp_cs", "bcsr_cols_cs", "amd_perm_cs",
                   "eigvals_cs"))


if __name__ == "__main__":
    main()
