"""Dense CPU restatement of the buckling eigenvalue coordinate sensitivities
-- TEST INFRASTRUCTURE (imported by tests/ only).

The formula is the body of the reference's commented-out
TACSLinearBuckling::evalEigenXptSens (src/TACSBuckling.cpp:457-497):

  dlam/dX = -[phi^T K' phi + lam phi^T G'(u) phi - lam psi^T (K u)'] / phi^T G phi,
  K psi = d(phi^T G(u) phi)/du,

with the element derivatives of TACSElement::addMatXptSensInnerProduct,
getMatSVSensInnerProduct and addAdjResXptProduct (src/elements/
TACSElement.cpp:270-581; central differences, dh = 1e-7) from the oracle's
element routines, and dense FP64 linear algebra for the solves.  About a
nonlinear preloaded state R(u, X) = s f the same formula holds with the
tangent K_T(u) in place of K and psi^T R' in place of psi^T (K u)'.
The thickness derivative (the documented evalEigenDVSens formula,
src/TACSBuckling.cpp:359-382) uses the same adjoint with the element
matrices differentiated exactly in the shell thickness (they are
t M1 + t^3 M3), for one thickness or per design group.
Sizes: a few hundred nodes (dense matrices).
"""
from __future__ import annotations

import numpy as np

from . import (GEOMETRIC, STIFFNESS, Material, element_adjres_xpt_product, element_jacobian,
               element_matrix, element_sv_inner_product, element_xpt_inner_product)


def _dofs(c):
    return (6 * np.asarray(c)[:, None] + np.arange(6)).ravel()


class DenseShell:
    """One-thickness shell mesh (a2ds.mesh.ShellMesh) on dense matrices."""

    def __init__(self, m, nonlinear=False):
        self.m, self.order, self.nl = m, m.order, int(nonlinear)
        self.mat = Material.iso(m.E, m.nu, float(m.thickness[0]))
        self.N = 6 * m.X.shape[0]
        self.free = np.ones(self.N, bool)
        for node, mask in zip(m.bc_nodes, m.bc_mask):
            for k in range(6):
                if int(mask) >> k & 1:
                    self.free[6 * node + k] = False

    def matrix(self, X, kind, u):
        A = np.zeros((self.N, self.N))
        for c in self.m.conn:
            d = _dofs(c)
            A[np.ix_(d, d)] += element_matrix(self.order, self.nl, kind, self.mat, X[c], u[d])
        return A

    def tangent(self, X, u):
        A, R = np.zeros((self.N, self.N)), np.zeros(self.N)
        for c in self.m.conn:
            d = _dofs(c)
            r, J = element_jacobian(self.order, self.nl, self.mat, X[c], u[d])
            A[np.ix_(d, d)] += J
            R[d] += r
        return A, R

    def state(self, X, load=None, nsteps=4, rtol=1e-11):
        """Linear path K u = f (load None) or Newton load stepping to
        load * f with the full tangent (nonlinear elements)."""
        f = self.m.rhs.ravel()
        fr = self.free
        u = np.zeros(self.N)
        if load is None:
            K = self.matrix(X, STIFFNESS, u)
            u[fr] = np.linalg.solve(K[np.ix_(fr, fr)], f[fr])
            return u
        for k in range(1, nsteps + 1):
            fk = load * k / nsteps * f
            for _ in range(40):
                KT, R = self.tangent(X, u)
                r = (R - fk)[fr]
                if np.linalg.norm(r) <= rtol * np.linalg.norm(fk[fr]):
                    break
                u[fr] -= np.linalg.solve(KT[np.ix_(fr, fr)], r)
            else:
                raise RuntimeError("Newton did not converge")
        return u

    def buckling(self, X, u):
        """K(u) phi + lam G(u) phi = 0 on the free DOFs, loads by magnitude;
        K(u) is the tangent at u (K itself for linear elements)."""
        import scipy.linalg as sla
        fr = self.free
        K = self.tangent(X, u)[0] if self.nl else self.matrix(X, STIFFNESS, u)
        G = self.matrix(X, GEOMETRIC, u)
        Kf, Gf = K[np.ix_(fr, fr)], G[np.ix_(fr, fr)]
        mu, V = sla.eigh(-0.5 * (Gf + Gf.T), 0.5 * (Kf + Kf.T))
        order = np.argsort(-np.abs(mu))
        lam = 1.0 / mu[order]
        phi = np.zeros((self.N, lam.size))
        phi[fr] = V[:, order]
        return lam, phi, K, G

    def xpt_sens(self, X, u, lam, phi, K, G, dh=1e-7):
        """dlam/dX (nodes x 3) of one load with eigenvector phi."""
        o, nl, mat = self.order, self.nl, self.mat
        fr = self.free
        g = np.zeros(self.N)
        for c in self.m.conn:
            d = _dofs(c)
            g[d] += lam * element_sv_inner_product(o, nl, GEOMETRIC, mat, X[c], u[d], phi[d],
                                                   phi[d], dh)
            if nl:
                g[d] += element_sv_inner_product(o, nl, STIFFNESS, mat, X[c], u[d], phi[d],
                                                 phi[d], dh)
        psi = np.zeros(self.N)
        psi[fr] = np.linalg.solve(K[np.ix_(fr, fr)], g[fr])
        out = np.zeros((self.N // 6, 3))
        nn = len(self.m.conn[0])
        for c in self.m.conn:
            d = _dofs(c)
            v = (element_xpt_inner_product(o, nl, STIFFNESS, mat, X[c], u[d], phi[d], phi[d], dh)
                 + lam * element_xpt_inner_product(o, nl, GEOMETRIC, mat, X[c], u[d], phi[d],
                                                   phi[d], dh))
            if nl:
                v -= element_adjres_xpt_product(o, nl, mat, X[c], u[d], psi[d], dh)
            else:  # R = K u for the linear element: psi^T (K u)'
                v -= element_xpt_inner_product(o, nl, STIFFNESS, mat, X[c], u[d], psi[d], u[d],
                                               dh)
            out[c] += v.reshape(nn, 3)
        return -out / float(phi @ G @ phi)

    def thickness_sens(self, X, u, lam, phi, K, G):
        """dlam/dt for the mesh's single thickness t (linear elements):
        -[phi^T K' phi + lam phi^T G'(u) phi - lam psi^T K' u] / phi^T G phi,
        K psi = G(phi) phi, ' = d/dt of the element matrices, exact
        (_dt_element: they are t M1 + t^3 M3)."""
        fr = self.free
        t0 = float(self.mat.t)
        g = self.matrix(X, GEOMETRIC, phi) @ phi
        psi = np.zeros(self.N)
        psi[fr] = np.linalg.solve(K[np.ix_(fr, fr)], g[fr])
        z = np.zeros(6 * self.order ** 2)
        num = 0.0
        for c in self.m.conn:
            d = _dofs(c)
            dK = _dt_element(self.order, STIFFNESS, self.m.E, self.m.nu, t0, X[c], z)
            dG = _dt_element(self.order, GEOMETRIC, self.m.E, self.m.nu, t0, X[c], u[d])
            num += phi[d] @ dK @ phi[d] + lam * (phi[d] @ dG @ phi[d]) - lam * (psi[d] @ dK @ u[d])
        return -num / float(phi @ G @ phi)


def _dt_element(order, kind, E, nu, t, X, v):
    """d M_e/dt of an element matrix, exactly: with no thickness offset the
    shell's constitutive matrix is t x (membrane, shear, drilling) plus
    t^3 x (bending), so M_e(t) = t M1 + t^3 M3 and M1, M3 follow from the
    matrices at t = 1 and t = 2; dM/dt = M1 + 3 t^2 M3."""
    M1t = element_matrix(order, 0, kind, Material.iso(E, nu, 1.0), X, v)
    M2t = element_matrix(order, 0, kind, Material.iso(E, nu, 2.0), X, v)
    M3 = (M2t - 2.0 * M1t) / 6.0
    M1 = M1t - M3
    return M1 + 3.0 * t * t * M3


def thickness_sens_groups(m, u, lam, phi, K, G):
    """dlam/dt_g for every thickness group of a mesh with per-element
    thickness m.thickness and groups m.dv_group (linear elements): the
    formula of DenseShell.thickness_sens with the element matrices of group
    g's elements differentiated in their thickness (exactly, _dt_element),
    the adjoint psi shared by all groups.  Dense FP64; returns one value per
    group id up to max(dv_group)."""
    ds = DenseShell(m)
    fr = ds.free
    X = m.X
    ng = int(np.max(m.dv_group)) + 1
    # G(phi) phi with per-element thickness
    g = np.zeros(ds.N)
    for e, c in enumerate(m.conn):
        d = _dofs(c)
        mat = Material.iso(m.E, m.nu, float(m.thickness[e]))
        g[d] += element_matrix(ds.order, 0, GEOMETRIC, mat, X[c], phi[d]) @ phi[d]
    psi = np.zeros(ds.N)
    psi[fr] = np.linalg.solve(K[np.ix_(fr, fr)], g[fr])
    num = np.zeros(ng)
    z = np.zeros(6 * ds.order ** 2)
    for e, c in enumerate(m.conn):
        d = _dofs(c)
        t = float(m.thickness[e])
        dK = _dt_element(ds.order, STIFFNESS, m.E, m.nu, t, X[c], z)
        dG = _dt_element(ds.order, GEOMETRIC, m.E, m.nu, t, X[c], u[d])
        num[m.dv_group[e]] += (phi[d] @ dK @ phi[d] + lam * (phi[d] @ dG @ phi[d])
                               - lam * (psi[d] @ dK @ u[d]))
    return -num / float(phi @ G @ phi)


def mesh_matrices(m, u):
    """Dense K (zero state) and G (along u) of a mesh with per-element
    thickness, without Dirichlet rows."""
    N = 6 * m.X.shape[0]
    K, G = np.zeros((N, N)), np.zeros((N, N))
    z = np.zeros(6 * m.order ** 2)
    for e, c in enumerate(m.conn):
        d = _dofs(c)
        mat = Material.iso(m.E, m.nu, float(m.thickness[e]))
        K[np.ix_(d, d)] += element_matrix(m.order, 0, STIFFNESS, mat, m.X[c], z)
        G[np.ix_(d, d)] += element_matrix(m.order, 0, GEOMETRIC, mat, m.X[c], u[d])
    return K, G


def dense_buckling_groups(m):
    """Path, lowest loads and eigenvectors of a per-element-thickness mesh
    (dense FP64): (u, lam, phi, K, G) on the full DOF vector."""
    import scipy.linalg as sla
    ds = DenseShell(m)
    fr = ds.free
    K, _ = mesh_matrices(m, np.zeros(ds.N))
    f = m.rhs.ravel()
    u = np.zeros(ds.N)
    u[fr] = np.linalg.solve(K[np.ix_(fr, fr)], f[fr])
    K, G = mesh_matrices(m, u)
    Kf, Gf = K[np.ix_(fr, fr)], G[np.ix_(fr, fr)]
    mu, V = sla.eigh(-0.5 * (Gf + Gf.T), 0.5 * (Kf + Kf.T))
    order = np.argsort(-np.abs(mu))
    lam = 1.0 / mu[order]
    phi = np.zeros((ds.N, lam.size))
    phi[fr] = V[:, order]
    return u, lam, phi, K, G
