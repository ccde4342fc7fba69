"""Seeded synthetic meshes for the buckling workloads.

The reference drives its solver from BDF files (examples/cylinder-buckling/
mech-cylinder.bdf through TACSMeshLoader); the workloads here are generated
instead, with the same node-major / tensor-order conventions the reference
assembler expects:

* nodes are numbered ring by ring (axial index i slowest, circumferential
  index j fastest);
* element connectivity is in tensor order (xi fastest, then eta), the order
  TACSMeshLoader produces after its CQUAD4 reorder
  (src/io/TACSMeshLoader.cpp:932-937);
* a Dirichlet condition is (node, 6-bit DOF mask, 6 values), the content of
  one TACSAssembler::addBCs call (src/TACSAssembler.h:104).
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

DEFAULT_SEED = 20261203

# Gauss points/weights on [-1, 1] (3-point rule, used for consistent edge loads)
_G3 = (np.array([-0.774596669241483, 0.0, 0.774596669241483]),
       np.array([5.0 / 9.0, 8.0 / 9.0, 5.0 / 9.0]))


@dataclass
class ShellMesh:
    """A shell mesh with loads: everything a buckling solve consumes."""
    X: np.ndarray            # (nn, 3) float64 node coordinates
    conn: np.ndarray         # (ne, npe) int32 tensor-order connectivity
    bc_nodes: np.ndarray     # (nb,) int32
    bc_mask: np.ndarray      # (nb,) int32, bit k set = DOF k fixed
    bc_vals: np.ndarray      # (nb, 6) float64 prescribed values
    rhs: np.ndarray          # (nn, 6) float64 consistent nodal loads
    thickness: np.ndarray    # (ne,) float64 shell thickness per element
    dv_group: np.ndarray     # (ne,) int32 thickness design group per element
    E: float = 70e9
    nu: float = 0.3
    order: int = 2           # nodes per direction (2 = Quad4, 3 = Quad9)
    meta: dict = field(default_factory=dict)

    @property
    def num_nodes(self) -> int:
        return int(self.X.shape[0])

    @property
    def num_elements(self) -> int:
        return int(self.conn.shape[0])


def _lagrange_lobatto(order: int, u: np.ndarray) -> np.ndarray:
    if order == 2:
        return np.stack([0.5 * (1.0 - u), 0.5 * (1.0 + u)], axis=-1)
    return np.stack([-0.5 * u * (1.0 - u), (1.0 - u) * (1.0 + u), 0.5 * (1.0 + u) * u], axis=-1)


def cylinder(nx: int, ny: int, order: int = 2, R: float = 1.0, L: float = 2.0,
             t: float = 2e-3, E: float = 70e9, nu: float = 0.3, load: float = 1.0,
             imperfection: float = 0.01, seed: int = DEFAULT_SEED) -> ShellMesh:
    """Axially compressed cylinder, axis along x, clamped at x = 0.

    nx, ny: elements along the axis and around the circumference.  The x = L
    ring carries a uniform compressive axial edge load `load` [N/m] as
    consistent nodal forces.  A radial imperfection
    r = R + imperfection*t*sum_k sin(m_k pi x/L) sin(n_k theta + phi_k),
    (m, n) in {(1, 8), (2, 12), (3, 16)}, phi_k ~ U[0, 2 pi) from `seed`.
    """
    p = order - 1
    nxn, nyn = nx * p + 1, ny * p            # nodes along axis, around
    rng = np.random.default_rng(seed)
    phi = rng.uniform(0.0, 2.0 * np.pi, size=3)
    xs = np.linspace(0.0, L, nxn)
    th = 2.0 * np.pi * np.arange(nyn) / nyn
    xx, tt = np.meshgrid(xs, th, indexing="ij")      # (nxn, nyn)
    r = np.full_like(xx, R)
    for (m, n), ph in zip(((1, 8), (2, 12), (3, 16)), phi):
        r += imperfection * t * np.sin(m * np.pi * xx / L) * np.sin(n * tt + ph)
    X = np.stack([xx, r * np.cos(tt), r * np.sin(tt)], axis=-1).reshape(-1, 3)

    def nid(i, j):
        return i * nyn + (j % nyn)

    ei, ej = np.meshgrid(np.arange(nx), np.arange(ny), indexing="ij")
    ei, ej = ei.ravel(), ej.ravel()
    cols = []
    for b in range(order):           # eta (circumferential) slowest
        for a in range(order):       # xi (axial) fastest
            cols.append(nid(ei * p + a, ej * p + b))
    conn = np.stack(cols, axis=1).astype(np.int32)

    bc_nodes = np.array([nid(0, j) for j in range(nyn)], dtype=np.int32)
    bc_mask = np.full(bc_nodes.shape, 0b111111, dtype=np.int32)
    bc_vals = np.zeros((bc_nodes.size, 6))

    # Consistent nodal forces of a uniform line load -load*e_x along the
    # x = L ring: integrate the 1-D shape functions of each element edge.
    rhs = np.zeros((X.shape[0], 6))
    gp, gw = _G3
    N = _lagrange_lobatto(order, gp)              # (3, order)
    seg = 2.0 * np.pi * R / ny                    # edge length per element
    for e in range(ny):
        for a in range(order):
            node = nid(nx * p, e * p + a)
            rhs[node, 0] -= load * 0.5 * seg * np.sum(gw * N[:, a])

    ne = conn.shape[0]
    return ShellMesh(X=X, conn=conn, bc_nodes=bc_nodes, bc_mask=bc_mask, bc_vals=bc_vals,
                     rhs=rhs, thickness=np.full(ne, t), dv_group=np.zeros(ne, np.int32),
                     E=E, nu=nu, order=order,
                     meta=dict(kind="cylinder", nx=nx, ny=ny, R=R, L=L, t=t, load=load,
                               imperfection=imperfection, seed=seed, phases=phi.tolist()))


def radial_shape_modes(m: ShellMesh, mmax: int = 8, nmax: int = 8) -> np.ndarray:
    """Node-coordinate derivatives dX/ds_p (P x nn x 3) of a cylinder's radial
    shape parameters: delta r = sum_p s_p sin(m_p pi x/L) cos(n_p theta),
    (m_p, n_p) = (1 + p // nmax, p % nmax) on an mmax x nmax grid (64
    parameters by default), along each node's radial direction (axis x)."""
    X = m.X
    L = float(m.meta.get("L", X[:, 0].max()))
    th = np.arctan2(X[:, 2], X[:, 1])
    radial = np.stack([np.zeros_like(th), np.cos(th), np.sin(th)], axis=1)
    out = np.zeros((mmax * nmax, X.shape[0], 3))
    for p in range(mmax * nmax):
        mp, n_p = 1 + p // nmax, p % nmax
        amp = np.sin(mp * np.pi * X[:, 0] / L) * np.cos(n_p * th)
        out[p] = amp[:, None] * radial
    return out


def seeded_shape_parameters(num: int = 64, scale: float = 1e-4, seed: int = DEFAULT_SEED):
    """Seeded values s_p ~ scale * U[-1, 1] of the radial shape parameters."""
    return scale * np.random.default_rng(seed + 5).uniform(-1.0, 1.0, size=num)


def shaped_coordinates(m: ShellMesh, s, modes=None) -> np.ndarray:
    """X + sum_p s_p dX/ds_p: the cylinder moved by the radial shape
    parameters s (modes: radial_shape_modes(m) unless given).  The modes are
    linear in s, so dlambda/ds_p = sum over nodes of dlambda/dX . modes[p]."""
    if modes is None:
        modes = radial_shape_modes(m)
    s = np.asarray(s, dtype=np.float64)
    return m.X + np.tensordot(s, modes[:s.size], axes=1)


def stiffened_panel(nx: int, ny: int, nz: int, order: int = 3, Lx: float = 2.0,
                    Ly: float = 0.6, H: float = 0.06, nstiff: int = 8, E: float = 70e9,
                    nu: float = 0.3, load: float = 1e3, tmin: float = 2e-3, tmax: float = 20e-3,
                    nseg: int = 20, nlanes_skin: int = 12,
                    seed: int = DEFAULT_SEED) -> ShellMesh:
    """Flat skin Lx x Ly (x-y plane) with `nstiff` blade webs of height H in
    x-z planes at y_k = Ly (2k+1) / (2 nstiff), sharing the skin's nodes
    along their roots.  nx x ny skin elements, nx x nz elements per web.

    Thickness design groups g = L * a + lane with L = nlanes_skin + nstiff
    lanes, a = the element's axial segment (nseg equal
    segments of x), lane = its skin strip (nlanes_skin equal strips of y) or
    nlanes_skin + k for web k; t_g ~ U[tmin, tmax] from `seed`.
    Supports: x = 0 edge u = v = w = 0, x = Lx edge v = w = 0, skin y-edges
    w = 0; the x = Lx edge (skin and webs) carries a uniform compressive line
    load `load` [N/m] along -x as consistent nodal forces."""
    p = order - 1
    nxn, nyn, nzn = nx * p + 1, ny * p + 1, nz * p
    if (ny * p) % (2 * nstiff):
        raise ValueError("the skin needs node lines at the web roots: "
                         "(order - 1) * ny must be a multiple of 2 * nstiff")
    rng = np.random.default_rng(seed)
    nlanes = nlanes_skin + nstiff
    tvals = rng.uniform(tmin, tmax, size=nseg * nlanes)
    xs = np.linspace(0.0, Lx, nxn)
    ys = np.linspace(0.0, Ly, nyn)
    zs = np.linspace(0.0, H, nzn + 1)

    def skin(ix, iy):
        return ix * nyn + iy
    nskin = nxn * nyn
    root = [(2 * k + 1) * (ny * p) // (2 * nstiff) for k in range(nstiff)]

    def web(k, ix, iz):
        if iz == 0:
            return skin(ix, root[k])
        return nskin + (k * nxn + ix) * nzn + (iz - 1)
    nn = nskin + nstiff * nxn * nzn
    X = np.zeros((nn, 3))
    for ix in range(nxn):
        for iy in range(nyn):
            X[skin(ix, iy)] = (xs[ix], ys[iy], 0.0)
        for k in range(nstiff):
            for iz in range(1, nzn + 1):
                X[web(k, ix, iz)] = (xs[ix], ys[root[k]], zs[iz])
    conn, group = [], []

    def seg(xc):
        return min(int(xc / (Lx / nseg)), nseg - 1)
    for ex in range(nx):
        for ey in range(ny):
            conn.append([skin(ex * p + a, ey * p + b) for b in range(order) for a in range(order)])
            xc, yc = (ex + 0.5) * Lx / nx, (ey + 0.5) * Ly / ny
            group.append(nlanes * seg(xc) + min(int(yc / (Ly / nlanes_skin)), nlanes_skin - 1))
    for k in range(nstiff):
        for ex in range(nx):
            for ez in range(nz):
                conn.append([web(k, ex * p + a, ez * p + b) for b in range(order)
                             for a in range(order)])
                group.append(nlanes * seg((ex + 0.5) * Lx / nx) + nlanes_skin + k)
    conn = np.array(conn, dtype=np.int32)
    group = np.array(group, dtype=np.int32)

    mask = np.zeros(nn, dtype=np.int32)
    mask[np.abs(X[:, 0]) < 1e-12] |= 0b111
    mask[np.abs(X[:, 0] - Lx) < 1e-12] |= 0b110
    for ix in range(nxn):
        mask[skin(ix, 0)] |= 0b100
        mask[skin(ix, nyn - 1)] |= 0b100
    bc_nodes = np.nonzero(mask)[0].astype(np.int32)
    bc_mask = mask[bc_nodes]
    bc_vals = np.zeros((bc_nodes.size, 6))

    rhs = np.zeros((nn, 6))
    gp, gw = _G3
    N = _lagrange_lobatto(order, gp)
    for ey in range(ny):
        for a in range(order):
            rhs[skin(nx * p, ey * p + a), 0] -= load * 0.5 * (Ly / ny) * np.sum(gw * N[:, a])
    for k in range(nstiff):
        for ez in range(nz):
            for a in range(order):
                rhs[web(k, nx * p, ez * p + a), 0] -= load * 0.5 * (H / nz) * np.sum(gw * N[:, a])
    return ShellMesh(X=X, conn=conn, bc_nodes=bc_nodes, bc_mask=bc_mask, bc_vals=bc_vals,
                     rhs=rhs, thickness=tvals[group], dv_group=group, E=E, nu=nu, order=order,
                     meta=dict(kind="stiffened_panel", nx=nx, ny=ny, nz=nz, Lx=Lx, Ly=Ly, H=H,
                               nstiff=nstiff, load=load, seed=seed, tvals=tvals))


def classical_cylinder_load(E: float, nu: float, t: float, R: float) -> float:
    """Classical axial buckling load per unit circumference, E t^2/(R sqrt(3(1-nu^2)))."""
    return E * t * t / (R * np.sqrt(3.0 * (1.0 - nu * nu)))
