"""CPU oracle for the SIMP compliance loop of TopOpt.jl (TEST INFRASTRUCTURE ONLY).

This module is test infrastructure, not the product.  Only ``tests/``,
``__graft_entry__.smoke()`` and the CPU-baseline leg of ``bench.py`` may import
it.  It restates, in plain numpy/scipy FP64, the reference algorithm of each
step on the hot path; every function cites the TopOpt.jl file:line it follows
(paths relative to the TopOpt.jl project root).

Indices are 0-based here.  The reference is 1-based; ``node_dofs`` /
``cell_dofs`` returned here are the reference's values minus one.

Parity pins (see tests/test_oracle_golden.py):
  * HalfMBB 2x2 node coordinates, cell connectivity, node_dofs, cell_dofs,
    node_cells -- test/topopt_problems/metadata.jl:53-132 (golden fixture
    tests/golden/metadata_2x2.json, extracted by tests/golden/make_golden.py).
  * PointLoadCantilever 160x40 force_dof == 161*21*2 -- test/topopt_problems/problems.jl:20.
  * Filter identities (uniform field preserved, pullback = J^T, sens filter
    forward identity, too-small rmin throws) -- test/CheqFilters/test_filters.jl.
  * Compliance gradient vs central finite differences on HalfMBB 2x2,
    p in {1,2,3}, xmin 0.01 -- test/Functions/test_common_fns.jl:32-49.
  * Matrix-free CG vs direct solve agreement on a 20x10x10 cantilever at
    x = 0.5 -- test/FEA/solvers.jl:32-59.
The Ferrite.jl numbering in 3D and the IterativeSolvers stopping rule are not
pinned by any reference fixture (Julia is not available to run the reference);
they follow the same first-touch rule and the published CG algorithm.  The OC
update has no reference implementation at all (the reference drives SIMP with
MMA); it restates the published optimality-criteria method (Andreassen et al.,
"Efficient topology optimization in MATLAB using 88 lines of code", 2011).
"""
from __future__ import annotations

import math
from collections import deque
from dataclasses import dataclass, field

import numpy as np
import scipy.sparse as sp
import scipy.sparse.linalg as spla

# --------------------------------------------------------------------------
# P1: structured grid  (src/TopOptProblems/grids.jl:66-92, Ferrite generate_grid)
# --------------------------------------------------------------------------

# Ferrite reference-element corner order (Quadrilateral / Hexahedron):
# local node -> offset (bx, by[, bz]) of the corner within the cell.
QUAD_CORNERS = [(0, 0), (1, 0), (1, 1), (0, 1)]
HEX_CORNERS = [(0, 0, 0), (1, 0, 0), (1, 1, 0), (0, 1, 0),
               (0, 0, 1), (1, 0, 1), (1, 1, 1), (0, 1, 1)]


def corners(dim):
    return QUAD_CORNERS if dim == 2 else HEX_CORNERS


@dataclass
class Grid:
    dim: int
    nels: tuple
    sizes: tuple
    coords: np.ndarray      # (nnodes, dim) float64
    cells: np.ndarray       # (ncells, 2**dim) int64, 0-based node ids (Ferrite local order)

    @property
    def nnodes(self):
        return self.coords.shape[0]

    @property
    def ncells(self):
        return self.cells.shape[0]


def rectilinear_grid(nels, sizes) -> Grid:
    """Nodes on [0, nels*sizes], node ids x-fastest, cells x-fastest
    (grids.jl:66-92; pinned in 2D by test/topopt_problems/metadata.jl:53-77)."""
    dim = len(nels)
    nn = [n + 1 for n in nels]
    # Ferrite generate_grid places nodes by linear interpolation between the corners.
    axes = [np.arange(nn[d], dtype=np.float64) * (nels[d] * sizes[d]) / nels[d] for d in range(dim)]
    if dim == 2:
        Y, X = np.meshgrid(axes[1], axes[0], indexing="ij")
        coords = np.stack([X.ravel(), Y.ravel()], axis=1)
        J, I = np.meshgrid(np.arange(nels[1]), np.arange(nels[0]), indexing="ij")
        base = (I + nn[0] * J).ravel()
        cells = np.stack([base + a + nn[0] * b for (a, b) in QUAD_CORNERS], axis=1)
    else:
        Z, Y, X = np.meshgrid(axes[2], axes[1], axes[0], indexing="ij")
        coords = np.stack([X.ravel(), Y.ravel(), Z.ravel()], axis=1)
        K, J, I = np.meshgrid(np.arange(nels[2]), np.arange(nels[1]), np.arange(nels[0]), indexing="ij")
        base = (I + nn[0] * (J + nn[1] * K)).ravel()
        cells = np.stack([base + a + nn[0] * (b + nn[1] * c) for (a, b, c) in HEX_CORNERS], axis=1)
    return Grid(dim, tuple(nels), tuple(float(s) for s in sizes), coords, cells.astype(np.int64))


# --------------------------------------------------------------------------
# P2: metadata  (src/TopOptProblems/metadata.jl:27-145)
# --------------------------------------------------------------------------

def dof_numbering(grid: Grid):
    """Ferrite DofHandler first-touch numbering for one Lagrange^dim field:
    cells in order, local vertices in order, each unseen node gets ``dim``
    consecutive dofs (metadata.jl:40-50, 116-145; pinned by metadata.jl:79-95).
    Returns node_dofs (dim, nnodes) and cell_dofs (dim*nv, ncells), 0-based."""
    dim = grid.dim
    flat = grid.cells.ravel()                      # visiting order: cell-major, local order
    _, first = np.unique(flat, return_index=True)  # first visit of every node
    order = np.argsort(first, kind="stable")       # nodes sorted by first visit
    rank = np.empty(grid.nnodes, dtype=np.int64)
    rank[order] = np.arange(grid.nnodes)
    node_dofs = dim * rank[None, :] + np.arange(dim)[:, None]
    nv = grid.cells.shape[1]
    cell_dofs = np.empty((dim * nv, grid.ncells), dtype=np.int64)
    for a in range(nv):
        for d in range(dim):
            cell_dofs[dim * a + d, :] = node_dofs[d, grid.cells[:, a]]
    return node_dofs, cell_dofs


def dof_cells(cell_dofs, ndofs):
    """dof -> [(cell, local dof)] in cell order (metadata.jl:64-76)."""
    out = [[] for _ in range(ndofs)]
    for c in range(cell_dofs.shape[1]):
        for l in range(cell_dofs.shape[0]):
            out[cell_dofs[l, c]].append((c, l))
    return out


def node_cells(grid: Grid):
    """node -> [(cell, local node)] in cell order (metadata.jl:99-109)."""
    out = [[] for _ in range(grid.nnodes)]
    for c in range(grid.ncells):
        for l, n in enumerate(grid.cells[c]):
            out[n].append((c, l))
    return out


# --------------------------------------------------------------------------
# P3: problems  (src/TopOptProblems/problem_types.jl:162-402, matrices_and_vectors.jl:346-365)
# --------------------------------------------------------------------------

@dataclass
class Problem:
    grid: Grid
    E: float
    nu: float
    force: float
    node_dofs: np.ndarray
    cell_dofs: np.ndarray
    fixed_dofs: np.ndarray      # sorted, 0-based
    f: np.ndarray               # dense load vector (ndofs,)
    force_dof: int
    load_node: int
    plane_stress: bool = False

    @property
    def ndofs(self):
        return self.node_dofs.size


def _approx(a, b):
    # Julia isapprox with default rtol = sqrt(eps) and atol = 0
    return abs(a - b) <= math.sqrt(np.finfo(np.float64).eps) * max(abs(a), abs(b))


def _approx_v(a, b):
    return np.abs(a - b) <= math.sqrt(np.finfo(np.float64).eps) * np.maximum(np.abs(a), abs(b))


def point_load_cantilever(nels, sizes, E=1.0, nu=0.3, force=1.0,
                          load="reference_first_node", plane_stress=False) -> Problem:
    """problem_types.jl:162-231.  Left face clamped (all components); load
    ``[0, -force, 0]`` at the first node (lowest id) of the set right & middley
    (problem_types.jl:194-196, 223-225, 398-402).  ``load='face_centre'`` puts it
    at the centre of the right face instead (a 3D variant, not the reference)."""
    dim = len(nels)
    if nels[1] % 2 or (dim == 3 and nels[2] % 2):
        raise ValueError("Grid does not have an even number of elements along the y and/or z axes.")
    g = rectilinear_grid(nels, sizes)
    node_dofs, cell_dofs = dof_numbering(g)
    lo, hi = np.zeros(dim), np.array(nels) * np.array(sizes, dtype=float)
    x = g.coords
    left = np.nonzero(_approx_v(x[:, 0], lo[0]))[0]
    fixed = np.sort(node_dofs[:, left].ravel())
    midy = (lo[1] + hi[1]) / 2
    sel = _approx_v(x[:, 0], hi[0]) & _approx_v(x[:, 1], midy)
    if load == "face_centre" and dim == 3:
        sel &= _approx_v(x[:, 2], (lo[2] + hi[2]) / 2)
    fnode = int(np.nonzero(sel)[0][0])          # first node of the ordered node set
    f = np.zeros(node_dofs.size)
    fdof = int(node_dofs[1, fnode])
    f[fdof] = -force
    return Problem(g, E, nu, force, node_dofs, cell_dofs, np.asarray(fixed, dtype=np.int64),
                   f, fdof, fnode, plane_stress)


def half_mbb(nels, sizes, E=1.0, nu=0.3, force=1.0, plane_stress=False) -> Problem:
    """problem_types.jl:324-395: u1 = 0 on the left face (:348, 376), u2 = 0 on
    bottom & right (:353-355, 378), load ``[0, -force]`` at the first node of
    top & left (:360, 387)."""
    dim = len(nels)
    g = rectilinear_grid(nels, sizes)
    node_dofs, cell_dofs = dof_numbering(g)
    lo, hi = np.zeros(dim), np.array(nels) * np.array(sizes, dtype=float)
    x = g.coords
    f1 = node_dofs[0, np.nonzero(_approx_v(x[:, 0], lo[0]))[0]]
    f2 = node_dofs[1, np.nonzero(_approx_v(x[:, 1], lo[1]) & _approx_v(x[:, 0], hi[0]))[0]]
    fixed = np.unique(np.concatenate([f1, f2]))
    fnode = int(np.nonzero(_approx_v(x[:, 1], hi[1]) & _approx_v(x[:, 0], lo[0]))[0][0])
    f = np.zeros(node_dofs.size)
    fdof = int(node_dofs[1, fnode])
    f[fdof] = -force
    return Problem(g, E, nu, force, node_dofs, cell_dofs, np.asarray(fixed, dtype=np.int64),
                   f, fdof, fnode, plane_stress)


# --------------------------------------------------------------------------
# E1: element stiffness  (src/TopOptProblems/matrices_and_vectors.jl:68-177)
# --------------------------------------------------------------------------

def _lame(E, nu, plane_stress):
    # matrices_and_vectors.jl:83-84: the 3D Lame constants for every dim (plane strain in 2D).
    lam = E * nu / ((1 + nu) * (1 - 2 * nu))
    mu = E / (2 * (1 + nu))
    if plane_stress:   # extra, not the reference: plane-stress lambda*
        lam = 2 * lam * mu / (lam + 2 * mu)
    return lam, mu


def element_stiffness(dim, sizes, E, nu, plane_stress=False, quad_order=4):
    """Ke_ab = sum_q dotdot(grad phi_a, C, grad phi_b) dOmega with Gauss-Legendre
    ``quad_order`` points per direction (default_quad_order = 4, solvers_api.jl:432-444);
    dof order dim*(a-1)+d (matrices_and_vectors.jl:162)."""
    lam, mu = _lame(E, nu, plane_stress)
    pts, wts = np.polynomial.legendre.leggauss(quad_order)
    cs = corners(dim)
    ref = [tuple(2 * c - 1 for c in cc) for cc in cs]   # reference coords in {-1, 1}
    nb = len(cs)
    h = np.asarray(sizes, dtype=np.float64)
    Ke = np.zeros((dim * nb, dim * nb))
    grids = np.meshgrid(*([np.arange(quad_order)] * dim), indexing="ij")
    for qidx in zip(*[gg.ravel() for gg in grids]):
        xi = np.array([pts[q] for q in qidx])
        w = np.prod([wts[q] for q in qidx])
        detJ = np.prod(h / 2)
        grads = np.zeros((nb, dim))
        for a in range(nb):
            for d in range(dim):
                g = ref[a][d] / 2.0
                for e in range(dim):
                    if e != d:
                        g *= (1 + ref[a][e] * xi[e]) / 2.0
                grads[a, d] = g * 2.0 / h[d]
        dO = detJ * w
        for b in range(nb):
            gb = grads[b]
            for a in range(nb):
                ga = grads[a]
                blk = lam * np.outer(ga, gb) + mu * (np.dot(ga, gb) * np.eye(dim) + np.outer(gb, ga))
                Ke[dim * a:dim * a + dim, dim * b:dim * b + dim] += blk * dO
    return Ke


# --------------------------------------------------------------------------
# E2: penalty / interpolation  (src/Utilities/penalties.jl:30-33, 121-130; utils.jl:77)
# --------------------------------------------------------------------------

def rho_drho(x, p, xmin):
    """PENALTY_BEFORE_INTERPOLATION = true (src/TopOpt.jl:16-23):
    rho = xmin + (1-xmin) x^p,  drho = (1-xmin) p x^(p-1)."""
    x = np.asarray(x, dtype=np.float64)
    rho = x ** p * (1 - xmin) + xmin
    drho = (1 - xmin) * p * x ** (p - 1) if p != 0 else np.zeros_like(x)
    return rho, drho


# --------------------------------------------------------------------------
# S1/S2: solver setup and matrix-free operator
#   (src/FEA/solvers_api.jl:468-574, matrix_free_operator.jl:66-105,
#    elementmatrix.jl:10-53, 64-109)
# --------------------------------------------------------------------------

@dataclass
class FEAState:
    prob: Problem
    Ke: np.ndarray
    xmin: float
    p: float
    meandiag: float
    free_mask: np.ndarray       # (ndofs,) bool
    elem_mask: np.ndarray       # (ndpc, ncells) bool, active-dof mask of ElementMatrix
    vars: np.ndarray = field(default=None)


def fea_setup(prob: Problem, xmin=1e-3, p=1.0) -> FEAState:
    Ke = element_stiffness(prob.grid.dim, prob.grid.sizes, prob.E, prob.nu, prob.plane_stress)
    # meandiag = sum over elements of each element's trace (solvers_api.jl:526-527).
    meandiag = float(prob.grid.ncells * np.trace(Ke))
    free = np.ones(prob.ndofs, dtype=bool)
    free[prob.fixed_dofs] = False
    elem_mask = free[prob.cell_dofs]    # elementmatrix.jl:64-109 (mask = not prescribed)
    st = FEAState(prob, Ke, float(xmin), float(p), meandiag, free, elem_mask)
    st.vars = np.ones(prob.grid.ncells)
    return st


def matvec(st: FEAState, x):
    """Masked element-by-element K*x with the two-phase gather
    (matrix_free_operator.jl:66-105): xes_e = rho_e * bcmatrix(Ke) * x_e, then each
    free dof sums its (cell, local) entries in cell order; fixed dofs get meandiag*x."""
    cd = st.prob.cell_dofs
    rho, _ = rho_drho(st.vars, st.p, st.xmin)
    xe = x[cd] * st.elem_mask                      # masked columns
    ye = (st.Ke @ xe) * st.elem_mask * rho[None, :]   # masked rows, scaled
    y = np.zeros_like(x)
    # phase 2: gather in cell order (np.add.at accumulates in index order)
    np.add.at(y, cd.T.ravel(), ye.T.ravel())
    y[~st.free_mask] = st.meandiag * x[~st.free_mask]
    return y


def assemble(st: FEAState):
    """Sparse K with Ferrite apply! (assemble.jl:28-90): prescribed rows/cols zeroed,
    diagonal set to the mean |diag| of the assembled K."""
    cd = st.prob.cell_dofs
    rho, _ = rho_drho(st.vars, st.p, st.xmin)
    nd = cd.shape[0]
    I = np.repeat(cd, nd, axis=0)          # (nd*nd, ncells): row index per entry
    J = np.tile(cd, (nd, 1))
    V = st.Ke.ravel()[:, None] * rho[None, :]
    K = sp.csr_matrix((V.ravel(), (I.ravel(), J.ravel())), shape=(st.prob.ndofs,) * 2)
    m = float(np.mean(np.abs(K.diagonal())))
    fixed = st.prob.fixed_dofs
    D = sp.diags(st.free_mask.astype(float))
    K = (D @ K @ D).tolil()
    for d in fixed:
        K[d, d] = m
    return K.tocsr()


def direct_solve(st: FEAState, f=None):
    """DirectSolver: Cholesky of the constrained K (solvers_api.jl:131-165)."""
    f = st.prob.f if f is None else f
    K = assemble(st)
    fr = f.copy()
    fr[~st.free_mask] = 0.0
    return spla.spsolve(K.tocsc(), fr)


def jacobi_diag(st: FEAState):
    """Diagonal of the masked operator (what DiagonalPreconditioner sees)."""
    cd = st.prob.cell_dofs
    rho, _ = rho_drho(st.vars, st.p, st.xmin)
    d = np.zeros(st.prob.ndofs)
    np.add.at(d, cd.T.ravel(), (np.diag(st.Ke)[:, None] * rho[None, :]).T.ravel())
    d[~st.free_mask] = st.meandiag
    return d


def pcg(st: FEAState, f=None, rtol=math.sqrt(np.finfo(np.float64).eps), abstol=0.0,
        maxiter=700, x0=None, precond=True, conv="default"):
    """Jacobi PCG as IterativeSolvers.cg! (called from solvers_api.jl:177-220):
    tol = max(rtol*||r0||, abstol); stop when the recurrence residual norm <= tol
    or after maxiter iterations.  conv="energy" replaces the stop test by EnergyCriteria's
    isconverged (src/FEA/convergence_criteria.jl:26-45), checked before every iteration
    as IterativeSolvers does.  Returns (x, iterations, ||r||)."""
    f = st.prob.f if f is None else f
    b = f.copy()
    b[~st.free_mask] = 0.0
    x = np.zeros_like(b) if x0 is None else x0.copy()
    r = b - matvec(st, x) if x0 is not None else b.copy()
    dinv = 1.0 / jacobi_diag(st) if precond else np.ones_like(b)
    res = np.linalg.norm(r)
    tol = max(rtol * res, abstol)
    u = np.zeros_like(b)
    rho = 1.0
    it = 0
    energy = [0.0]

    def converged():
        if conv != "energy":
            return res <= tol
        xtr = float(x @ r)
        xAx = float(b @ x) - xtr
        dE = xAx - energy[0]
        if math.isnan(dE) or math.isnan(xAx) or xAx < 0:
            raise FloatingPointError("EnergyCriteria: NaN or negative x'Ax")
        with np.errstate(divide="ignore", invalid="ignore"):
            ok = bool(np.float64(abs(dE)) / xAx <= tol and np.float64(abs(xtr)) / xAx <= tol)
        energy[0] = xAx
        return ok

    while it < maxiter and not converged():
        c = dinv * r
        rho_prev, rho = rho, float(c @ r)
        beta = rho / rho_prev
        u = c + beta * u
        c = matvec(st, u)
        alpha = rho / float(u @ c)
        x = x + alpha * u
        r = r - alpha * c
        res = np.linalg.norm(r)
        it += 1
    return x, it, res


# --------------------------------------------------------------------------
# C1/C2: compliance, sensitivities, volume
#   (src/Functions/compliance.jl:58-76, compute_element_energy.jl:18-38, volume.jl:47-67)
# --------------------------------------------------------------------------

def compliance(st: FEAState, u, x=None):
    """ce_e = u_e' Ke(raw) u_e; c = sum rho_e ce_e; grad_e = -drho_e ce_e."""
    x = st.vars if x is None else x
    ue = u[st.prob.cell_dofs]
    ce = np.einsum("ie,ij,je->e", ue, st.Ke, ue)
    rho, drho = rho_drho(x, st.p, st.xmin)
    return float(np.sum(rho * ce)), -drho * ce, ce


def cell_volumes(prob: Problem):
    return np.full(prob.grid.ncells, float(np.prod(prob.grid.sizes)))


def volume_fraction(prob: Problem, x):
    v = cell_volumes(prob)
    return float(np.sum(x * v) / np.sum(v)), v / np.sum(v)


# --------------------------------------------------------------------------
# F1-F3: node-based BESO filter  (src/CheqFilters/CheqFilters.jl:66-118,
#        density_filter.jl:25-121, sens_filter.jl:49-111)
# --------------------------------------------------------------------------

def neighbour_info(prob: Problem, rmin):
    """Literal BFS of get_neighbour_info (CheqFilters.jl:66-118): a node within
    rmin of the cell centre is pushed once for every traversed cell that holds it."""
    g = prob.grid
    ncl = node_cells(g)
    all_nodes, all_w = [], []
    for cid in range(g.ncells):
        center = g.coords[g.cells[cid]].mean(axis=0)
        q = deque([cid])
        visited = {cid}
        nodes, ws = [], []
        while q:
            c = q.popleft()
            for n in g.cells[c]:
                d = float(np.linalg.norm(g.coords[n] - center))
                if d < rmin:
                    nodes.append(int(n))
                    ws.append(max(rmin - d, 0.0))
                    for (c2, _) in ncl[n]:
                        if c2 not in visited:
                            q.append(c2)
                            visited.add(c2)
        all_nodes.append(nodes)
        all_w.append(ws)
    return all_nodes, all_w


def filter_matrices(prob: Problem, rmin):
    """M1 (nnodes x ncells): volume-weighted node average (density_filter.jl:62-73,
    scalecols! :110-121); M2 (ncells x nnodes): normalised cone weights
    (density_filter.jl:75-97).  J = M2 @ M1 (density_filter.jl:98-107)."""
    g = prob.grid
    vol = cell_volumes(prob)
    I, Jc, V = [], [], []
    for c in range(g.ncells):
        for n in g.cells[c]:
            I.append(n); Jc.append(c); V.append(vol[c])
    M1 = sp.csr_matrix((V, (I, Jc)), shape=(g.nnodes, g.ncells))
    rs = np.asarray(M1.sum(axis=1)).ravel()
    M1 = sp.diags(np.where(rs != 0, 1.0 / np.where(rs != 0, rs, 1), 0.0)) @ M1
    nodes, ws = neighbour_info(prob, rmin)
    I, Jc, V = [], [], []
    for i in range(g.ncells):
        if not nodes[i]:
            continue
        s = sum(ws[i])
        for n, w in zip(nodes[i], ws[i]):
            I.append(i); Jc.append(n); V.append(w / s)
    if not V:
        raise ValueError("DensityFilterFun: no neighbouring nodes were found within rmin")
    M2 = sp.csr_matrix((V, (I, Jc)), shape=(g.ncells, g.nnodes))
    return M1.tocsr(), M2.tocsr()


class DensityFilter:
    """DensityFilterFun forward y = J x and pullback J' * D (density_filter.jl:35-47)."""

    def __init__(self, prob, rmin):
        self.M1, self.M2 = filter_matrices(prob, rmin)
        self.J = (self.M2 @ self.M1).tocsr()

    def forward(self, x):
        return self.J @ x

    def pullback(self, d):
        return self.J.T @ d


class SensFilter:
    """SensFilterFun: identity forward; pullback applies the node average then the
    cone average to the gradient (sens_filter.jl:49-111), i.e. J (not J')."""

    def __init__(self, prob, rmin):
        self.M1, self.M2 = filter_matrices(prob, rmin)

    def forward(self, x):
        return np.array(x, dtype=np.float64, copy=True)

    def pullback(self, d):
        return self.M2 @ (self.M1 @ d)


# --------------------------------------------------------------------------
# O1: optimality-criteria update  -- no reference implementation; restates the
# published OC update of the 88-line code (Andreassen et al. 2011, eq. for x_new
# with move limit m and damping eta = 1/2, bisection on lambda in [0, 1e9] until
# (l2-l1)/(l1+l2) <= 1e-3, volume measured on the physical (filtered) field).
# --------------------------------------------------------------------------

def heaviside_projection(x, beta):
    """HeavisideProjectionFun (src/Utilities/penalties.jl:75-84): y = 1 - exp(-beta x)
    + x exp(-beta); returns (y, dy/dx)."""
    x = np.asarray(x, dtype=np.float64)
    e = np.exp(-beta * x)
    return 1.0 - e + x * np.exp(-beta), beta * e + np.exp(-beta)


def sigmoid_projection(x, beta):
    """SigmoidProjectionFun (penalties.jl:86-94): y = 1 / (1 + exp((beta + 1) (-x + 0.5)));
    returns (y, dy/dx)."""
    x = np.asarray(x, dtype=np.float64)
    y = 1.0 / (1.0 + np.exp((beta + 1.0) * (-x + 0.5)))
    return y, (beta + 1.0) * y * (1.0 - y)


class ProjectedDensityFilter:
    """ProjectedDensityFilterFun (src/CheqFilters/density_filter.jl:130-169):
    y = postproj(J(preproj(x))); pullback by the chain rule (what Zygote computes
    through the filter's rrule and the elementwise projections).  pre / post are
    None or (function, beta)."""

    def __init__(self, filt, pre=None, post=None):
        self.filt, self.pre, self.post = filt, pre, post

    def forward(self, x):
        x = np.asarray(x, dtype=np.float64)
        self.dpre = self.dpost = None
        if self.pre is not None:
            x, self.dpre = self.pre[0](x, self.pre[1])
        y = self.filt.forward(x)
        if self.post is not None:
            y, self.dpost = self.post[0](y, self.post[1])
        return y

    def pullback(self, d):
        d = np.asarray(d, dtype=np.float64)
        if self.dpost is not None:
            d = d * self.dpost
        d = self.filt.pullback(d)
        if self.dpre is not None:
            d = d * self.dpre
        return d


class FixedElementProjector:
    """FixedElementProjectorFun (src/Functions/fixed_element.jl:13-58): black cells at
    density 1, white at 0, free cells copied from x_free in cell order; the pullback
    returns the cotangent of the free cells (fixed_element.jl:68-79).  black / white are
    boolean masks of length nel; both-black-and-white and length errors raise ValueError
    (the reference's ArgumentError, fixed_element.jl:20-23, 46-50)."""

    def __init__(self, nel, black, white):
        black = np.asarray(black, dtype=bool)
        white = np.asarray(white, dtype=bool)
        if black.shape != (nel,):
            raise ValueError("black must have length %d" % nel)
        if white.shape != (nel,):
            raise ValueError("white must have length %d" % nel)
        if np.any(black & white):
            raise ValueError("an element cannot be both black and white")
        self.nel, self.black, self.white = nel, black, white
        self.free = ~black & ~white

    @classmethod
    def from_cells(cls, nel, black_cells, white_cells):
        """get_fixed_element_projector(nel, black_cells, white_cells)
        (fixed_element.jl:150-159), with 0-based cell indices."""
        black = np.zeros(nel, dtype=bool)
        white = np.zeros(nel, dtype=bool)
        black[np.asarray(black_cells, dtype=np.int64)] = True
        white[np.asarray(white_cells, dtype=np.int64)] = True
        return cls(nel, black, white)

    @property
    def nfree(self):
        return int(np.count_nonzero(self.free))

    def __call__(self, x_free):
        x_free = np.asarray(x_free, dtype=np.float64)
        if x_free.shape != (self.nfree,):
            raise ValueError("x_free length (%d) must match number of free elements (%d)"
                             % (x_free.size, self.nfree))
        rho = np.empty(self.nel)
        rho[self.black] = 1.0
        rho[self.white] = 0.0
        rho[self.free] = x_free
        return rho

    def pullback(self, d):
        return np.asarray(d, dtype=np.float64)[self.free]


def oc_update(x, dc, dv, vol_weights, volfrac, move=0.2, l1=0.0, l2=1e9, tol=1e-3, fixed=None):
    """x_new = clamp(x * sqrt(max(0,-dc)/(dv*lmid)), max(0,x-move), min(1,x+move));
    volume(x_new) = sum(vol_weights * x_new) compared with volfrac * sum(...)
    on the same weights' total (vol_weights = colsum(J) / ncells for the density
    filter, 1/ncells without a filter).  fixed (a FixedElementProjector) holds its
    black / white cells at 1 / 0: their bounds collapse onto that value, and their
    volume counts against volfrac.  Returns (x_new, change, lmid, steps)."""
    x = np.asarray(x, dtype=np.float64)
    B = x * np.sqrt(np.maximum(0.0, -dc) / dv)
    lo = np.maximum(0.0, x - move)
    hi = np.minimum(1.0, x + move)
    if fixed is not None:
        lo[fixed.black] = hi[fixed.black] = 1.0
        lo[fixed.white] = hi[fixed.white] = 0.0
    steps = 0
    xnew = x
    while (l2 - l1) / (l1 + l2) > tol:
        lmid = 0.5 * (l2 + l1)
        xnew = np.minimum(hi, np.maximum(lo, B / math.sqrt(lmid)))
        vol = float(np.dot(vol_weights, xnew))
        if vol > volfrac:
            l1 = lmid
        else:
            l2 = lmid
        steps += 1
    lmid = 0.5 * (l2 + l1)
    xnew = np.minimum(hi, np.maximum(lo, B / math.sqrt(lmid)))
    change = float(np.max(np.abs(xnew - x)))
    return xnew, change, lmid, steps


class MMA:
    """MMA, the method of moving asymptotes (Svanberg 1987), for min f s.t. g <= 0 on
    x in [0, 1]^n: the optimizer of TopOpt.jl's SIMP scripts (Nonconvex MMA87,
    docs/tutorials/simp.qmd:107-114, test/integration/test_end_to_end.jl:30-47).
    Nonconvex is not part of TopOpt.jl (parity unpinned): this restates the published
    method with the rules of Svanberg's 2007 notes on MMA -- asymptotes x -/+ 0.5 for the
    first two iterations, then widened by 1.2 / narrowed by 0.7 as the last two steps
    agree / oscillate, kept in [x - 10, x - 0.01] / [x + 0.01, x + 10]; bounds
    alpha = max(L + 0.1 (x - L), x - move, 0), beta = min(U - 0.1 (U - x), x + move, 1);
    p = (U - x)^2 (max(df, 0) + 1e-3 |df| + 1e-5), q = (x - L)^2 (max(-df, 0) + 1e-3 |df|
    + 1e-5) -- and the subproblem solved through its dual in the single multiplier
    lambda by bisection in log lambda on [1e-30, 1e30] (lambda = 0 when the approximated
    constraint is inactive there)."""

    def __init__(self, n, move=0.5, fixed=None):
        self.n, self.move, self.fixed = n, move, fixed
        self.k = 0
        self.low = self.upp = self.x1 = self.x2 = None

    @staticmethod
    def _xlam(lam, p0, q0, p1, q1, L, U, a, b):
        sp, sq = np.sqrt(p0 + lam * p1), np.sqrt(q0 + lam * q1)
        return np.minimum(b, np.maximum(a, (L * sp + U * sq) / (sp + sq)))

    def update(self, x, df0, g, dg):
        """One MMA step from x with f's gradient df0, the constraint value g and its
        gradient dg.  Returns (x_new, change, lambda, dual evaluations)."""
        x = np.asarray(x, dtype=np.float64)
        df0 = np.asarray(df0, dtype=np.float64)
        dg = np.asarray(dg, dtype=np.float64)
        self.k += 1
        if self.k <= 2:
            L, U = x - 0.5, x + 0.5
        else:
            zz = (x - self.x1) * (self.x1 - self.x2)
            f = np.where(zz > 0, 1.2, np.where(zz < 0, 0.7, 1.0))
            L = x - f * (self.x1 - self.low)
            U = x + f * (self.upp - self.x1)
            L = np.minimum(np.maximum(L, x - 10.0), x - 0.01)
            U = np.minimum(np.maximum(U, x + 0.01), x + 10.0)
        a = np.maximum(np.maximum(L + 0.1 * (x - L), x - self.move), 0.0)
        b = np.minimum(np.minimum(U - 0.1 * (U - x), x + self.move), 1.0)
        if self.fixed is not None:
            a[self.fixed.black] = b[self.fixed.black] = 1.0
            a[self.fixed.white] = b[self.fixed.white] = 0.0
        ux2, xl2 = (U - x) ** 2, (x - L) ** 2
        r0, r1 = 1e-3 * np.abs(df0) + 1e-5, 1e-3 * np.abs(dg) + 1e-5
        p0, q0 = (np.maximum(df0, 0) + r0) * ux2, (np.maximum(-df0, 0) + r0) * xl2
        p1, q1 = (np.maximum(dg, 0) + r1) * ux2, (np.maximum(-dg, 0) + r1) * xl2
        r = float(np.sum(p1 / (U - x) + q1 / (x - L))) - g

        def h(lam):
            xe = self._xlam(lam, p0, q0, p1, q1, L, U, a, b)
            return float(np.sum(p1 / (U - xe) + q1 / (xe - L))) - r

        steps = 1
        if h(0.0) <= 0.0:
            lam = 0.0
        else:
            lo, hi = math.log(1e-30), math.log(1e30)
            while True:
                mid = 0.5 * (lo + hi)
                if h(math.exp(mid)) > 0.0:
                    lo = mid
                else:
                    hi = mid
                steps += 1
                if hi - lo <= 1e-12 or steps >= 72:
                    break
            lam = math.exp(0.5 * (lo + hi))
        xn = self._xlam(lam, p0, q0, p1, q1, L, U, a, b)
        self.low, self.upp = L, U
        self.x2, self.x1 = self.x1, x.copy()
        return xn, float(np.max(np.abs(xn - x))), lam, steps


def simp_iteration_mma(st: FEAState, x, filt, volfrac, mma: MMA, solve="direct", rtol=1e-10, maxiter=100000):
    """One design iteration with MMA in place of OC: the volume constraint
    g = sum(w x) - volfrac, w = J'(1/n) (the filtered volume fraction) with the density
    filter, 1/n otherwise (docs/tutorials/simp.qmd:86-114)."""
    xf = filt.forward(x) if filt is not None else x.copy()
    st.vars = xf
    if solve == "direct":
        u, its = direct_solve(st), 0
    else:
        u, its, _ = pcg(st, rtol=rtol, maxiter=maxiter)
    c, gr, _ = compliance(st, u, xf)
    n = st.prob.grid.ncells
    dv = np.full(n, 1.0 / n)
    if filt is not None:
        dc = filt.pullback(gr)
        dv = filt.pullback(dv) if isinstance(filt, DensityFilter) else dv
    else:
        dc = gr
    g = float(np.dot(dv, x)) - volfrac
    xnew, change, lam, steps = mma.update(x, dc, g, dv)
    return dict(x_new=xnew, xf=xf, u=u, c=c, dc=dc, dv=dv, change=change, lam=lam, steps=steps, cg_iters=its)


def multiload_compliance(st: FEAState, F, x):
    """Per-column compliance and cell gradient of a load matrix F (ndofs x n, reference
    dof rows): every column solved directly with its prescribed dofs zeroed, as the
    solver's matrix-rhs call (src/FEA/solvers_api.jl:293-348) followed by
    compute_compliance (src/Functions/mean_compliance.jl:78-99).  Returns (c[n],
    G[ncells, n])."""
    st.vars = np.asarray(x, dtype=np.float64)
    F = sp.csc_matrix(F)
    c = np.empty(F.shape[1])
    G = np.empty((st.prob.grid.ncells, F.shape[1]))
    for i in range(F.shape[1]):
        u = direct_solve(st, np.asarray(F[:, i].toarray()).ravel())
        c[i], G[:, i], _ = compliance(st, u, st.vars)
    return c, G


def mean_compliance(st: FEAState, F, x, method="exact"):
    """MeanComplianceFun (mean_compliance.jl:8-150) with method exact (mean over F's
    columns) or exact_svd (the columns U S of the thin SVD of F's nonzero rows, singular
    values > 1e-6, src/Functions/trace.jl:15-34, divided by F's column count).
    Returns (mean, gradient)."""
    F = sp.csc_matrix(F)
    n = F.shape[1]
    if method == "exact_svd":
        rows = np.unique(F.indices)
        U, S, _ = np.linalg.svd(F[rows, :].toarray(), full_matrices=False)
        keep = S > 1e-6
        US = np.zeros((F.shape[0], int(keep.sum())))
        US[rows, :] = U[:, keep] * S[keep]
        F = sp.csc_matrix(US)
    c, G = multiload_compliance(st, F, x)
    return float(c.sum() / n), G.sum(axis=1) / n


def simp_iteration(st: FEAState, x, filt, volfrac, move=0.2, solve="direct",
                   rtol=1e-10, maxiter=100000, vol_weights=None, fixed=None):
    """One design iteration: filter -> solve -> compliance/sens -> filter pullback
    -> OC (docs/tutorials/simp.qmd:86-114 with OC in place of MMA)."""
    xf = filt.forward(x) if filt is not None else x.copy()
    st.vars = xf
    if solve == "direct":
        u = direct_solve(st)
        its = 0
    else:
        u, its, _ = pcg(st, rtol=rtol, maxiter=maxiter)
    c, g, _ = compliance(st, u, xf)
    n = st.prob.grid.ncells
    dv = np.full(n, 1.0 / n)
    if filt is not None:
        dc = filt.pullback(g)
        dv = filt.pullback(dv) if isinstance(filt, DensityFilter) else dv
    else:
        dc = g
    if vol_weights is None:
        if isinstance(filt, DensityFilter):
            vol_weights = np.asarray(filt.J.sum(axis=0)).ravel() / n
        else:
            vol_weights = np.full(n, 1.0 / n)
    xnew, change, lam, steps = oc_update(x, dc, dv, vol_weights, volfrac, move, fixed=fixed)
    return dict(x_new=xnew, xf=xf, u=u, c=c, g=g, dc=dc, dv=dv, change=change,
                lam=lam, oc_steps=steps, cg_iters=its)
