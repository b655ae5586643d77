"""Host-side mirror of TopOpt.jl's API for the SIMP compliance path, driving
libtopopt_gb300 through its C ABI.  Names, argument meanings, defaults and
error behaviour follow the reference (paths relative to the TopOpt.jl root):

  PointLoadCantilever, HalfMBB      src/TopOptProblems/problem_types.jl:162-231, 324-395
  FEASolver(GB300Solver, problem)   src/FEA/solvers_api.jl:468-603 (CGMatrixFreeSolver's slot)
  PowerPenaltyFun                   src/Utilities/penalties.jl:30-33
  PseudoDensities                   src/TopOpt.jl:30-74
  ComplianceFun (+ pullback)        src/Functions/compliance.jl:28-76
  VolumeFun (+ pullback)            src/Functions/volume.jl:47-67
  DensityFilterFun / SensFilterFun  src/CheqFilters/density_filter.jl:25-47, sens_filter.jl:29-111
  oc_update, SIMPLoop               published OC update (no reference counterpart)
"""
import math

import numpy as np

from . import _lib as L


# --------------------------------------------------------------------------- numbering
def grid_counts(nels):
    nel = (L.C.c_int32 * 3)(*(list(nels) + [1] * (3 - len(nels))))
    nn, nc, nd = L.C.c_int64(), L.C.c_int64(), L.C.c_int64()
    L.check(L.lib().tog_grid_counts(len(nels), nel, L.C.byref(nn), L.C.byref(nc), L.C.byref(nd)))
    return nn.value, nc.value, nd.value


def node_dofs(nels):
    """Metadata.node_dofs as a (nnodes, dim) array of 0-based dofs (metadata.jl:116-145)."""
    dim = len(nels)
    nn, _, _ = grid_counts(nels)
    out = np.empty(nn * dim, dtype=np.int32)
    nel = (L.C.c_int32 * 3)(*(list(nels) + [1] * (3 - dim)))
    L.check(L.lib().tog_node_dofs(dim, nel, L.iptr(out)))
    return out.reshape(nn, dim)


def cell_dofs(nels):
    """Metadata.cell_dofs as a (ncells, ndpc) array of 0-based dofs (metadata.jl:40-50)."""
    dim = len(nels)
    _, nc, _ = grid_counts(nels)
    ndpc = (2 ** dim) * dim
    out = np.empty(nc * ndpc, dtype=np.int32)
    nel = (L.C.c_int32 * 3)(*(list(nels) + [1] * (3 - dim)))
    L.check(L.lib().tog_cell_dofs(dim, nel, L.iptr(out)))
    return out.reshape(nc, ndpc)


def element_stiffness(dim, sizes, E, nu, plane_stress=False):
    nd = (2 ** dim) * dim
    Ke = np.empty(nd * nd)
    sz = (L.C.c_double * 3)(*(list(sizes) + [1.0] * (3 - dim)))
    L.check(L.lib().tog_element_stiffness(dim, sz, E, nu, int(plane_stress), L.dptr(Ke)))
    return Ke.reshape(nd, nd)


# --------------------------------------------------------------------------- problems
class _StructuredProblem:
    def __init__(self, nels, sizes, E, nu, force, plane_stress):
        self.nels = tuple(int(n) for n in nels)
        self.sizes = tuple(float(s) for s in sizes)
        self.dim = len(self.nels)
        if self.dim not in (2, 3) or len(self.sizes) != self.dim:
            raise ValueError("nels and sizes must both have 2 or 3 entries")
        self.E, self.nu, self.force = float(E), float(nu), float(force)
        self.plane_stress = bool(plane_stress)
        self.nnodes, self.ncells, self.ndofs = grid_counts(self.nels)
        self.node_dofs = node_dofs(self.nels)          # (nnodes, dim)
        self.nn = tuple(n + 1 for n in self.nels)

    def node_id(self, ix, iy, iz=0):
        return ix + self.nn[0] * (iy + self.nn[1] * iz)

    def _node_grid(self):
        idx = np.arange(self.nnodes)
        ix = idx % self.nn[0]
        iy = (idx // self.nn[0]) % self.nn[1]
        iz = idx // (self.nn[0] * self.nn[1]) if self.dim == 3 else np.zeros_like(idx)
        return ix, iy, iz

    def load_vector(self):
        f = np.zeros(self.ndofs)
        f[self.force_dof] = -self.force     # getcloaddict: [0, -force, 0] (problem_types.jl:398-402)
        return f


class PointLoadCantilever(_StructuredProblem):
    """Left face clamped; load [0, -force, 0] at the first node of right & middley
    (problem_types.jl:162-231).  load='face_centre' moves the 3D load to the
    centre of the right face (not the reference's node)."""

    def __init__(self, nels, sizes, E=1.0, nu=0.3, force=1.0, *, load="reference_first_node",
                 plane_stress=False):
        if nels[1] % 2 or (len(nels) == 3 and nels[2] % 2):
            raise ValueError("Grid does not have an even number of elements along the y and/or z axes.")
        super().__init__(nels, sizes, E, nu, force, plane_stress)
        ix, iy, iz = self._node_grid()
        left = np.nonzero(ix == 0)[0]
        self.fixed_dofs = np.sort(self.node_dofs[left].ravel()).astype(np.int32)
        kz = self.nels[2] // 2 if (self.dim == 3 and load == "face_centre") else 0
        self.load_node = self.node_id(self.nels[0], self.nels[1] // 2, kz)
        self.force_dof = int(self.node_dofs[self.load_node, 1])


class LoadedCantilever(_StructuredProblem):
    """3D cantilever with the left face clamped and a point load of magnitude `force` in
    direction `direction` at the node (nelx, iy, iz) of the free face (the training runs of
    the learned warm start; PointLoadCantilever is the case iy = nely / 2, iz = 0,
    direction -y)."""

    def __init__(self, nels, sizes, node, direction, E=1.0, nu=0.3, force=1.0):
        super().__init__(nels, sizes, E, nu, force, False)
        if self.dim != 3:
            raise ValueError("LoadedCantilever is 3D")
        ix, iy, iz = self._node_grid()
        self.fixed_dofs = np.sort(self.node_dofs[np.nonzero(ix == 0)[0]].ravel()).astype(np.int32)
        self.load_node = self.node_id(self.nels[0], int(node[0]), int(node[1]))
        d = np.asarray(direction, dtype=np.float64)
        self.direction = d / np.linalg.norm(d)

    def load_vector(self):
        f = np.zeros(self.ndofs)
        f[self.node_dofs[self.load_node]] = self.force * self.direction
        return f


class HalfMBB(_StructuredProblem):
    """u1 = 0 on the left face, u2 = 0 on bottom & right, load [0, -force] at the
    first node of top & left (problem_types.jl:324-395)."""

    def __init__(self, nels, sizes, E=1.0, nu=0.3, force=1.0, *, plane_stress=False):
        super().__init__(nels, sizes, E, nu, force, plane_stress)
        ix, iy, iz = self._node_grid()
        f1 = self.node_dofs[np.nonzero(ix == 0)[0], 0]
        f2 = self.node_dofs[np.nonzero((iy == 0) & (ix == self.nels[0]))[0], 1]
        self.fixed_dofs = np.sort(np.concatenate([f1, f2])).astype(np.int32)
        self.load_node = self.node_id(0, self.nels[1], 0)
        self.force_dof = int(self.node_dofs[self.load_node, 1])


# --------------------------------------------------------------------------- solver
class PowerPenaltyFun:
    def __init__(self, p):
        self.p = float(p)


class PseudoDensities:
    def __init__(self, x):
        self.x = np.ascontiguousarray(x, dtype=np.float64)


class DefaultCriteria:
    """The residual-norm stop of IterativeSolvers' cg! (src/FEA/convergence_criteria.jl:13)."""
    code = L.TOG_CONV_DEFAULT


class EnergyCriteria:
    """EnergyCriteria (src/FEA/convergence_criteria.jl:20-45): stop when the relative change
    of x'Ax and |x'r| / x'Ax are both within the solve tolerance (FP64 solves)."""
    code = L.TOG_CONV_ENERGY


class GB300Solver:
    """Marker type: FEASolver(GB300Solver, problem; ...) -- the AbstractLinearSolver
    slot of solvers_api.jl:44 filled by libtopopt_gb300."""


PRECISIONS = {"fp64": L.TOG_FP64, "fp32_ir": L.TOG_FP32_IR}
WARM_MODES = {False: 0, True: 1, 0: 0, 1: 1, 2: 2, 3: 3, "cold": 0, "previous": 1, "learned": 2, "extrapolate": 3}


class GB300FEASolver:
    """Matrix-free SIMP solver resident on the GPU.  Defaults follow
    FEASolver (solvers_api.jl:468-489): xmin = 1e-3, penalty = PowerPenaltyFun(1),
    cg_max_iter = 700, abstol = 1e-7, rtol = sqrt(eps) (IterativeSolvers' reltol)."""

    def __init__(self, problem, *, xmin=None, penalty=None, cg_max_iter=700, abstol=None, rtol=None,
                 precision="fp64", warm_start=False, conv=None):
        self.problem = problem
        self.xmin = 1e-3 if xmin is None else float(xmin)
        self.penalty = PowerPenaltyFun(1.0) if penalty is None else penalty
        self.cg_max_iter = int(cg_max_iter)
        self.abstol = 1e-7 if abstol is None else float(abstol)
        self.rtol = math.sqrt(np.finfo(np.float64).eps) if rtol is None else float(rtol)
        if precision not in PRECISIONS:
            raise ValueError("precision must be one of %s" % sorted(PRECISIONS))
        self.precision = precision
        # False / True (previous displacement) / "learned" (previous displacement moved by
        # the Galerkin step on an attached WarmStartNet's correction and the last change) /
        # "extrapolate" (the same step along the last change alone); SIMP steps of 3D problems
        self.warm_start = WARM_MODES[warm_start]
        self.net = None
        d = L.ProblemDesc()
        d.dim = problem.dim
        for i in range(problem.dim):
            d.nel[i] = problem.nels[i]
            d.size[i] = problem.sizes[i]
        d.E, d.nu, d.plane_stress = problem.E, problem.nu, int(problem.plane_stress)
        d.xmin, d.penalty = self.xmin, self.penalty.p
        h = L.C.c_void_p()
        L.check(L.lib().tog_create(L.C.byref(d), L.C.byref(h)))
        self.handle = h
        fd = np.ascontiguousarray(problem.fixed_dofs, dtype=np.int32)
        L.check(L.lib().tog_set_fixed_dofs(h, len(fd), L.iptr(fd)))
        f = np.ascontiguousarray(problem.load_vector())
        L.check(L.lib().tog_set_rhs(h, L.dptr(f)))
        # conv = DefaultCriteria() (solvers_api.jl:482) or EnergyCriteria()
        self.conv = DefaultCriteria() if conv is None else conv
        L.check(L.lib().tog_set_convergence(h, self.conv.code))
        self.vars = np.ones(problem.ncells)          # solvers_api.jl:502
        self.last_stats = None

    # -- reference-style accessors
    def close(self):
        if getattr(self, "handle", None):
            L.lib().tog_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def attach_network(self, net):
        """Use a WarmStartNet (created for this grid's nodes, batch 1) for warm_start="learned"."""
        L.check(L.lib().tog_set_warm_start_net(self.handle, net.handle if net is not None else None))
        self.net = net

    def enable_previous_state(self):
        """Keep the previous iteration's state on the device (needed by warm_start="extrapolate")."""
        L.check(L.lib().tog_keep_previous_state(self.handle))

    def record_next_step(self, inp, target):
        """The next SIMP step writes its network input / target into these CUDA tensors
        (shapes (1, nz, ny, nx, 8) and (1, nz, ny, nx, 3)) when it has a previous iteration."""
        L.check(L.lib().tog_record_next_step(self.handle, L.C.c_void_p(inp.data_ptr()),
                                             L.C.c_void_p(target.data_ptr())))

    def record_status(self):
        w = L.C.c_int32()
        L.check(L.lib().tog_record_status(self.handle, L.C.byref(w)))
        return bool(w.value)

    def setpenalty(self, p):
        self.penalty = p if isinstance(p, PowerPenaltyFun) else PowerPenaltyFun(p)
        L.check(L.lib().tog_set_penalty(self.handle, self.penalty.p))

    def _push_vars(self):
        v = np.ascontiguousarray(self.vars, dtype=np.float64)
        if v.shape != (self.problem.ncells,):
            raise ValueError("DimensionMismatch: vars must have one entry per cell")
        L.check(L.lib().tog_set_vars(self.handle, L.dptr(v)))

    def __call__(self, precision=None, warm_start=None):
        """solver(): solve K(vars) u = f (solvers_api.jl:285-374)."""
        self._push_vars()
        st = L.SolveStats()
        prec = PRECISIONS[precision or self.precision]
        warm = self.warm_start if warm_start is None else WARM_MODES[warm_start]
        L.check(L.lib().tog_solve(self.handle, prec, self.rtol, self.abstol, self.cg_max_iter, int(warm),
                                  L.C.byref(st)))
        self.last_stats = st
        return None

    @property
    def u(self):
        out = np.empty(self.problem.ndofs)
        L.check(L.lib().tog_get_u(self.handle, L.dptr(out)))
        return out

    @u.setter
    def u(self, v):
        v = np.ascontiguousarray(v, dtype=np.float64)
        L.check(L.lib().tog_set_u(self.handle, L.dptr(v)))

    def matvec(self, x):
        """mul!(y, MatrixFreeOperator, x) at the current vars (matrix_free_operator.jl:66-105)."""
        self._push_vars()
        x = np.ascontiguousarray(x, dtype=np.float64)
        y = np.empty_like(x)
        L.check(L.lib().tog_matvec(self.handle, L.dptr(x), L.dptr(y)))
        return y

    def pcg_operator(self, r, p_old, beta, precision="fp32_ir"):
        """One launch of the PCG's fused operator kernel at the current vars:
        p = D^-1 r + beta p_old and q = K p (prescribed rows meandiag p), p.q
        (the inner loop of cg!, solvers_api.jl:197-218)."""
        self._push_vars()
        r = np.ascontiguousarray(r, dtype=np.float64)
        p_old = np.ascontiguousarray(p_old, dtype=np.float64)
        p, q = np.empty_like(r), np.empty_like(r)
        pq = L.C.c_double()
        prec = L.TOG_FP64 if precision == "fp64" else L.TOG_FP32_IR
        L.check(L.lib().tog_pcg_operator(self.handle, prec, float(beta), L.dptr(r), L.dptr(p_old), L.dptr(p),
                                         L.dptr(q), L.C.byref(pq)))
        return p, q, pq.value


def FEASolver(solver_type, problem, **kw):
    if solver_type is not GB300Solver:
        raise ValueError("this library provides FEASolver(GB300Solver, problem; ...)")
    return GB300FEASolver(problem, **kw)


# --------------------------------------------------------------------------- functions
class ComplianceFun:
    """J = sum rho_e u_e' Ke u_e with dJ/dx_e = -drho_e u_e' Ke u_e (compliance.jl:58-76)."""

    def __init__(self, solver):
        self.solver = solver
        self.grad = np.zeros(solver.problem.ncells)
        self.cell_comp = None

    def __call__(self, x):
        if not isinstance(x, PseudoDensities):
            x = PseudoDensities(x)
        s = self.solver
        s.vars = x.x.copy()
        s()
        c = L.C.c_double()
        g = np.empty(s.problem.ncells)
        L.check(L.lib().tog_compliance(s.handle, L.C.byref(c), L.dptr(g)))
        self.grad = g
        return c.value

    def pullback(self, delta=1.0):
        return self.grad * delta


class VolumeFun:
    """Volume fraction sum x_e v_e / sum v_e and its constant gradient (volume.jl:47-67)."""

    def __init__(self, solver, fraction=True):
        n = solver.problem.ncells
        self.cellvolumes = np.full(n, float(np.prod(solver.problem.sizes)))
        self.total_volume = float(self.cellvolumes.sum())
        self.fraction = fraction
        self.grad = self.cellvolumes / self.total_volume if fraction else self.cellvolumes.copy()

    def __call__(self, x):
        x = x.x if isinstance(x, PseudoDensities) else np.asarray(x)
        v = float(np.dot(self.cellvolumes, x))
        return v / self.total_volume if self.fraction else v

    def pullback(self, delta=1.0):
        return self.grad * delta


# --------------------------------------------------------------------------- multiple loads
class MultiLoad:
    """MultiLoad(problem, F) (src/TopOptProblems/multiload.jl:21-46): a structured problem
    with a load matrix F (ndofs x nscenarios, scipy sparse or dense, 0-based reference dof
    rows) in place of its single load.  MultiLoad(problem, N, load_rules) builds F from
    [(position, f)] pairs, f() returning the load vector of one scenario, placed on the dofs
    of the node nearest to position (find_nearest_dofs, multiload.jl:48-61).  Other
    attributes are the base problem's."""

    def __init__(self, problem, F, load_rules=None):
        import scipy.sparse as sp
        self.problem = problem
        if load_rules is not None:
            N = int(F)
            I, J, V = [], [], []
            for pos, f in load_rules:
                dofs = find_nearest_dofs(problem, pos)
                for i in range(N):
                    load = np.asarray(f(), dtype=np.float64)
                    I.extend(dofs.tolist())
                    J.extend([i] * len(dofs))
                    V.extend(load.tolist())
            F = sp.csc_matrix((V, (I, J)), shape=(problem.ndofs, N))
        self.F = sp.csc_matrix(F, dtype=np.float64)
        if self.F.shape[0] != problem.ndofs:
            raise ValueError("DimensionMismatch: F must have one row per dof")

    def __getattr__(self, name):
        return getattr(self.__dict__["problem"], name)


def find_nearest_dofs(problem, pos):
    """The dofs of the node nearest to pos (multiload.jl:48-61)."""
    ix, iy, iz = problem._node_grid()
    coords = np.stack([ix * problem.sizes[0], iy * problem.sizes[1]] +
                      ([iz * problem.sizes[2]] if problem.dim == 3 else []), axis=1)
    d = np.linalg.norm(coords - np.asarray(pos, dtype=np.float64)[None, :], axis=1)
    return problem.node_dofs[int(np.argmin(d))]


def generate_scenarios(dof, size, f, perturb=None, rng=None):
    """Sparse ndofs x nscenarios load matrix with load f (1 + perturb()) at the single dof
    `dof` (0-based) in every scenario (mean_compliance.jl:209-219); perturb defaults to
    U(-0.5, 0.5) from a seeded numpy generator."""
    import scipy.sparse as sp
    ndofs, ns = size
    if perturb is None:
        g = rng if rng is not None else np.random.default_rng(0)
        perturb = lambda: g.random() - 0.5   # noqa: E731
    V = [f * (1.0 + perturb()) for _ in range(ns)]
    return sp.csc_matrix((V, ([dof] * ns, list(range(ns)))), shape=(ndofs, ns))


def hutch_rand(V, rng=None):
    """Rademacher (+-1) samples into V (hutch_rand!, mean_compliance.jl:151-158)."""
    g = rng if rng is not None else np.random.default_rng(0)
    V[...] = g.choice(np.array([-1.0, 1.0]), size=V.shape)
    return V


def hadamard(V):
    """Hadamard (+-1) columns into V (hadamard!, mean_compliance.jl:186-197): the first nv
    columns of a Sylvester matrix, its rows repeated down to n."""
    n, nv = V.shape
    H = np.ones((1, 1))
    while H.shape[0] < nv:
        H = np.block([[H, H], [H, -H]])
    H = H[:, :nv]
    H = np.tile(H, (int(np.ceil(n / nv)), 1))
    V[...] = H[:n, :]
    return V


def _svd_columns(F):
    """US of the thin SVD of F's nonzero rows, singular values > 1e-6 (ExactSVDMean,
    src/Functions/trace.jl:15-34)."""
    import scipy.sparse as sp
    rows = np.unique(F.indices)
    Fc = F[rows, :].toarray()
    U, S, _ = np.linalg.svd(Fc, full_matrices=False)
    keep = np.nonzero(S > 1e-6)[0]
    US = U[:, keep] * S[keep]
    out = np.zeros((F.shape[0], len(keep)))
    out[rows, :] = US
    return sp.csc_matrix(out)


class _MultiLoadSolves:
    def __init__(self, solver):
        self.solver = solver
        self.last_stats = None

    def solve(self, cols, x, precision=None):
        """Per-column compliance f_i' K(x)^-1 f_i of the CSC columns at densities x (the
        column gradients stay on the device)."""
        s = self.solver
        s.vars = np.asarray(x.x if isinstance(x, PseudoDensities) else x, dtype=np.float64).copy()
        s._push_vars()
        cols = cols.tocsc()
        cols.sort_indices()
        colptr = np.ascontiguousarray(cols.indptr, dtype=np.int64)
        rowval = np.ascontiguousarray(cols.indices, dtype=np.int32)
        nzval = np.ascontiguousarray(cols.data, dtype=np.float64)
        c = np.empty(cols.shape[1])
        st = L.SolveStats()
        L.check(L.lib().tog_multiload_compliance(s.handle, cols.shape[1], colptr.ctypes.data_as(L._I64),
                                                 L.iptr(rowval), L.dptr(nzval),
                                                 PRECISIONS[precision or s.precision], s.rtol, s.abstol,
                                                 s.cg_max_iter, L.dptr(c), L.C.byref(st)))
        self.last_stats = st
        return c

    def gradient(self, w):
        w = np.ascontiguousarray(w, dtype=np.float64)
        out = np.empty(self.solver.problem.ncells)
        L.check(L.lib().tog_multiload_gradient(self.solver.handle, len(w), L.dptr(w), L.dptr(out)))
        return out


class MeanComplianceFun:
    """Mean compliance over the load cases of a MultiLoad problem (mean_compliance.jl:8-150):
    method "exact" (every column of F), "exact_svd" (the columns U S of F's thin SVD; the
    default), "trace" (Hutchinson / Hadamard estimation with nv probe vectors: the columns
    F v) or "trace_svd" (the same on U S).  The solves, compliances and gradients run on the
    device; F's SVD and the probes are set up once on the host, as in the reference."""

    def __init__(self, problem, solver, method="exact_svd", sample_once=True, nv=None, V=None,
                 sample_method="hutch", rng=None):
        if not isinstance(problem, MultiLoad):
            raise ValueError("MeanComplianceFun needs a MultiLoad problem")
        self.F, self.n = problem.F, problem.F.shape[1]
        self.method, self.sample_once = method, sample_once
        self.rng = rng if rng is not None else np.random.default_rng(0)
        self._ml = _MultiLoadSolves(solver)
        self.solver = solver
        if method == "exact":
            self.base, self.V = self.F, None
        elif method == "exact_svd":
            self.base, self.V = _svd_columns(self.F), None
        elif method in ("trace", "approx", "trace_svd"):
            self.base = self.F if method != "trace_svd" else _svd_columns(self.F)
            self.sampler = hadamard if sample_method == "hadamard" else (lambda A: hutch_rand(A, self.rng))
            if V is None:   # probes sampled at construction (and again per call unless sample_once)
                self.V = np.zeros((self.base.shape[1], 1 if nv is None else int(nv)))
                self.sampler(self.V)
            else:
                V = np.asarray(V, dtype=np.float64)
                self.V = V[:, :(V.shape[1] if nv is None else int(nv))].copy()
            if method == "trace_svd" and sample_method == "hadamard":
                self.sample_once = True
        else:
            raise ValueError("method must be exact, exact_svd, trace or trace_svd")
        self.grad = np.zeros(solver.problem.ncells)

    def _columns(self):
        import scipy.sparse as sp
        if self.V is None:
            return self.base, self.n
        if not self.sample_once:
            self.sampler(self.V)
        return sp.csc_matrix(self.base @ self.V), self.V.shape[1] * self.n

    def __call__(self, x):
        cols, div = self._columns()
        c = self._ml.solve(cols, x)
        self.grad = self._ml.gradient(np.full(cols.shape[1], 1.0 / div))
        return float(np.sum(c) / div)

    def pullback(self, delta=1.0):
        return self.grad * delta


class BlockComplianceFun:
    """The vector of per-load-case compliances f_i' K^-1 f_i of a MultiLoad problem
    (block_compliance.jl:7-110, method "exact"); pullback(delta) = sum_i delta_i dc_i/dx."""

    def __init__(self, problem, solver, method="exact"):
        if not isinstance(problem, MultiLoad):
            raise ValueError("BlockComplianceFun needs a MultiLoad problem")
        if method != "exact":
            raise ValueError("BlockComplianceFun: only method exact is provided")
        self.F = problem.F
        self._ml = _MultiLoadSolves(solver)
        self.solver = solver
        self.val = np.zeros(self.F.shape[1])
        self.fevals = 0

    def __call__(self, x):
        self.fevals += 1
        self.val = self._ml.solve(self.F, x)
        return self.val.copy()

    def pullback(self, delta):
        d = np.asarray(delta, dtype=np.float64)
        if d.shape != (self.F.shape[1],):
            raise ValueError("DimensionMismatch: BlockComplianceFun pullback expects one weight per load case")
        return self._ml.gradient(d)


class _NodeFilter:
    def __init__(self, solver, rmin):
        self.solver = solver
        self.rmin = float(rmin)
        try:
            L.check(L.lib().tog_filter_setup(solver.handle, self.rmin))
        except L.TopOptError as e:
            if e.code == L.TOG_ERR_ARG:
                raise ValueError(str(e)) from None   # ArgumentError in the reference
            raise

    def _apply(self, op, v):
        v = np.ascontiguousarray(v.x if isinstance(v, PseudoDensities) else v, dtype=np.float64)
        out = np.empty_like(v)
        L.check(L.lib().tog_filter_apply(self.solver.handle, op, L.dptr(v), L.dptr(out)))
        return out


class DensityFilterFun(_NodeFilter):
    """y = J x; pullback J' * delta (density_filter.jl:35-47)."""

    def __call__(self, x):
        return PseudoDensities(self._apply(L.TOG_FILTER_J, x))

    def pullback(self, delta):
        return self._apply(L.TOG_FILTER_JT, delta)


class SensFilterFun(_NodeFilter):
    """Identity forward; pullback applies the node and cone averages, J * delta
    (sens_filter.jl:49-111)."""

    def __call__(self, x):
        return PseudoDensities(np.array(x.x if isinstance(x, PseudoDensities) else x, dtype=np.float64))

    def pullback(self, delta):
        return self._apply(L.TOG_FILTER_J, delta)


class HeavisideProjectionFun:
    """y = 1 - exp(-beta x) + x exp(-beta) (penalties.jl:75-84)."""
    kind = L.TOG_PROJ_HEAVISIDE

    def __init__(self, beta):
        self.beta = float(beta)


class SigmoidProjectionFun:
    """y = 1 / (1 + exp((beta + 1) (0.5 - x))) (penalties.jl:86-94)."""
    kind = L.TOG_PROJ_SIGMOID

    def __init__(self, beta):
        self.beta = float(beta)


def _project(solver, proj, x):
    x = np.ascontiguousarray(x, dtype=np.float64)
    if x.shape != (solver.problem.ncells,):
        raise ValueError("DimensionMismatch: one value per cell")
    y, dy = np.empty_like(x), np.empty_like(x)
    L.check(L.lib().tog_projection(solver.handle, proj.kind, proj.beta, L.dptr(x), L.dptr(y), L.dptr(dy)))
    return y, dy


class ProjectedDensityFilterFun:
    """y = postproj(J(preproj(x))) (density_filter.jl:130-169): a density filter with a
    projection before and/or after it; the pullback is the chain rule,
    preproj'(x) * J'(postproj'(Jx~) * delta).  ProjectedDensityFilterFun(solver, rmin=...,
    projection=HeavisideProjectionFun(10.0)) is the reference's convenience constructor
    (filter, then the projection)."""

    def __init__(self, filter_or_solver, preproj=None, postproj=None, *, rmin=None, projection="default"):
        if isinstance(filter_or_solver, DensityFilterFun):
            self.filter = filter_or_solver
            self.preproj, self.postproj = preproj, postproj
        else:
            if rmin is None:
                raise ValueError("ProjectedDensityFilterFun(solver; rmin, projection) needs rmin")
            self.filter = DensityFilterFun(filter_or_solver, rmin)
            self.preproj = None
            self.postproj = HeavisideProjectionFun(10.0) if projection == "default" else projection
        self.solver = self.filter.solver
        self._d_pre = self._d_post = None

    def __call__(self, x):
        x = np.asarray(x.x if isinstance(x, PseudoDensities) else x, dtype=np.float64)
        self._d_pre = None
        if self.preproj is not None:
            x, self._d_pre = _project(self.solver, self.preproj, x)
        fx = self.filter(x).x
        self._d_post = None
        if self.postproj is not None:
            fx, self._d_post = _project(self.solver, self.postproj, fx)
        return PseudoDensities(fx)

    def pullback(self, delta):
        d = np.asarray(delta, dtype=np.float64)
        if self._d_post is not None:
            d = d * self._d_post
        d = self.filter.pullback(d)
        if self._d_pre is not None:
            d = d * self._d_pre
        return d


class FixedElementProjectorFun:
    """FixedElementProjectorFun(nel, black, white) (src/Functions/fixed_element.jl:13-58):
    maps the free design variables to the full density vector, black cells at 1, white at
    0, free cells copied in cell order; the pullback passes the cotangent of the free cells
    only (fixed_element.jl:68-79).  black / white are boolean masks of length nel (the
    reference's BitVectors); a cell that is both, or a mask of another length, raises
    ValueError (the reference's ArgumentError).

    The projection runs on the device of the solver it is attached to
    (get_fixed_element_projector(solver, ...) or attach(solver)).  Attaching also sets
    that solver's active-element mask, so its SIMPLoop and oc_update hold the fixed cells
    at their densities."""

    def __init__(self, nel, black, white):
        nel = int(nel)
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
        self.solver = None

    def attach(self, solver):
        if solver.problem.ncells != self.nel:
            raise ValueError("DimensionMismatch: the projector has %d cells, the problem %d"
                             % (self.nel, solver.problem.ncells))
        state = np.zeros(self.nel, dtype=np.uint8)
        state[self.black] = L.TOG_ELEM_BLACK
        state[self.white] = L.TOG_ELEM_WHITE
        L.check(L.lib().tog_set_fixed_elements(solver.handle, state.ctypes.data_as(L.C.c_void_p)))
        self.solver = solver
        return self

    def detach(self):
        """Make every cell of the attached solver free again."""
        if self.solver is not None:
            L.check(L.lib().tog_set_fixed_elements(self.solver.handle, None))
            self.solver = None

    def _handle(self):
        if self.solver is None:
            raise RuntimeError("FixedElementProjectorFun runs on the device: attach it to a GB300FEASolver "
                               "(get_fixed_element_projector(solver, black_cells, white_cells)) first")
        return self.solver.handle

    def __call__(self, x_free):
        h = self._handle()
        x = np.ascontiguousarray(x_free.x if isinstance(x_free, PseudoDensities) else x_free, dtype=np.float64)
        if x.ndim != 1:
            raise ValueError("x_free must be a vector")
        rho = np.empty(self.nel)
        try:
            L.check(L.lib().tog_fixed_element_project(h, L.dptr(x) if x.size else None, x.size, L.dptr(rho)))
        except L.TopOptError as e:
            if e.code == L.TOG_ERR_ARG:
                raise ValueError(str(e)) from None   # ArgumentError in the reference
            raise
        return rho

    def pullback(self, drho):
        h = self._handle()
        d = np.ascontiguousarray(drho, dtype=np.float64)
        if d.shape != (self.nel,):
            raise ValueError("DimensionMismatch: one cotangent per cell")
        out = np.empty(get_free_variable_count(self))
        L.check(L.lib().tog_fixed_element_pullback(h, L.dptr(d), L.dptr(out) if out.size else None))
        return out


def get_free_variables(p):
    """The free-cell mask (fixed_element.jl:88)."""
    return p.free


def get_free_variable_count(p):
    """count(free) (fixed_element.jl:95)."""
    return int(np.count_nonzero(p.free))


def get_fixed_element_projector(target, black_cells, white_cells):
    """get_fixed_element_projector(problem | nel, black_cells, white_cells)
    (fixed_element.jl:127-159) with 0-based cell indices (the reference's are 1-based).
    Given a GB300FEASolver it also attaches the projector to it."""
    if isinstance(target, GB300FEASolver):
        nel = target.problem.ncells
    elif hasattr(target, "ncells"):
        nel = target.ncells
    else:
        nel = int(target)
    black = np.zeros(nel, dtype=bool)
    white = np.zeros(nel, dtype=bool)
    black[np.asarray(black_cells, dtype=np.int64)] = True
    white[np.asarray(white_cells, dtype=np.int64)] = True
    p = FixedElementProjectorFun(nel, black, white)
    if isinstance(target, GB300FEASolver):
        p.attach(target)
    return p


def oc_update(solver, x, dc, dv, vol_weights, volfrac, move=0.2):
    """Optimality-criteria update (published method; no reference counterpart).
    Returns (x_new, change, lambda)."""
    x = np.ascontiguousarray(x, dtype=np.float64)
    dc = np.ascontiguousarray(dc, dtype=np.float64)
    dv = np.ascontiguousarray(dv, dtype=np.float64)
    w = np.ascontiguousarray(vol_weights, dtype=np.float64)
    xn = np.empty_like(x)
    ch, lam = L.C.c_double(), L.C.c_double()
    L.check(L.lib().tog_oc_update(solver.handle, L.dptr(x), L.dptr(dc), L.dptr(dv), L.dptr(w), float(volfrac),
                                  float(move), L.dptr(xn), L.C.byref(ch), L.C.byref(lam)))
    return xn, ch.value, lam.value


def mma_update(solver, x, df0, g, dg, move=0.5):
    """One MMA step on the device (Svanberg's method of moving asymptotes, the optimizer
    of the reference's SIMP scripts through Nonconvex MMA87; see include/topopt_gb300.h):
    min f s.t. g(x) <= 0 on [0, 1]^n, with the asymptotes and the last two iterates kept
    in the solver's handle between calls (mma_reset(solver) starts over).
    Returns (x_new, change, lambda)."""
    x = np.ascontiguousarray(x, dtype=np.float64)
    df0 = np.ascontiguousarray(df0, dtype=np.float64)
    dg = np.ascontiguousarray(dg, dtype=np.float64)
    xn = np.empty_like(x)
    ch, lam = L.C.c_double(), L.C.c_double()
    L.check(L.lib().tog_mma_update(solver.handle, L.dptr(x), L.dptr(df0), float(g), L.dptr(dg), float(move),
                                   L.dptr(xn), L.C.byref(ch), L.C.byref(lam)))
    return xn, ch.value, lam.value


def mma_reset(solver):
    L.check(L.lib().tog_mma_reset(solver.handle))


class SIMPLoop:
    """Device-resident SIMP design loop: filter -> solve -> compliance/sensitivities
    -> filter pullback -> OC, one C-ABI call per design iteration."""

    FILTERS = {"none": L.TOG_FILTER_NONE, "density": L.TOG_FILTER_DENSITY, "sens": L.TOG_FILTER_SENS}

    OPTIMIZERS = {"oc": L.TOG_OPT_OC, "mma": L.TOG_OPT_MMA}

    def __init__(self, solver, *, volfrac, rmin=0.0, filter="density", move=None, x0=None, optimizer="oc"):
        """optimizer "oc" (move default 0.2) or "mma" (the volume constraint through MMA,
        move default 0.5)."""
        self.solver = solver
        n = solver.problem.ncells
        if optimizer not in self.OPTIMIZERS:
            raise ValueError("optimizer must be one of %s" % sorted(self.OPTIMIZERS))
        x0 = np.full(n, float(volfrac)) if x0 is None else np.ascontiguousarray(x0, dtype=np.float64)
        oc_move = 0.2 if (move is None or optimizer != "oc") else float(move)
        L.check(L.lib().tog_simp_set_optimizer(solver.handle, self.OPTIMIZERS[optimizer],
                                               0.0 if (move is None or optimizer != "mma") else float(move)))
        L.check(L.lib().tog_simp_init(solver.handle, self.FILTERS[filter], float(rmin), float(volfrac), oc_move,
                                      L.dptr(x0)))

    def step(self, precision=None, rtol=None, maxiter=None, warm_start=None):
        s = self.solver
        st = L.IterStats()
        code = L.lib().tog_simp_step(s.handle, PRECISIONS[precision or s.precision],
                                     s.rtol if rtol is None else float(rtol),
                                     s.cg_max_iter if maxiter is None else int(maxiter),
                                     s.warm_start if warm_start is None else WARM_MODES[warm_start],
                                     L.C.byref(st))
        L.check(code)
        return st

    @property
    def x(self):
        out = np.empty(self.solver.problem.ncells)
        L.check(L.lib().tog_get_design(self.solver.handle, L.dptr(out)))
        return out

    @x.setter
    def x(self, v):
        v = np.ascontiguousarray(v, dtype=np.float64)
        L.check(L.lib().tog_set_design(self.solver.handle, L.dptr(v)))

    @property
    def physical(self):
        out = np.empty(self.solver.problem.ncells)
        L.check(L.lib().tog_get_physical(self.solver.handle, L.dptr(out)))
        return out


# --------------------------------------------------------------------------- batched 2D
def uneven_cantilever_set(n=256, seed=0):
    """The seeded set of uneven 2D cantilevers of the batched benchmark: nelx ~ U{64..512} (even),
    nely = nelx / 2, the load node uniform on the right edge, volume fraction
    ~ U[0.3, 0.6], rmin ~ U[1.5, 3.0], from numpy default_rng(seed)."""
    rng = np.random.default_rng(seed)
    nelx = 2 * rng.integers(32, 257, size=n)
    nely = nelx // 2
    load_j = np.array([rng.integers(0, ny + 1) for ny in nely])
    volfrac = rng.uniform(0.3, 0.6, size=n)
    rmin = rng.uniform(1.5, 3.0, size=n)
    return dict(nelx=nelx, nely=nely, load_j=load_j, volfrac=volfrac, rmin=rmin, seed=seed)


class BatchedSIMP:
    """Many independent 2D cantilevers (left edge clamped, unit load [0, -1] at node
    (nelx, load_j)), each with its own size, volume fraction and filter radius.
    One call to step() is one design iteration of every problem: a single CUDA
    graph launch with device-side PCG and bisection loops (FP32-IR solves with
    reliable updates, warm-started from the previous iteration)."""

    def __init__(self, nelx, nely, load_j, volfrac, rmin, *, E=1.0, nu=0.3, xmin=1e-9, penalty=3.0, rtol=1e-8,
                 maxiter=0):
        self.nprob = len(nelx)
        self.nelx = np.ascontiguousarray(nelx, dtype=np.int32)
        self.nely = np.ascontiguousarray(nely, dtype=np.int32)
        lj = np.ascontiguousarray(load_j, dtype=np.int32)
        vf = np.ascontiguousarray(volfrac, dtype=np.float64)
        rm = np.ascontiguousarray(rmin, dtype=np.float64)
        d = L.ProblemDesc()
        d.dim = 2
        d.size[0] = d.size[1] = 1.0
        d.E, d.nu, d.xmin, d.penalty = float(E), float(nu), float(xmin), float(penalty)
        h = L.C.c_void_p()
        L.check(L.lib().tog_batch_create(self.nprob, L.iptr(self.nelx), L.iptr(self.nely), L.iptr(lj), L.dptr(vf),
                                         L.dptr(rm), L.C.byref(d), float(rtol), int(maxiter), L.C.byref(h)))
        self.handle = h

    def close(self):
        if getattr(self, "handle", None):
            L.lib().tog_batch_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def autotune(self):
        ly = L.C.c_int32()
        L.check(L.lib().tog_batch_autotune(self.handle, L.C.byref(ly)))
        return ly.value

    def set_tile_rows(self, rows):
        """Pin the operator's band height (8, 16, 32 or 64 node rows per work item)."""
        L.check(L.lib().tog_batch_set_tile_rows(self.handle, int(rows)))

    def set_stream(self, stream_ptr):
        L.check(L.lib().tog_batch_set_stream(self.handle, L.C.c_void_p(stream_ptr)))

    def step(self):
        st = L.BatchStats()
        L.check(L.lib().tog_batch_step(self.handle, L.C.byref(st)))
        return st

    def results(self):
        c = np.empty(self.nprob)
        ch = np.empty(self.nprob)
        it = np.empty(self.nprob, dtype=np.int32)
        L.check(L.lib().tog_batch_results(self.handle, L.dptr(c), L.dptr(ch), L.iptr(it)))
        return c, ch, it

    def solve_info(self):
        """Per problem: final FP64 residual norm, reliable updates, status code."""
        res = np.empty(self.nprob)
        ref = np.empty(self.nprob, dtype=np.int32)
        stt = np.empty(self.nprob, dtype=np.int32)
        L.check(L.lib().tog_batch_solve_info(self.handle, L.dptr(res), L.iptr(ref), L.iptr(stt)))
        return res, ref, stt

    def design(self, p):
        x = np.empty(int(self.nelx[p]) * int(self.nely[p]))
        L.check(L.lib().tog_batch_get_design(self.handle, int(p), L.dptr(x)))
        return x

    def bench_kernel(self, kernel, nlaunch=20):
        """Mean microseconds per launch of one PCG-loop kernel over all problems
        (0 operator, 1 update, 2 FP64 residual, 3 operator + update) and its
        algorithmic bytes.  Changes only solver scratch."""
        us, by = L.C.c_double(), L.C.c_double()
        L.check(L.lib().tog_batch_bench_kernel(self.handle, int(kernel), int(nlaunch), L.C.byref(us)))
        L.check(L.lib().tog_batch_kernel_bytes(self.handle, int(kernel), L.C.byref(by)))
        return us.value, by.value


# --------------------------------------------------------------------------- learned warm start
class WarmStartNet:
    """The learned warm-start network of libtopopt_gb300 (tog_nn_*): a 3D
    convolutional encoder-decoder on a structured node grid, trained and run by
    the library's tensor-core kernels.  Tensors are CUDA float32 torch tensors,
    channels-last: inputs (batch, nz, ny, nx, 8), outputs / targets (batch, nz,
    ny, nx, 3)."""

    def __init__(self, nodes, batch=1, seed=0):
        self.nodes = tuple(int(n) for n in nodes)
        self.batch = int(batch)
        h = L.C.c_void_p()
        nn = (L.C.c_int32 * 3)(*self.nodes)
        L.check(L.lib().tog_nn_create(nn, self.batch, int(seed), L.C.byref(h)))
        self.handle = h
        c = L.C.c_int64()
        L.check(L.lib().tog_nn_param_count(h, L.C.byref(c)))
        self.n_params = c.value

    def close(self):
        if getattr(self, "handle", None):
            L.lib().tog_nn_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_stream(self, stream_ptr):
        L.check(L.lib().tog_nn_set_stream(self.handle, L.C.c_void_p(stream_ptr)))

    def get_params(self):
        p = np.empty(self.n_params, dtype=np.float32)
        L.check(L.lib().tog_nn_get_params(self.handle, p.ctypes.data_as(L.C.POINTER(L.C.c_float))))
        return p

    def set_params(self, p):
        p = np.ascontiguousarray(p, dtype=np.float32)
        assert p.size == self.n_params
        L.check(L.lib().tog_nn_set_params(self.handle, p.ctypes.data_as(L.C.POINTER(L.C.c_float))))

    def _shape(self, t, c):
        nx, ny, nz = self.nodes
        if tuple(t.shape) != (self.batch, nz, ny, nx, c) or not t.is_cuda or not t.is_contiguous():
            raise ValueError("expected a contiguous CUDA tensor of shape %s" % ((self.batch, nz, ny, nx, c),))

    def forward(self, inp, out=None):
        import torch
        self._shape(inp, 8)
        if out is None:
            out = torch.empty(inp.shape[:-1] + (3,), dtype=torch.float32, device=inp.device)
        L.check(L.lib().tog_nn_forward(self.handle, L.C.c_void_p(inp.data_ptr()), L.C.c_void_p(out.data_ptr())))
        return out

    def gradients(self, inp, target):
        self._shape(inp, 8)
        self._shape(target, 3)
        g = np.empty(self.n_params, dtype=np.float32)
        loss = L.C.c_double()
        L.check(L.lib().tog_nn_gradients(self.handle, L.C.c_void_p(inp.data_ptr()), L.C.c_void_p(target.data_ptr()),
                                         L.C.byref(loss), g.ctypes.data_as(L.C.POINTER(L.C.c_float))))
        return loss.value, g

    def train_step(self, inp, target, lr=1e-3):
        loss = L.C.c_double()
        L.check(L.lib().tog_nn_train_step(self.handle, L.C.c_void_p(inp.data_ptr()), L.C.c_void_p(target.data_ptr()),
                                          float(lr), L.C.byref(loss)))
        return loss.value
