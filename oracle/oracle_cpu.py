"""ctypes wrapper of the C oracle (TEST INFRASTRUCTURE AND CPU BASELINE ONLY).

Runs TopOpt.jl's matrix-free SIMP path on the host cores (see oracle_cpu.c for
the reference file:line each routine follows)."""
import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "_build", "liboracle_cpu.so")
_D = C.POINTER(C.c_double)
_I = C.POINTER(C.c_int32)
_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB):
            import build_oracle
            build_oracle.build()
        L = C.CDLL(LIB)
        L.orc_create.restype = C.c_void_p
        L.orc_create.argtypes = [C.c_int, _I, _I, _D, C.POINTER(C.c_uint8), C.c_double, C.c_double]
        L.orc_destroy.argtypes = [C.c_void_p]
        L.orc_set_threads.argtypes = [C.c_int]
        L.orc_max_threads.restype = C.c_int
        L.orc_set_vars.argtypes = [C.c_void_p, _D]
        L.orc_matvec.argtypes = [C.c_void_p, _D, _D]
        L.orc_pcg.restype = C.c_int
        L.orc_pcg.argtypes = [C.c_void_p, _D, _D, C.c_double, C.c_double, C.c_int, _D]
        L.orc_compliance.restype = C.c_double
        L.orc_compliance.argtypes = [C.c_void_p, _D, _D, _D]
        L.orc_filter_J.argtypes = [C.c_void_p, _I, _D, C.c_int, _D, _D, _D]
        L.orc_filter_JT.argtypes = [C.c_void_p, _I, _D, C.c_int, _D, _D, _D, _D]
        L.orc_oc.restype = C.c_double
        L.orc_oc.argtypes = [C.c_int64, _D, _D, _D, _D, C.c_double, C.c_double, _D, C.POINTER(C.c_double)]
        _lib = L
    return _lib


def _d(a):
    return a.ctypes.data_as(_D)


def _i(a):
    return a.ctypes.data_as(_I)


def stencil(dim, sizes, rmin):
    """Node offsets (from the cell's lower corner) within rmin of the cell centre,
    weight rmin - d (CheqFilters.jl:66-118)."""
    R = [int(np.ceil(rmin / s)) + 1 for s in sizes]
    offs, ws = [], []
    rz = range(-R[2], R[2] + 2) if dim == 3 else [0]
    for dz in rz:
        for dy in range(-R[1], R[1] + 2):
            for dx in range(-R[0], R[0] + 2):
                o = (dx, dy, dz)
                dist = np.sqrt(sum((o[d] * sizes[d] - sizes[d] / 2.0) ** 2 for d in range(dim)))
                if dist < rmin:
                    offs.append(o)
                    ws.append(max(rmin - dist, 0.0))
    return np.asarray(offs, dtype=np.int32).ravel(), np.asarray(ws)


class CPUSolver:
    """The reference's matrix-free path on the host: per-element Ke copies,
    two-phase gather, Jacobi PCG, compliance, filter, OC."""

    def __init__(self, prob, Ke, xmin, p, threads=1):
        self.prob = prob
        g = prob.grid
        self.dim = g.dim
        self.nel = np.array(list(g.nels) + [1] * (3 - g.dim), dtype=np.int32)
        self.cell_dofs = np.ascontiguousarray(prob.cell_dofs.T, dtype=np.int32)
        self.Ke = np.ascontiguousarray(Ke, dtype=np.float64)
        fixed = np.zeros(prob.ndofs, dtype=np.uint8)
        fixed[prob.fixed_dofs] = 1
        self.fixed = fixed
        self.threads = threads
        lib().orc_set_threads(threads)
        self.h = lib().orc_create(g.dim, _i(self.nel), _i(self.cell_dofs), _d(self.Ke),
                                  fixed.ctypes.data_as(C.POINTER(C.c_uint8)), xmin, p)
        self.ncells, self.nnodes = g.ncells, g.nnodes
        self.nodal = np.empty(g.nnodes)
        self.invW = np.empty(g.ncells)

    def close(self):
        if self.h:
            lib().orc_destroy(self.h)
            self.h = None

    def set_vars(self, x):
        self.vars = np.ascontiguousarray(x, dtype=np.float64)
        lib().orc_set_threads(self.threads)
        lib().orc_set_vars(self.h, _d(self.vars))

    def matvec(self, x):
        y = np.empty_like(x)
        lib().orc_matvec(self.h, _d(np.ascontiguousarray(x)), _d(y))
        return y

    def pcg(self, b, rtol, abstol=0.0, maxit=100000):
        x = np.empty(self.prob.ndofs)
        res = C.c_double()
        it = lib().orc_pcg(self.h, _d(np.ascontiguousarray(b)), _d(x), rtol, abstol, maxit, C.byref(res))
        return x, it, res.value

    def compliance(self, u):
        g = np.empty(self.ncells)
        c = lib().orc_compliance(self.h, _d(u), _d(self.vars), _d(g))
        return c, g

    def filter_setup(self, rmin):
        self.soff, self.sw = stencil(self.dim, self.prob.grid.sizes, rmin)
        self.S = len(self.sw)

    def filter_J(self, x):
        y = np.empty(self.ncells)
        lib().orc_filter_J(self.h, _i(self.soff), _d(self.sw), self.S, _d(np.ascontiguousarray(x)), _d(y),
                           _d(self.nodal))
        return y

    def filter_JT(self, d):
        y = np.empty(self.ncells)
        lib().orc_filter_JT(self.h, _i(self.soff), _d(self.sw), self.S, _d(np.ascontiguousarray(d)), _d(y),
                            _d(self.nodal), _d(self.invW))
        return y

    def oc(self, x, dc, dv, w, volfrac, move=0.2):
        xn = np.empty(self.ncells)
        ch = C.c_double()
        lam = lib().orc_oc(self.ncells, _d(x), _d(dc), _d(dv), _d(w), volfrac, move, _d(xn), C.byref(ch))
        return xn, ch.value, lam
