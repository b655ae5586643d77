"""The benchmark configurations themselves against the C oracle (the reference's
matrix-free path restated in C, FP64 Jacobi PCG as cg!: src/FEA/solvers_api.jl:177-220,
253-282; compliance and sensitivities: src/Functions/compliance.jl:58-76; the density
filter: src/CheqFilters/density_filter.jl:25-121), on all host threads.

* 3D PointLoadCantilever 160x80x80 (1,024,000 cells, the headline workload): design
  iteration 1 from the uniform start and design iteration 3 from the design the GPU loop
  reached after iteration 2.  Compliance 1e-6 relative, sensitivities and filtered
  densities 1e-5 relative (max norm), new design 1e-5 absolute; the displacement's
  relative 2-norm error is printed and bounded by 1e-4 (both sides solve to rtol 1e-10,
  the GPU in FP32 inside FP64 refinement).
* The 256-problem batch of uneven 2D cantilevers: 8 problems spread over the size range,
  after design iterations 1, 2 and 3, each iteration checked from the GPU's previous
  design; compliance 1e-6, new design 1e-5.
"""
import ctypes
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

NELS = (160, 80, 80)
VOLFRAC, RMIN, PEN, XMIN, MOVE = 0.3, 1.5, 3.0, 1e-9, 0.2


def _oracle_cpu():
    import oracle_cpu as OC
    return OC


def _relmax(a, b):
    return float(np.max(np.abs(a - b)) / np.max(np.abs(b)))


def _oracle_iteration(cs, f, x, volfrac, rmin_unused=None, rtol=1e-10):
    """One design iteration of the C oracle from design x (filter, PCG, compliance,
    pullback, OC); returns its intermediate results."""
    n = x.size
    xf = cs.filter_J(x)
    cs.set_vars(xf)
    u, it, _ = cs.pcg(f, rtol=rtol, abstol=0.0, maxit=400000)
    c, g = cs.compliance(u)
    dc = cs.filter_JT(g)
    dv = cs.filter_JT(np.full(n, 1.0 / n))
    xn, _, _ = cs.oc(x, dc, dv, dv, volfrac, MOVE)
    return dict(xf=xf, u=u, c=c, g=g, x_new=xn, cg=it)


def _cantilever_2d(O, nelx, nely, load_j):
    """The batch's problem in the oracle: left edge clamped, load [0, -1] at node
    (nelx, load_j); nely may be odd (the reference's PointLoadCantilever needs it even)."""
    g = O.rectilinear_grid((nelx, nely), (1.0, 1.0))
    nd, cd = O.dof_numbering(g)
    left = np.nonzero(np.isclose(g.coords[:, 0], 0.0))[0]
    fixed = np.unique(nd[:, left].ravel())
    node = nelx + (nelx + 1) * load_j
    f = np.zeros(g.nnodes * 2)
    f[nd[1, node]] = -1.0
    return O.Problem(g, 1.0, 0.3, 1.0, nd, cd, fixed, f, int(nd[1, node]), node)


def test_headline_160x80x80_matches_oracle(tg, O):
    OC = _oracle_cpu()
    prob = tg.PointLoadCantilever(NELS, (1.0, 1.0, 1.0), load="face_centre")
    op = O.point_load_cantilever(NELS, (1.0, 1.0, 1.0), load="face_centre")
    assert np.array_equal(prob.fixed_dofs, op.fixed_dofs) and prob.force_dof == op.force_dof
    n = prob.ncells
    rtol = 1e-10
    s = tg.FEASolver(tg.GB300Solver, prob, xmin=XMIN, penalty=tg.PowerPenaltyFun(PEN), rtol=rtol, abstol=0.0,
                     cg_max_iter=400000, precision="fp32_ir", warm_start=True)
    loop = tg.SIMPLoop(s, volfrac=VOLFRAC, rmin=RMIN, filter="density")
    L = tg._lib

    def gpu_step():
        st = loop.step()
        grad = np.empty(n)
        c = ctypes.c_double()
        L.check(L.lib().tog_compliance(s.handle, ctypes.byref(c), L.dptr(grad)))
        return dict(c=st.compliance, c_again=c.value, g=grad, xf=loop.physical, u=s.u, x_new=loop.x)

    g1 = gpu_step()
    g2 = gpu_step()
    x2 = g2["x_new"]
    g3 = gpu_step()
    s.close()

    Ke = O.element_stiffness(3, (1.0, 1.0, 1.0), 1.0, 0.3)
    threads = OC.lib().orc_max_threads()
    cs = OC.CPUSolver(op, Ke, XMIN, PEN, threads=threads)
    cs.filter_setup(RMIN)
    f = op.f.copy()
    f[op.fixed_dofs] = 0.0
    for it, (g, x_prev) in enumerate(((g1, np.full(n, VOLFRAC)), (g3, x2))):
        r = _oracle_iteration(cs, f, x_prev, VOLFRAC, rtol=rtol)
        du = float(np.linalg.norm(g["u"] - r["u"]) / np.linalg.norm(r["u"]))
        print("160x80x80 iteration %d: compliance %.3e, sensitivities %.3e, filtered densities %.3e, "
              "displacement %.3e, new design %.3e (oracle PCG %d iterations, %d threads)"
              % ((1, 3)[it], abs(g["c"] - r["c"]) / r["c"], _relmax(g["g"], r["g"]), _relmax(g["xf"], r["xf"]), du,
                 float(np.max(np.abs(g["x_new"] - r["x_new"]))), r["cg"], threads))
        assert abs(g["c"] - r["c"]) / r["c"] < 1e-6
        assert abs(g["c_again"] - r["c"]) / r["c"] < 1e-6
        assert _relmax(g["g"], r["g"]) < 1e-5
        assert _relmax(g["xf"], r["xf"]) < 1e-5
        assert float(np.max(np.abs(g["x_new"] - r["x_new"]))) < 1e-5
        assert du < 1e-4
    cs.close()


def test_batch_set_of_256_matches_oracle_on_8_problems(tg, O):
    OC = _oracle_cpu()
    P = tg.uneven_cantilever_set(256, seed=0)
    b = tg.BatchedSIMP(P["nelx"], P["nely"], P["load_j"], P["volfrac"], P["rmin"], rtol=1e-10)
    order = np.argsort(P["nelx"], kind="stable")
    pick = [int(order[i]) for i in np.linspace(0, 255, 8).round().astype(int)]
    designs = {p: [np.full(int(P["nelx"][p] * P["nely"][p]), float(P["volfrac"][p]))] for p in pick}
    comps = []
    for _ in range(3):
        st = b.step()
        assert st.failed == 0
        comps.append(b.results()[0].copy())
        for p in pick:
            designs[p].append(b.design(p))
    b.close()
    Ke = O.element_stiffness(2, (1.0, 1.0), 1.0, 0.3)
    threads = OC.lib().orc_max_threads()
    for p in pick:
        nelx, nely = int(P["nelx"][p]), int(P["nely"][p])
        op = _cantilever_2d(O, nelx, nely, int(P["load_j"][p]))
        f = op.f
        cs = OC.CPUSolver(op, Ke, XMIN, PEN, threads=threads)
        cs.filter_setup(float(P["rmin"][p]))
        for k in range(3):
            r = _oracle_iteration(cs, f, designs[p][k], float(P["volfrac"][p]))
            assert abs(comps[k][p] - r["c"]) / r["c"] < 1e-6, (p, k)
            assert float(np.max(np.abs(designs[p][k + 1] - r["x_new"]))) < 1e-5, (p, k)
        cs.close()
