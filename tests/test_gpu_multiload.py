"""MultiLoad + MeanComplianceFun / BlockComplianceFun (src/TopOptProblems/multiload.jl,
src/Functions/mean_compliance.jl, block_compliance.jl) on the device, through the C ABI,
against the oracle's direct solves: compliances 1e-6 relative, gradients 1e-5 relative
(solver rtol 1e-10)."""
import itertools

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def rel(a, b):
    return float(np.max(np.abs(np.asarray(a) - np.asarray(b))) / max(np.max(np.abs(b)), 1e-300))


def _cycle(vals):
    it = itertools.cycle(vals)
    return lambda: np.asarray(next(it), dtype=np.float64)


@pytest.mark.parametrize("nels,precision", [((20, 10), "fp64"), ((8, 4, 4), "fp32_ir")])
def test_mean_and_block_compliance_match_oracle(tg, O, nels, precision):
    dim = len(nels)
    sizes = (1.0,) * dim
    p = tg.PointLoadCantilever(nels, sizes)
    op = O.point_load_cantilever(nels, sizes)
    e2 = [0.0] * dim
    down, side = list(e2), list(e2)
    down[1], side[0] = -1.0, 1.0
    rules = [(tuple([nels[0], nels[1] / 2] + ([0.0] if dim == 3 else [])), _cycle([down, [2 * v for v in down]])),
             (tuple([nels[0] / 2, nels[1]] + ([nels[2] / 2] if dim == 3 else [])), _cycle([side, [-0.5 * v for v in side]]))]
    ml = tg.MultiLoad(p, 4, rules)
    s = tg.FEASolver(tg.GB300Solver, p, xmin=1e-3, penalty=tg.PowerPenaltyFun(3.0), rtol=1e-10, abstol=0.0,
                     cg_max_iter=200000, precision=precision)
    st = O.fea_setup(op, xmin=1e-3, p=3.0)
    rng = np.random.default_rng(7)
    x = rng.uniform(0.3, 0.9, p.ncells)
    c_single = tg.ComplianceFun(s)(tg.PseudoDensities(x))
    for method in ("exact", "exact_svd"):
        mc = tg.MeanComplianceFun(ml, s, method=method)
        m = mc(tg.PseudoDensities(x))
        mr, gr = O.mean_compliance(st, ml.F, x, method)
        assert abs(m - mr) / mr < 1e-6, method
        assert rel(mc.pullback(1.0), gr) < 1e-5, method
    # trace estimation with given probes: the columns F v, divided by nv n
    V = tg.hadamard(np.zeros((4, 2)))
    mt = tg.MeanComplianceFun(ml, s, method="trace", V=V)(x)
    ct, _ = O.multiload_compliance(st, ml.F @ V, x)
    assert abs(mt - ct.sum() / 8) / abs(ct.sum() / 8) < 1e-6
    # block compliance and its pullback
    bc = tg.BlockComplianceFun(ml, s)
    c = bc(tg.PseudoDensities(x))
    cr, G = O.multiload_compliance(st, ml.F, x)
    assert rel(c, cr) < 1e-6
    d = rng.standard_normal(4)
    assert rel(bc.pullback(d), G @ d) < 1e-5
    with pytest.raises(ValueError):
        bc.pullback(np.ones(3))
    # the handle's own load is untouched
    assert abs(tg.ComplianceFun(s)(tg.PseudoDensities(x)) - c_single) / c_single < 1e-9
    s.close()


def test_multiload_rejects_bad_columns(tg):
    import ctypes
    p = tg.HalfMBB((6, 2), (1.0, 1.0))
    s = tg.FEASolver(tg.GB300Solver, p)
    L = tg.lib()
    c = np.empty(1)
    colptr = np.array([0, 1], dtype=np.int64)
    rows = np.array([p.ndofs], dtype=np.int32)   # out of range
    vals = np.array([1.0])
    rc = L.tog_multiload_compliance(s.handle, 1, colptr.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)),
                                    rows.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)),
                                    vals.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), 0, 1e-8, 0.0, 1000,
                                    c.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), None)
    assert rc == tg._lib.TOG_ERR_ARG
    w = np.ones(1)
    assert L.tog_multiload_gradient(s.handle, 1, w.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                                    c.ctypes.data_as(ctypes.POINTER(ctypes.c_double))) == tg._lib.TOG_ERR_STATE
    s.close()
