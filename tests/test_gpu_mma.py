"""MMA (the method of moving asymptotes, the optimizer of the reference's SIMP scripts)
on the device, through the C ABI, against the oracle restatement: every step's design
at 1e-9 relative (the dual bisection is the same sequence up to rounding of the dual
gradient's sum), the analytic optimum of a separable problem, and the device SIMP loop
with MMA against the oracle loop (compliance 1e-6, densities 1e-5 every iteration)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def rel(a, b):
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


def test_mma_steps_match_oracle(tg, O):
    p = tg.HalfMBB((30, 10), (1.0, 1.0))
    s = tg.FEASolver(tg.GB300Solver, p)
    n = p.ncells
    rng = np.random.default_rng(11)
    c = rng.uniform(0.5, 1.5, n)
    V = 0.35
    ref = O.MMA(n)
    x = np.full(n, 0.5)
    dg = np.full(n, 1.0 / n)
    for k in range(12):   # past the first two iterations, so the asymptotes adapt
        df0 = -c / x ** 2
        g = float(np.mean(x)) - V
        xn, ch, lam = tg.mma_update(s, x, df0, g, dg)
        xr, chr_, lamr, _ = ref.update(x, df0, g, dg)
        assert rel(xn, xr) < 1e-9, k
        assert abs(lam - lamr) <= 1e-9 * max(lamr, 1e-300), k
        assert abs(ch - chr_) < 1e-9, k
        x = xr
    xs = V * n * np.sqrt(c) / np.sum(np.sqrt(c))
    for _ in range(40):
        x, _, _ = tg.mma_update(s, x, -c / x ** 2, float(np.mean(x)) - V, dg)
    assert np.max(np.abs(x - xs)) < 1e-6
    tg.mma_reset(s)
    with pytest.raises(tg.TopOptError):
        tg.mma_update(s, x, -c, float("nan"), dg)
    s.close()


def test_mma_holds_fixed_cells(tg, O):
    p = tg.HalfMBB((20, 10), (1.0, 1.0))
    s = tg.FEASolver(tg.GB300Solver, p)
    n = p.ncells
    g = tg.get_fixed_element_projector(s, range(0, 20), range(n - 20, n))
    ref = O.FixedElementProjector.from_cells(n, range(0, 20), range(n - 20, n))
    m = O.MMA(n, fixed=ref)
    rng = np.random.default_rng(2)
    x = ref(rng.uniform(0.2, 0.8, ref.nfree))
    dg = np.full(n, 1.0 / n)
    for k in range(4):
        df0 = -rng.uniform(0.1, 1.0, n)
        xn, _, _ = tg.mma_update(s, x, df0, float(np.mean(x)) - 0.4, dg)
        xr, _, _, _ = m.update(x, df0, float(np.mean(x)) - 0.4, dg)
        assert rel(xn, xr) < 1e-9, k
        assert np.all(xn[ref.black] == 1.0) and np.all(xn[ref.white] == 0.0)
        x = xr
    s.close()


@pytest.mark.parametrize("precision", ["fp64", "fp32_ir"])
def test_simp_loop_with_mma(tg, O, precision):
    """The SIMP loop of docs/tutorials/simp.qmd (compliance, density filter, volume
    constraint through MMA) on a 40x20 cantilever, p = 3, V = 0.4, rmin 2: 25 device
    iterations, each against the oracle's direct-solve iteration from the same design."""
    nels, V, rmin, xmin, pen = (40, 20), 0.4, 2.0, 1e-3, 3.0
    p = tg.PointLoadCantilever(nels, (1.0, 1.0))
    op = O.point_load_cantilever(nels, (1.0, 1.0))
    s = tg.FEASolver(tg.GB300Solver, p, xmin=xmin, penalty=tg.PowerPenaltyFun(pen), rtol=1e-10, abstol=0.0,
                     cg_max_iter=200000, precision=precision)
    loop = tg.SIMPLoop(s, volfrac=V, rmin=rmin, filter="density", optimizer="mma")
    st = O.fea_setup(op, xmin=xmin, p=pen)
    filt = O.DensityFilter(op, rmin)
    m = O.MMA(p.ncells)
    x = np.full(p.ncells, V)
    c0 = None
    for it in range(25):
        gst = loop.step()
        r = O.simp_iteration_mma(st, x, filt, V, m)
        assert abs(gst.compliance - r["c"]) / r["c"] < 1e-6, it
        assert rel(loop.physical, r["xf"]) < 1e-5, it
        xg = loop.x
        assert rel(xg, r["x_new"]) < 1e-5, it
        x = xg
        c0 = c0 or r["c"]
    assert r["c"] < 0.7 * c0                        # the design improved
    assert abs(gst.volume - V) < 0.02               # and meets the volume constraint
    s.close()
