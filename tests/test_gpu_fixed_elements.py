"""FixedElementProjectorFun (src/Functions/fixed_element.jl:13-159) on the device, through
the C ABI: projection and pullback bit-exact against the oracle, the reference's error
cases, and the SIMP loop with an active-element mask checked every design iteration
against the oracle (compliance 1e-6, densities 1e-5 relative; fixed cells exact)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def rel(a, b):
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


def _masks(n, black, white):
    b = np.zeros(n, bool)
    w = np.zeros(n, bool)
    b[list(black)] = True
    w[list(white)] = True
    return b, w


@pytest.mark.parametrize("nels,kind", [((10, 6), "cant"), ((2, 2), "cant"), ((1, 1), "mbb"), ((7, 4, 6), "cant")])
def test_projection_and_pullback_match_oracle(tg, O, nels, kind):
    cls = tg.HalfMBB if kind == "mbb" else tg.PointLoadCantilever
    p = cls(nels, (1.0,) * len(nels))
    s = tg.FEASolver(tg.GB300Solver, p)
    n = p.ncells
    rng = np.random.default_rng(n)
    layouts = [((), ()), (range(0, n), ()), ((), range(0, n))]
    if n >= 4:
        layouts += [(range(0, n // 4), range(n - n // 4, n))]
        sel = rng.permutation(n)
        layouts += [(sel[: n // 3], sel[n // 3: n // 2])]
    for black, white in layouts:
        b, w = _masks(n, black, white)
        g = tg.FixedElementProjectorFun(n, b, w).attach(s)
        ref = O.FixedElementProjector(n, b, w)
        x = rng.uniform(0.0, 1.0, ref.nfree)
        assert np.array_equal(g(x), ref(x))
        d = rng.standard_normal(n)
        assert np.array_equal(g.pullback(d), ref.pullback(d))
        with pytest.raises(ValueError):
            g(np.zeros(ref.nfree + 1))
    s.close()


def test_projection_rejects_bad_state(tg):
    import ctypes
    p = tg.PointLoadCantilever((4, 2), (1.0, 1.0))
    s = tg.FEASolver(tg.GB300Solver, p)
    st = np.zeros(8, np.uint8)
    st[3] = 3
    assert tg.lib().tog_set_fixed_elements(s.handle, st.ctypes.data_as(ctypes.c_void_p)) == tg._lib.TOG_ERR_ARG
    s.close()


def test_oc_with_fixed_cells_matches_oracle(tg, O):
    p = tg.HalfMBB((30, 10), (1.0, 1.0))
    s = tg.FEASolver(tg.GB300Solver, p)
    n = p.ncells
    rng = np.random.default_rng(9)
    g = tg.get_fixed_element_projector(s, range(0, 30), range(n - 30, n))
    ref = O.FixedElementProjector.from_cells(n, range(0, 30), range(n - 30, n))
    x = ref(rng.uniform(0.05, 0.95, ref.nfree))
    dc = -rng.uniform(0.0, 2.0, n)
    w = np.full(n, 1.0 / n)
    xn, ch, lam = tg.oc_update(s, x, dc, w, w, 0.4, 0.2)
    xr, chr_, lamr, _ = O.oc_update(x, dc, w, w, 0.4, 0.2, fixed=ref)
    assert lam == lamr
    assert rel(xn, xr) < 1e-14 and abs(ch - chr_) < 1e-14
    assert np.all(xn[ref.black] == 1.0) and np.all(xn[ref.white] == 0.0)
    g.detach()
    xn2, _, _ = tg.oc_update(s, x, dc, w, w, 0.4, 0.2)
    xr2, _, _, _ = O.oc_update(x, dc, w, w, 0.4, 0.2)
    assert rel(xn2, xr2) < 1e-14
    s.close()


@pytest.mark.parametrize("precision", ["fp64", "fp32_ir"])
def test_simp_loop_with_fixed_regions(tg, O, precision):
    """The layout of docs/tutorials/fixed_elements.qmd on a 40x20 cantilever: a solid
    support column, a solid load column and a void keep-out block, V = 0.4, density
    filter rmin 2, 30 design iterations, each against the oracle's direct solve."""
    nels, volfrac, rmin, xmin, pen = (40, 20), 0.4, 2.0, 1e-3, 3.0
    nx, ny = nels
    p = tg.PointLoadCantilever(nels, (1.0, 1.0))
    op = O.point_load_cantilever(nels, (1.0, 1.0))
    n = p.ncells
    black = [r * nx + c for r in range(ny) for c in (0, nx - 1)]
    white = [r * nx + c for r in range(12, ny) for c in range(29, nx - 1)]
    s = tg.FEASolver(tg.GB300Solver, p, xmin=xmin, penalty=tg.PowerPenaltyFun(pen), rtol=1e-10, abstol=0.0,
                     cg_max_iter=200000, precision=precision)
    g = tg.get_fixed_element_projector(s, black, white)
    ref = O.FixedElementProjector.from_cells(n, black, white)
    x0 = g(np.full(tg.get_free_variable_count(g), volfrac))
    loop = tg.SIMPLoop(s, volfrac=volfrac, rmin=rmin, filter="density", x0=x0)
    st = O.fea_setup(op, xmin=xmin, p=pen)
    filt = O.DensityFilter(op, rmin)
    x = ref(np.full(ref.nfree, volfrac))
    for it in range(30):
        gst = loop.step()
        r = O.simp_iteration(st, x, filt, volfrac, fixed=ref)
        assert abs(gst.compliance - r["c"]) / r["c"] < 1e-6, it
        assert rel(loop.physical, r["xf"]) < 1e-5, it
        xg = loop.x
        assert rel(xg, r["x_new"]) < 1e-5, it
        assert np.all(xg[ref.black] == 1.0) and np.all(xg[ref.white] == 0.0), it
        x = xg
    s.close()
