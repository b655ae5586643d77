"""Batched 2D SIMP (many uneven cantilevers in one graph launch per design
iteration) against the single-problem path, problem by problem, through the C ABI.
Tolerances: compliance 1e-6 relative, designs 1e-5 (the SIMP accuracy bar)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def single_run(tg, nelx, nely, volfrac, rmin, steps, rtol):
    p = tg.PointLoadCantilever((nelx, nely), (1.0, 1.0))
    s = tg.FEASolver(tg.GB300Solver, p, xmin=1e-9, penalty=tg.PowerPenaltyFun(3.0), rtol=rtol, abstol=0.0,
                     cg_max_iter=200000, precision="fp32_ir", warm_start=True)
    loop = tg.SIMPLoop(s, volfrac=volfrac, rmin=rmin, filter="density")
    comps = []
    for _ in range(steps):
        comps.append(loop.step().compliance)
    x = loop.x
    s.close()
    return np.array(comps), x


@pytest.mark.parametrize("autotune", [False, True, 8, 16, 64])
def test_batch_matches_single_problems(tg, autotune):
    nelx = [64, 30, 96, 48]
    nely = [32, 16, 20, 48]
    vf = [0.4, 0.5, 0.35, 0.6]
    rm = [1.5, 2.0, 2.7, 3.0]
    lj = [n // 2 for n in nely]
    rtol, steps = 1e-10, 3
    b = tg.BatchedSIMP(nelx, nely, lj, vf, rm, rtol=rtol)
    if autotune is True:
        assert b.autotune() in (8, 16, 32, 64)
    elif autotune:
        b.set_tile_rows(autotune)
    comps = []
    for _ in range(steps):
        st = b.step()
        assert st.failed == 0
        comps.append(b.results()[0].copy())
    comps = np.array(comps)
    for p in range(len(nelx)):
        c_ref, x_ref = single_run(tg, nelx[p], nely[p], vf[p], rm[p], steps, rtol)
        assert np.max(np.abs(comps[:, p] - c_ref) / c_ref) < 1e-6, p
        x = b.design(p)
        assert np.max(np.abs(x - x_ref)) < 1e-5, p
    b.close()


def test_batch_matches_oracle_off_centre_load(tg, O):
    """A load node away from mid-height (the benchmark's set draws it on the whole right edge):
    first design iteration against the oracle's direct solve."""
    nelx, nely, lj, vf, rm = 24, 12, 3, 0.45, 2.2
    b = tg.BatchedSIMP([nelx, 40], [nely, 20], [lj, 20], [vf, 0.5], [rm, 1.5], rtol=1e-10)
    b.step()
    c = b.results()[0][0]
    x = b.design(0)
    op = O.point_load_cantilever((nelx, nely), (1.0, 1.0))
    # move the load to node (nelx, lj)
    f = np.zeros(op.ndofs)
    fnode = nelx + (nelx + 1) * lj
    f[op.node_dofs[1, fnode]] = -1.0
    op.f = f
    st = O.fea_setup(op, xmin=1e-9, p=3.0)
    ref = O.simp_iteration(st, np.full(nelx * nely, vf), O.DensityFilter(op, rm), vf)
    assert abs(c - ref["c"]) / ref["c"] < 1e-6
    assert np.max(np.abs(x - ref["x_new"])) < 1e-5
    b.close()


def test_batch_rejects_bad_problems(tg):
    with pytest.raises(tg.TopOptError):
        tg.BatchedSIMP([10], [5], [9], [0.5], [2.0])       # load node beyond the edge
    with pytest.raises(tg.TopOptError):
        tg.BatchedSIMP([10], [6], [3], [0.5], [0.1])       # rmin below the element size


@pytest.mark.parametrize("rows", [8, 16, 64])
def test_batch_tile_rows_same_results(tg, rows):
    """Every tile height gives the same design iteration on problems that span
    many tiles; compliance agrees to the solve tolerance."""
    P = tg.uneven_cantilever_set(8, seed=3)
    out = []
    for r in (rows, None):
        b = tg.BatchedSIMP(P["nelx"], P["nely"], P["load_j"], P["volfrac"], P["rmin"], rtol=1e-8)
        if r:
            b.set_tile_rows(r)
        st = b.step()
        assert st.failed == 0
        res, nref, status = b.solve_info()
        assert np.all(status == 0) and np.all(res <= 1e-8)
        out.append(b.results()[0])
        b.close()
    assert np.max(np.abs(out[0] - out[1]) / out[1]) < 1e-6
