"""The oracle pinned to the reference's own golden vectors and known answers
(CPU only).  Sources: tests/golden/*.json, extracted from the TopOpt.jl test
files by tests/golden/make_golden.py."""
import json
import os

import numpy as np
import pytest

GOLD = os.path.join(os.path.dirname(__file__), "golden")


def load(name):
    return json.load(open(os.path.join(GOLD, name)))


def test_halfmbb_2x2_metadata_fixture(O):
    """test/topopt_problems/metadata.jl:53-132."""
    g = load("metadata_2x2.json")
    p = O.half_mbb((2, 2), (1.0, 1.0))
    assert p.grid.coords.tolist() == g["coords"]
    assert (p.grid.cells + 1).tolist() == g["cells"]
    assert (p.node_dofs + 1).tolist() == g["node_dofs"]
    assert (p.cell_dofs + 1).tolist() == g["cell_dofs"]
    nc = O.node_cells(p.grid)
    for k, v in g["node_cells"].items():
        assert [[c + 1, l + 1] for c, l in nc[int(k) - 1]] == v
    dc = O.dof_cells(p.cell_dofs, p.ndofs)
    for d, lst in enumerate(dc):
        for c, l in lst:
            assert p.cell_dofs[l, c] == d


def test_cantilever_force_dof(O):
    """test/topopt_problems/problems.jl:13-20."""
    pin = load("reference_pins.json")["cantilever_force_dof"]
    p = O.point_load_cantilever(tuple(pin["nels"]), (1.0, 1.0))
    assert p.force_dof + 1 == pin["force_dof_1based"]


def test_element_stiffness_properties(O):
    for dim, sizes in [(2, (1.0, 1.0)), (3, (1.0, 1.0, 1.0)), (3, (1.0, 2.0, 0.5))]:
        Ke = O.element_stiffness(dim, sizes, 1.0, 0.3)
        assert np.allclose(Ke, Ke.T, atol=1e-15)
        ev = np.linalg.eigvalsh(Ke)
        nrigid = 3 if dim == 2 else 6
        assert np.all(np.abs(ev[:nrigid]) < 1e-12) and np.all(ev[nrigid:] > 1e-6)
    # plane strain = the 3D Lame constants (matrices_and_vectors.jl:83-84)
    lam, mu = O._lame(1.0, 0.3, False)
    assert lam == pytest.approx(1.0 * 0.3 / (1.3 * 0.4))
    assert mu == pytest.approx(1.0 / 2.6)


@pytest.mark.parametrize("pen", [1.0, 2.0, 3.0])
def test_compliance_gradient_fd(O, pen):
    """test/Functions/test_common_fns.jl:32-49: 2x2 HalfMBB, xmin 0.01, gradient vs
    5-point central differences within 1e-5."""
    pin = load("reference_pins.json")["compliance_fd"]
    p = O.half_mbb(tuple(pin["nels"]), (1.0, 1.0))
    st = O.fea_setup(p, xmin=pin["xmin"], p=pen)
    rng = np.random.default_rng(0)

    def f(x):
        st.vars = x
        return O.compliance(st, O.direct_solve(st), x)[0]

    for _ in range(3):
        x = np.clip(rng.random(p.grid.ncells), 0.1, 1.0)
        st.vars = x
        _, g, _ = O.compliance(st, O.direct_solve(st), x)
        h = 1e-3
        fd = np.zeros_like(x)
        for i in range(len(x)):
            e = np.zeros_like(x)
            e[i] = h
            fd[i] = (-f(x + 2 * e) + 8 * f(x + e) - 8 * f(x - e) + f(x - 2 * e)) / (12 * h)
        assert np.linalg.norm(g - fd) <= pin["tol"]


def test_matvec_equals_assembled_K(O):
    for p in [O.half_mbb((5, 3), (1.0, 1.0)), O.point_load_cantilever((4, 2, 2), (1.0, 1.0, 1.0))]:
        st = O.fea_setup(p, xmin=1e-3, p=3.0)
        rng = np.random.default_rng(1)
        st.vars = rng.random(p.grid.ncells)
        x = rng.standard_normal(p.ndofs)
        x[~st.free_mask] = 0
        K = O.assemble(st)
        assert np.allclose(O.matvec(st, x), K @ x, rtol=0, atol=1e-13)


def test_solver_agreement_pcg_vs_direct(O):
    """test/FEA/solvers.jl:32-59 (matrix-free CG vs direct, rtol 1e-4, abstol 1e-7)
    and test/FEA/test_preconditioner.jl:147-172 (Jacobi PCG vs direct, rtol 1e-6)."""
    pin = load("reference_pins.json")["solver_agreement"]
    nels = tuple(pin["nels"])
    p = O.point_load_cantilever(nels, (1.0, 1.0, 1.0), force=pin["force"])
    st = O.fea_setup(p)
    st.vars = np.full(p.grid.ncells, pin["x"])
    ud = O.direct_solve(st)
    u, it, _ = O.pcg(st, abstol=pin["abstol"], precond=False)
    assert np.linalg.norm(u - ud) <= pin["rtol"] * np.linalg.norm(ud)
    u, it, _ = O.pcg(st, rtol=1e-12, abstol=1e-9, maxiter=5000)
    assert np.linalg.norm(u - ud) <= 1e-6 * np.linalg.norm(ud)


def test_filter_identities(O):
    """test/CheqFilters/test_filters.jl: uniform density preserved (:126-141),
    pullback = J' (:160-198), sens filter identity forward (:200-244),
    too-small rmin throws (:71-73)."""
    p = O.half_mbb((5, 5), (1.0, 1.0))
    df = O.DensityFilter(p, 2.0)
    n = p.grid.ncells
    assert np.allclose(df.forward(np.full(n, 0.5)), 0.5, rtol=1e-12)
    rng = np.random.default_rng(2)
    x, d = rng.random(n), rng.random(n)
    assert np.isclose(d @ df.forward(x), df.pullback(d) @ x, rtol=1e-12)
    sf = O.SensFilter(p, 2.0)
    assert np.array_equal(sf.forward(x), x)
    g = np.full(n, -0.3)
    assert np.allclose(sf.pullback(g), -0.3, rtol=1e-12)
    with pytest.raises(ValueError):
        O.DensityFilter(p, load("reference_pins.json")["filter_too_small_rmin"]["rmin"])


def test_filter_duplicate_node_weights(O):
    """Each node within rmin is pushed once per traversed cell holding it
    (CheqFilters.jl:96-101): its total weight is (rmin - d) * valence."""
    p = O.half_mbb((6, 6), (1.0, 1.0))
    nodes, ws = O.neighbour_info(p, 2.0)
    ncl = O.node_cells(p.grid)
    for i in range(p.grid.ncells):
        agg = {}
        for n, w in zip(nodes[i], ws[i]):
            agg[n] = agg.get(n, 0.0) + w
        centre = p.grid.coords[p.grid.cells[i]].mean(axis=0)
        for n, w in agg.items():
            d = np.linalg.norm(p.grid.coords[n] - centre)
            assert np.isclose(w, (2.0 - d) * len(ncl[n]), rtol=1e-14)


def test_oc_update_volume_and_bounds(O):
    rng = np.random.default_rng(3)
    n = 500
    x = rng.uniform(0.05, 0.95, n)
    dc = -rng.uniform(0.0, 1.0, n)
    w = np.full(n, 1.0 / n)
    xn, ch, lam, steps = O.oc_update(x, dc, w, w, 0.4, 0.2)
    assert np.all(xn >= np.maximum(0, x - 0.2) - 1e-15) and np.all(xn <= np.minimum(1, x + 0.2) + 1e-15)
    assert abs(w @ xn - 0.4) < 5e-3
    assert ch == pytest.approx(np.max(np.abs(xn - x)))
    assert steps > 10


def test_oracle_projections_and_projected_filter_gradient(O):
    """Heaviside / sigmoid projections and the projected density filter of the oracle:
    derivatives and the chain-rule pullback against central finite differences."""
    x = np.linspace(0.0, 1.0, 11)
    for proj in (O.heaviside_projection, O.sigmoid_projection):
        for beta in (1.0, 8.0):
            y, dy = proj(x, beta)
            fd = (proj(x + 1e-6, beta)[0] - proj(x - 1e-6, beta)[0]) / 2e-6
            assert np.max(np.abs(fd - dy)) < 1e-6 * max(1.0, np.max(np.abs(dy)))
    op = O.half_mbb((6, 4), (1.0, 1.0))
    filt = O.DensityFilter(op, 1.6)
    pf = O.ProjectedDensityFilter(filt, pre=(O.sigmoid_projection, 2.0), post=(O.heaviside_projection, 5.0))
    rng = np.random.default_rng(0)
    x0 = rng.uniform(0.1, 0.9, 24)
    w = rng.standard_normal(24)
    pf.forward(x0)
    g = pf.pullback(w)
    for i in range(0, 24, 5):
        e = np.zeros(24)
        e[i] = 1e-6
        fd = (w @ pf.forward(x0 + e) - w @ pf.forward(x0 - e)) / 2e-6
        assert abs(fd - g[i]) < 1e-6 * max(1.0, abs(g[i]))


# ---------------------------------------------------------------- FixedElementProjectorFun
def _mask(n, idx):
    m = np.zeros(n, dtype=bool)
    m[list(idx)] = True
    return m


def test_fixed_element_projector_pins(O):
    """The known answers of test/Functions/test_fixed_element.jl:22-236 (0-based cells)."""
    black, white = _mask(10, range(0, 3)), _mask(10, range(7, 10))
    p = O.FixedElementProjector(10, black, white)
    assert p.nfree == 4
    assert p.free.tolist() == [False, False, False, True, True, True, True, False, False, False]
    with pytest.raises(ValueError):   # element 3 both black and white
        O.FixedElementProjector(5, _mask(5, range(0, 3)), _mask(5, range(2, 5)))
    with pytest.raises(ValueError):   # mismatched lengths
        O.FixedElementProjector(5, np.zeros(5, bool), np.zeros(6, bool))
    rho = p(np.array([0.0, 0.25, 0.5, 0.75]))
    assert rho.tolist() == [1.0, 1.0, 1.0, 0.0, 0.25, 0.5, 0.75, 0.0, 0.0, 0.0]
    for bad in (np.zeros(2), np.zeros(5)):
        with pytest.raises(ValueError):
            p(bad)
    # sum(p(x)) has gradient ones; sum(abs2, p(x)) has gradient 2 x (finite differences)
    x = np.array([0.1, 0.2, 0.3, 0.4])
    assert np.allclose(p.pullback(np.ones(10)), np.ones(4), rtol=1e-10)
    h = 1e-6
    fd = [(np.sum(p(x + h * np.eye(4)[i]) ** 2) - np.sum(p(x) ** 2)) / h for i in range(4)]
    assert np.allclose(p.pullback(2 * p(x)), fd, rtol=1e-5)
    # the pullback keeps only the free cells (free: element 3 of 5)
    q = O.FixedElementProjector(5, _mask(5, range(0, 2)), _mask(5, range(3, 5)))
    assert q.pullback(np.ones(5)).tolist() == [1.0]
    # identity without fixed cells
    x5 = np.array([0.0, 0.25, 0.5, 0.75, 1.0])
    assert O.FixedElementProjector(5, np.zeros(5, bool), np.zeros(5, bool))(x5).tolist() == x5.tolist()
    # edge cases: all black, all white, none fixed, one element
    assert O.FixedElementProjector(5, np.ones(5, bool), np.zeros(5, bool))(np.zeros(0)).tolist() == [1.0] * 5
    assert O.FixedElementProjector(5, np.zeros(5, bool), np.ones(5, bool))(np.zeros(0)).tolist() == [0.0] * 5
    assert O.FixedElementProjector(1, np.zeros(1, bool), np.zeros(1, bool))(np.array([0.5])).tolist() == [0.5]
    # get_fixed_element_projector by nel
    assert O.FixedElementProjector.from_cells(100, [], []).nfree == 100
    g = O.FixedElementProjector.from_cells(100, range(0, 10), range(90, 100))
    assert (g.nfree, int(g.black.sum()), int(g.white.sum())) == (80, 10, 10)


def test_oc_holds_fixed_cells(O):
    """OC with an active-element mask: fixed cells keep 1 / 0 exactly, the volume of the
    black cells counts against volfrac, and free cells follow the unmasked rule with the
    new multiplier."""
    rng = np.random.default_rng(2)
    n = 200
    fx = O.FixedElementProjector.from_cells(n, range(0, 20), range(180, 200))
    x = fx(rng.uniform(0.1, 0.9, fx.nfree))
    dc = -rng.uniform(0.1, 2.0, n)
    w = np.full(n, 1.0 / n)
    xn, ch, lam, _ = O.oc_update(x, dc, w, w, 0.4, 0.2, fixed=fx)
    assert np.all(xn[fx.black] == 1.0) and np.all(xn[fx.white] == 0.0)
    assert abs(float(w @ xn) - 0.4) < 2e-3
    B = x * np.sqrt(-dc / w)
    free = np.clip(B / np.sqrt(lam), np.maximum(0, x - 0.2), np.minimum(1, x + 0.2))
    assert np.array_equal(xn[fx.free], free[fx.free])


# ---------------------------------------------------------------- MMA (Nonconvex MMA87's method)
def test_mma_reaches_the_analytic_optimum(O):
    """MMA on min sum(c_j / x_j) s.t. mean(x) <= V over [0, 1]^n, whose optimum is
    x_j = V n sqrt(c_j) / sum(sqrt(c)) (inside the bounds here): the restated method
    converges to it, and an inactive constraint gives lambda = 0."""
    rng = np.random.default_rng(3)
    n, V = 50, 0.4
    c = rng.uniform(0.5, 1.5, n)
    xs = V * n * np.sqrt(c) / np.sum(np.sqrt(c))
    assert xs.max() < 1.0
    m = O.MMA(n)
    x = np.full(n, V)
    for _ in range(60):
        x, ch, lam, _ = m.update(x, -c / x ** 2, float(np.mean(x)) - V, np.full(n, 1.0 / n))
    assert np.max(np.abs(x - xs)) < 1e-6
    assert lam > 0
    # an objective that lowers x leaves the constraint inactive: lambda = 0 after one
    # dual evaluation, and x moves down to its lower bound max(L + 0.1 (x - L), x - move, 0)
    m2 = O.MMA(n)
    x2, _, lam2, steps = m2.update(np.full(n, 0.5), c, 0.5 - 0.9, np.full(n, 1.0 / n))
    assert lam2 == 0.0 and steps == 1
    assert np.all(x2 < 0.5)


# ---------------------------------------------------------------- MultiLoad / MeanComplianceFun
def test_mean_compliance_svd_equals_exact_and_fd(O):
    """The SVD form of the mean compliance equals the column mean (tr(F' K^-1 F) / n is
    invariant under F -> U S), and the gradient matches finite differences."""
    prob = O.point_load_cantilever((8, 4), (1.0, 1.0))
    st = O.fea_setup(prob, xmin=1e-3, p=3.0)
    rng = np.random.default_rng(5)
    F = np.zeros((prob.ndofs, 5))
    dofs = rng.choice(np.arange(prob.ndofs), 3, replace=False)
    F[dofs, :] = rng.standard_normal((3, 5))
    x = rng.uniform(0.3, 0.9, prob.grid.ncells)
    m1, g1 = O.mean_compliance(st, F, x, "exact")
    m2, g2 = O.mean_compliance(st, F, x, "exact_svd")
    assert abs(m1 - m2) / m1 < 1e-12
    assert np.max(np.abs(g1 - g2)) / np.max(np.abs(g1)) < 1e-10
    h = 1e-6
    for e in (0, 7, 19):
        xp = x.copy()
        xp[e] += h
        fd = (O.mean_compliance(st, F, xp, "exact")[0] - m1) / h
        assert abs(fd - g1[e]) < 1e-4 * max(1.0, abs(g1[e]))


def test_energy_criteria_stop_rule(O):
    """EnergyCriteria (src/FEA/convergence_criteria.jl:26-45): the oracle's PCG stops once
    the relative change of x'Ax and |x'r| / x'Ax are within tol, with a solution that
    agrees with the direct solve (the reference's solver-agreement bar, 1e-4)."""
    prob = O.point_load_cantilever((12, 6), (1.0, 1.0))
    st = O.fea_setup(prob, xmin=1e-3, p=3.0)
    st.vars = np.random.default_rng(1).uniform(0.3, 1.0, prob.grid.ncells)
    ud = O.direct_solve(st)
    u, its, _ = O.pcg(st, rtol=1e-8, maxiter=10000, conv="energy")
    assert 0 < its < 10000
    assert np.linalg.norm(u - ud) / np.linalg.norm(ud) < 1e-4
    # the residual-norm rule on the same system stops elsewhere, at the same solution
    u2, its2, _ = O.pcg(st, rtol=1e-8, maxiter=10000)
    assert its2 > 0 and np.linalg.norm(u2 - ud) / np.linalg.norm(ud) < 1e-4
