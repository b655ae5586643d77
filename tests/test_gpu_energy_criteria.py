"""EnergyCriteria (src/FEA/convergence_criteria.jl:26-45) as the FP64 PCG stop rule on the
device, through the C ABI.  Both of its ratios hover near the tolerance over several
iterations (x'r is zero in exact arithmetic and grows with the loss of orthogonality),
so where it stops moves with rounding: perturbing the densities by 1e-15 moves the
oracle's stop over 163..168 (24x12) and 102..110 (8x4x4) iterations.  The bar is
therefore the device's stop inside the spread the oracle itself shows over twelve such
perturbations (two iterations of margin either side), and its solution within the
reference's solver-agreement bar (1e-4, test/FEA/solvers.jl:32-59) of the direct solve;
the residual-norm rule, which does not hover, stays within one iteration of the oracle.
FP32-IR rejects EnergyCriteria."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("nels", [(24, 12), (8, 4, 4)])
def test_energy_criteria_matches_oracle(tg, O, nels):
    sizes = (1.0,) * len(nels)
    p = tg.PointLoadCantilever(nels, sizes)
    op = O.point_load_cantilever(nels, sizes)
    s = tg.FEASolver(tg.GB300Solver, p, xmin=1e-3, penalty=tg.PowerPenaltyFun(3.0), rtol=1e-8, abstol=0.0,
                     cg_max_iter=20000, conv=tg.EnergyCriteria())
    x = np.random.default_rng(3).uniform(0.3, 1.0, p.ncells)
    s.vars = x
    s()
    st = O.fea_setup(op, xmin=1e-3, p=3.0)
    stops = []
    for k in range(12):
        st.vars = x * (1.0 + (0.0 if k == 0 else 1e-15) * np.random.default_rng(k).standard_normal(x.size))
        stops.append(O.pcg(st, rtol=1e-8, maxiter=20000, conv="energy")[1])
    assert min(stops) - 2 <= s.last_stats.iterations <= max(stops) + 2, (s.last_stats.iterations, stops)
    assert s.last_stats.iterations < 20000
    st.vars = x
    u = s.u
    ud = O.direct_solve(st)
    assert np.linalg.norm(u - ud) / np.linalg.norm(ud) < 1e-4
    # the default criterion on the same handle afterwards
    s2 = tg.FEASolver(tg.GB300Solver, p, xmin=1e-3, penalty=tg.PowerPenaltyFun(3.0), rtol=1e-8, abstol=0.0,
                      cg_max_iter=20000)
    s2.vars = x
    s2()
    _, its_d, _ = O.pcg(st, rtol=1e-8, maxiter=20000)
    assert abs(s2.last_stats.iterations - its_d) <= 1
    s.close()
    s2.close()


def test_energy_criteria_rejected_for_fp32_ir(tg):
    p = tg.HalfMBB((8, 4), (1.0, 1.0))
    s = tg.FEASolver(tg.GB300Solver, p, precision="fp32_ir", conv=tg.EnergyCriteria())
    with pytest.raises(tg.TopOptError):
        s()
    s.close()
