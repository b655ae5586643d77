"""The shared-memory filter stencils (topopt.jl_gb300/csrc/tog_filter.cuh) carry nodal sums
instead of the reference's nodal means and drop the valence weights of
CheqFilters.jl:66-118, because in a structured grid the valence of a node equals the number of
cells it averages and both are powers of two: w * valence * (sum / valence) == w * sum and
valence * acc / valence == acc exactly in IEEE double.  This checks that identity on random
values over the whole exponent range the filter meets (densities in [1e-9, 1], weights in
(0, rmin))."""
import numpy as np


def test_valence_scaling_is_exact():
    rng = np.random.default_rng(3)
    n = 200000
    s = rng.uniform(1e-9, 8.0, n) * 10.0 ** rng.uniform(-9, 0, n)   # nodal sums of up to 8 cells
    w = rng.uniform(1e-6, 9.0, n)                                    # stencil weights rmin - d
    acc = rng.standard_normal(n) * 10.0 ** rng.uniform(-12, 3, n)    # transpose accumulators
    for val in (1.0, 2.0, 4.0, 8.0):
        mean = s / val
        assert np.array_equal((w * val) * mean, w * s)
        assert np.array_equal((acc * val) * (1.0 / val), acc)
