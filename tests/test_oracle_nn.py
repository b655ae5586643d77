"""The learned warm-start oracle (torch CPU float64) is itself checked against
central finite differences before it is trusted as the gradient checker."""
import numpy as np


def test_oracle_gradient_finite_differences():
    import nn_oracle as NO
    rng = np.random.default_rng(0)
    p = rng.standard_normal(NO.n_params()) * 0.05
    inp = rng.standard_normal((1, 5, 4, 6, 8))
    tgt = rng.standard_normal((1, 5, 4, 6, 3))
    _, g = NO.loss_and_grads(p, inp, tgt)
    sizes = [(27 * ci * co, co) for ci, co, _ in NO.LAYERS]
    picks, off = [], 0
    for nw, nb in sizes:     # one weight and one bias of every layer, where the gradient is nonzero
        w = off + int(np.argmax(np.abs(g[off:off + nw])))
        b = off + nw + int(np.argmax(np.abs(g[off + nw:off + nw + nb])))
        picks += [w, b]
        off += nw + nb
    for idx in picks:
        e = np.zeros_like(p)
        e[idx] = 1e-6
        lp, _ = NO.loss_and_grads(p + e, inp, tgt)
        lm, _ = NO.loss_and_grads(p - e, inp, tgt)
        fd = (lp - lm) / 2e-6
        assert abs(fd - g[idx]) <= 1e-6 + 1e-5 * abs(g[idx]), (idx, fd, g[idx])


def test_oracle_upsampling_is_nearest():
    import torch
    import nn_oracle as NO
    c = torch.arange(2 * 2 * 3, dtype=torch.float64).reshape(1, 1, 2, 2, 3)
    f = NO._up(c, torch.zeros(1, 1, 3, 4, 5))
    assert f.shape == (1, 1, 3, 4, 5)
    assert f[0, 0, 2, 3, 4] == c[0, 0, 1, 1, 2] and f[0, 0, 1, 1, 1] == c[0, 0, 0, 0, 0]
