"""Learned warm-start network: the GPU forward pass and the gradients of the
GPU backward pass (tensor-core BF16 kernels, FP32 accumulation) against the
torch-CPU float64 oracle, on a small grid with a batch of two.  The oracle sees
the same BF16-rounded weights and inputs; the remaining differences are the
BF16 roundings of the activations and gradients, hence normwise tolerances."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def setup_case(tg, nodes=(9, 7, 5), batch=2, seed=1):
    import torch
    import nn_oracle as NO
    rng = np.random.default_rng(seed)
    nx, ny, nz = nodes
    inp = rng.standard_normal((batch, nz, ny, nx, 8)).astype(np.float32)
    tgt = (0.3 * rng.standard_normal((batch, nz, ny, nx, 3))).astype(np.float32)
    net = tg.WarmStartNet(nodes, batch=batch, seed=seed)
    p = net.get_params()
    assert p.size == NO.n_params()
    return net, NO, inp, tgt, p, torch.as_tensor(inp).cuda(), torch.as_tensor(tgt).cuda()


def test_forward_matches_oracle(tg):
    net, NO, inp, tgt, p, ti, tt = setup_case(tg)
    y = net.forward(ti).cpu().numpy()
    layers = NO.unpack(NO.bf16_round(p))
    ref = NO.forward(layers, NO.bf16_round(inp)).detach().numpy()
    err = np.linalg.norm(y - ref) / np.linalg.norm(ref)
    assert err < 3e-2, err


def test_gradients_match_oracle(tg):
    net, NO, inp, tgt, p, ti, tt = setup_case(tg)
    loss, g = net.gradients(ti, tt)
    lref, gref = NO.loss_and_grads(NO.bf16_round(p), NO.bf16_round(inp), tgt)
    assert abs(loss - lref) / lref < 2e-2
    off = 0
    for ci, co, _ in NO.LAYERS:
        for n in (27 * ci * co, co):
            a, b = g[off:off + n], gref[off:off + n]
            off += n
            nb = np.linalg.norm(b)
            if nb == 0:
                assert np.linalg.norm(a) < 1e-6
                continue
            rel = np.linalg.norm(a - b) / nb
            cos = float(np.dot(a, b) / (np.linalg.norm(a) * nb))
            assert rel < 5e-2 and cos > 0.998, (ci, co, n, rel, cos)


def test_training_reduces_loss(tg):
    net, NO, inp, tgt, p, ti, tt = setup_case(tg, nodes=(17, 9, 9), batch=1, seed=2)
    l0 = net.train_step(ti, tt, lr=3e-3)
    for _ in range(150):
        l = net.train_step(ti, tt, lr=3e-3)
    assert l < 0.5 * l0, (l0, l)
