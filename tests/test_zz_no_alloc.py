"""The allocation-free OC entry point, through the C ABI, against the handle-based one.

tog_oc_update_noalloc serves callers that cannot call cudaMalloc (their device
memory is owned by someone else, or their loop must not allocate): it runs the
OC update on device arrays the caller passes and keeps its scratch in a static
device array of the library.  Two calls in a row must both match tog_oc_update
within the OC tolerance of the other GPU tests (1e-14 relative on x_new), the
second one with the scratch still holding the first call's contents.  This file
is collected last so that a run stopping at the first failure has run every
other test first; it also passes alone in a fresh process.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _dptr(t):
    return ctypes.cast(t.data_ptr(), ctypes.POINTER(ctypes.c_double))


def _check_against_handle(tg, nels, volfrac, seed):
    import torch
    L = tg._lib
    prob = tg.HalfMBB(nels, (1.0, 1.0))
    solver = tg.FEASolver(tg.GB300Solver, prob)
    n = prob.ncells
    rng = np.random.default_rng(seed)
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    x = rng.uniform(0.05, 0.95, n)
    dc = -rng.uniform(0.0, 2.0, n)
    dv = np.full(n, 1.0 / n)
    w = dv.copy()
    x_ref, change_ref, lam_ref = tg.oc_update(solver, x, dc, dv, w, volfrac, 0.2)
    solver.close()
    dev = [torch.tensor(a, dtype=torch.float64, device="cuda") for a in (x, dc, dv, w)]
    xnew = torch.empty(n, dtype=torch.float64, device="cuda")
    res = torch.zeros(3, dtype=torch.float64, device="cuda")
    code = L.lib().tog_oc_update_noalloc(n, *[_dptr(t) for t in dev], volfrac, 0.2, _dptr(xnew), _dptr(res), stream)
    assert code == 0, L.lib().tog_last_error()
    torch.cuda.synchronize()
    xg = xnew.cpu().numpy()
    change, lam, vol = res.cpu().numpy()
    assert np.max(np.abs(xg - x_ref)) / np.max(np.abs(x_ref)) < 1e-14, nels
    assert abs(change - change_ref) < 1e-14, nels
    assert abs(lam - lam_ref) <= 1e-12 * lam_ref, nels
    assert abs(vol - float(np.dot(w, xg))) < 1e-12 * max(1.0, abs(vol)), nels


def test_noalloc_oc_matches_handle_entry_point(tg):
    """Two calls in a row on the same grid, the second with the scratch still holding the first."""
    for call, volfrac in enumerate((0.3, 0.5)):
        _check_against_handle(tg, (200, 100), volfrac, 11 + call)


def test_noalloc_oc_sizes_in_sequence(tg):
    """The scratch capacity itself (1,048,576 cells: 1024 blocks, many passes of the
    grid-stride loops, every partial-sum slot), a multi-pass size (300,000 cells), then a
    smaller grid, whose call must not pick up the larger calls' stale partial sums."""
    for nels, volfrac, seed in (((1024, 1024), 0.4, 21), ((600, 500), 0.35, 22), ((30, 10), 0.5, 23)):
        _check_against_handle(tg, nels, volfrac, seed)


def test_noalloc_rejects_sizes_beyond_the_static_scratch(tg):
    import torch
    L = tg._lib
    t = torch.zeros(4, dtype=torch.float64, device="cuda")
    p = _dptr(t)
    code = L.lib().tog_oc_update_noalloc((1 << 20) + 1, p, p, p, p, 0.5, 0.2, p, p, None)
    assert code == L.TOG_ERR_ARG
    assert b"capacity" in L.lib().tog_last_error()
