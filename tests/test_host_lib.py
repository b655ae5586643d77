"""The C-ABI library without a GPU: it loads, exports every symbol declared in
include/topopt_gb300.h, and its host-only entry points (numbering, element
stiffness) match the oracle bit-exactly / to rounding."""
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def header_symbols():
    src = open(os.path.join(ROOT, "include", "topopt_gb300.h")).read()
    return sorted(set(re.findall(r"^\s*(?:const char\*|int64_t|int)\s+(tog_\w+)\s*\(", src, re.M)))


def test_library_exports_every_header_symbol(tg):
    import ctypes
    L = ctypes.CDLL(tg._lib.LIB_PATH)
    syms = header_symbols()
    assert len(syms) >= 25
    for s in syms:
        assert hasattr(L, s), s
    assert set(syms) == set(tg._lib.SIGNATURES)
    assert tg.lib().tog_version().startswith(b"libtopopt_gb300")


@pytest.mark.parametrize("nels", [(2, 2), (5, 3), (60, 20), (160, 40), (2, 2, 2), (3, 2, 2), (5, 4, 3), (20, 10, 10)])
def test_numbering_bit_exact(tg, O, nels):
    """Element-to-dof maps must be bit-exact with the oracle's Ferrite restatement."""
    g = O.rectilinear_grid(nels, (1.0,) * len(nels))
    nd, cd = O.dof_numbering(g)
    assert np.array_equal(tg.node_dofs(nels), nd.T)
    assert np.array_equal(tg.cell_dofs(nels), cd.T)
    nn, nc, ndof = tg.grid_counts(nels)
    assert (nn, nc, ndof) == (g.nnodes, g.ncells, g.nnodes * len(nels))


def test_problem_bcs_match_oracle(tg, O):
    for nels in [(60, 20), (12, 6), (6, 4, 4)]:
        p, op = tg.HalfMBB(nels, (1.0,) * len(nels)), O.half_mbb(nels, (1.0,) * len(nels))
        assert np.array_equal(p.fixed_dofs, op.fixed_dofs) and p.force_dof == op.force_dof
    for nels in [(160, 40), (20, 10, 10), (8, 4, 6)]:
        p, op = tg.PointLoadCantilever(nels, (1.0,) * len(nels)), O.point_load_cantilever(nels, (1.0,) * len(nels))
        assert np.array_equal(p.fixed_dofs, op.fixed_dofs) and p.force_dof == op.force_dof
    p = tg.PointLoadCantilever((8, 4, 6), (1.0, 1.0, 1.0), load="face_centre")
    op = O.point_load_cantilever((8, 4, 6), (1.0, 1.0, 1.0), load="face_centre")
    assert p.force_dof == op.force_dof
    with pytest.raises(ValueError):
        tg.PointLoadCantilever((8, 3), (1.0, 1.0))


@pytest.mark.parametrize("dim,sizes,ps", [(2, (1.0, 1.0), 0), (2, (1.0, 3.0), 0), (2, (1.0, 1.0), 1),
                                          (3, (1.0, 1.0, 1.0), 0), (3, (1.0, 2.0, 0.5), 0)])
def test_element_stiffness_matches_oracle(tg, O, dim, sizes, ps):
    Ke = tg.element_stiffness(dim, sizes, 1.0, 0.3, bool(ps))
    Ko = O.element_stiffness(dim, sizes, 1.0, 0.3, bool(ps))
    assert np.max(np.abs(Ke - Ko)) < 1e-14 * np.max(np.abs(Ko))


def test_host_argument_errors(tg):
    import ctypes
    L = tg.lib()
    nel = (ctypes.c_int32 * 3)(2, 2, 2)
    assert L.tog_grid_counts(4, nel, None, None, None) == 1
    bad = (ctypes.c_int32 * 3)(0, 2, 2)
    assert L.tog_grid_counts(3, bad, None, None, None) == 1
    assert b"nel" in L.tog_last_error()
    assert L.tog_destroy(None) == 0


def test_uneven_cantilever_set(tg):
    """The batched benchmark's problem set: nelx even in [64, 512], nely = nelx / 2, load node
    on the right edge, volume fraction in [0.3, 0.6], rmin in [1.5, 3.0]; seeded."""
    P = tg.uneven_cantilever_set(256, seed=0)
    assert len(P["nelx"]) == 256
    assert np.all(P["nelx"] % 2 == 0) and P["nelx"].min() >= 64 and P["nelx"].max() <= 512
    assert np.all(P["nely"] * 2 == P["nelx"])
    assert np.all((P["load_j"] >= 0) & (P["load_j"] <= P["nely"]))
    assert P["volfrac"].min() >= 0.3 and P["volfrac"].max() <= 0.6
    assert P["rmin"].min() >= 1.5 and P["rmin"].max() <= 3.0
    Q = tg.uneven_cantilever_set(256, seed=0)
    assert all(np.array_equal(P[k], Q[k]) for k in ("nelx", "nely", "load_j", "volfrac", "rmin"))


def test_fixed_element_projector_host_logic(tg):
    """FixedElementProjectorFun's constructor and queries are host logic
    (fixed_element.jl:19-27, 88-95, 127-159): no device call."""
    black = np.zeros(10, bool)
    black[:3] = True
    white = np.zeros(10, bool)
    white[7:] = True
    p = tg.FixedElementProjectorFun(10, black, white)
    assert tg.get_free_variable_count(p) == 4
    assert tg.get_free_variables(p).tolist() == [False] * 3 + [True] * 4 + [False] * 3
    with pytest.raises(ValueError):
        tg.FixedElementProjectorFun(5, np.array([1, 1, 1, 0, 0], bool), np.array([0, 0, 1, 1, 1], bool))
    with pytest.raises(ValueError):
        tg.FixedElementProjectorFun(5, np.zeros(5, bool), np.zeros(6, bool))
    q = tg.get_fixed_element_projector(100, range(0, 10), range(90, 100))
    assert (tg.get_free_variable_count(q), int(q.black.sum()), int(q.white.sum())) == (80, 10, 10)
    prob = tg.PointLoadCantilever((10, 6), (1.0, 1.0))
    r = tg.get_fixed_element_projector(prob, range(10), [])
    assert r.nel == 60 and tg.get_free_variable_count(r) == 50
    with pytest.raises(RuntimeError):   # the projection itself runs on a solver's device
        r(np.full(50, 0.5))


def test_multiload_host_setup(tg, O):
    """MultiLoad's load matrix from rules (multiload.jl:31-46, find_nearest_dofs :48-61),
    generate_scenarios (mean_compliance.jl:209-219) and the SVD columns of
    MeanComplianceFun's exact_svd method (trace.jl:15-34): host logic, no device call."""
    import scipy.sparse as sp
    from topopt_gb300 import topopt_api as api
    p = tg.PointLoadCantilever((10, 6), (1.0, 1.0))
    op = O.point_load_cantilever((10, 6), (1.0, 1.0))
    # nearest node of (9.6, 3.2) is (10, 3); its dofs in the reference (Ferrite) numbering
    # (the oracle keeps node_dofs as (dim, nnodes), as the reference)
    nid = 10 + 11 * 3
    assert list(tg.find_nearest_dofs(p, (9.6, 3.2))) == list(op.node_dofs[:, nid])
    mags = iter([1.0, 2.0, 3.0])
    ml = tg.MultiLoad(p, 3, [((10.0, 3.0), lambda: np.array([0.0, -next(mags)]))])
    F = ml.F.toarray()
    assert F.shape == (p.ndofs, 3) and ml.ncells == p.ncells
    assert np.array_equal(F[op.node_dofs[1, nid]], [-1.0, -2.0, -3.0])
    assert np.count_nonzero(F) == 3
    G = tg.generate_scenarios(5, (p.ndofs, 4), 2.0, perturb=lambda: 0.25).toarray()
    assert np.array_equal(G[5], [2.5] * 4) and np.count_nonzero(G) == 4
    # exact_svd: F F' is preserved by the U S columns (so is tr(F' K^-1 F))
    rng = np.random.default_rng(0)
    Fr = np.zeros((p.ndofs, 6))
    Fr[[3, 17, 40], :] = rng.standard_normal((3, 6))
    US = api._svd_columns(sp.csc_matrix(Fr)).toarray()
    assert US.shape[1] == 3
    assert np.allclose(US @ US.T, Fr @ Fr.T, atol=1e-12)
    with pytest.raises(ValueError):
        tg.MultiLoad(p, sp.csc_matrix((p.ndofs + 1, 2)))
    with pytest.raises(ValueError):
        tg.MeanComplianceFun(p, None)
