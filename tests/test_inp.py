"""Abaqus .inp import (InpStiffness, src/TopOptProblems/IO/INP/inpstiffness.jl:37-52;
parser src/TopOptProblems/IO/INP/Parser/Parser.jl:61-170) on structured grids.

The reference's MBB.inp (a structured CPS4 mesh, recorded in tests/golden/inp_mbb.json by
tests/golden/make_golden.py as its lattice, sets, supports, load and material) is written
back as text and parsed: every value test/inp_parser/parser.jl:36-59 asserts for it must
come out.  The structured problem built from it must equal the directly built one,
export / import round trips must be exact, and unstructured or unsupported input must
raise ValueError (the reference's ArgumentError)."""
import json
import os

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


def _mbb_text(tmp_path, boundary=None):
    d = json.load(open(os.path.join(HERE, "golden", "inp_mbb.json")))
    if boundary is not None:
        d = dict(d, boundary=boundary)
    lat = d["lattice"]
    nnx, nny = lat["nn"]
    hx, hy = lat["spacing"]
    lines = ["*Heading", "*Node, NSET=Nall"]
    for k in range(nnx * nny):
        lines.append("%d, %r, %r" % (k + 1, hx * (k % nnx), hy * (k // nnx)))
    lines.append("*Element, TYPE=%s, ELSET=EALL" % lat["celltype"])
    for e in range((nnx - 1) * (nny - 1)):
        n = 1 + e % (nnx - 1) + nnx * (e // (nnx - 1))
        lines.append("%d, %d, %d, %d, %d " % (e + 1, n, n + 1, n + 1 + nnx, n + nnx))
    lines += ["*MATERIAL, NAME=Steel", "*ELASTIC", "%r, %r" % tuple(d["material"])]
    for name, members in d["nsets"].items():
        lines += ["*NSET, NSET=%s" % name, ", ".join(map(str, members))]
    lines.append("*BOUNDARY")
    lines += ["%s, %d" % (n, c) for n, c in d["boundary"]]
    lines.append("*CLOAD")
    lines += ["%d, %d, %r" % (n, c, v) for n, c, v in d["cload"]]
    lines.append("*End Step")
    path = tmp_path / "mbb.inp"
    path.write_text("\n".join(lines) + "\n")
    return path, d


def test_parser_matches_reference_assertions_on_mbb(tg, tmp_path):
    path, d = _mbb_text(tmp_path)
    c = tg.parse_inp(str(path))
    pins = d["pins"]
    assert c.celltype == pins["celltype"]
    for k, v in pins["node_coords"].items():
        assert list(c.node_coords[int(k) - 1]) == v
    for k, v in pins["cells"].items():
        assert list(c.cells[int(k) - 1]) == v
    for k, v in pins["nodedbcs"].items():
        assert [list(t) for t in c.nodedbcs[k]] == v
    for k, v in pins["cloads"].items():
        assert list(c.cloads[int(k)]) == v
    assert c.density == pins["density"] and c.E == pins["E"] and c.nu == pins["nu"]
    assert c.cellsets["EALL"] == list(range(1, 401))


def test_inp_stiffness_is_the_structured_problem(tg, tmp_path):
    path, d = _mbb_text(tmp_path)
    p = tg.InpStiffness(str(path))
    assert p.nels == (40, 10) and p.sizes == (5.0, 5.0) and p.E == 42000.0 and p.nu == 0.2
    nd = p.node_dofs
    # roller_support: node 1 (0, 0) in x; fixed_support: node 41 (200, 0) in x and y
    want = sorted([nd[0, 0], nd[40, 0], nd[40, 1]])
    assert list(p.fixed_dofs) == want
    f = p.load_vector()
    assert f[nd[430, 1]] == -3.0 and np.count_nonzero(f) == 1
    # the file lists nodes and cells in this library's order: the maps are identities
    assert np.array_equal(p.inp_node_to_grid, np.arange(p.nnodes))
    assert np.array_equal(p.inp_cell_to_grid, np.arange(p.ncells))
    u = np.arange(p.ndofs, dtype=float)
    assert np.array_equal(p.to_inp_dofs(u), u)


@pytest.mark.parametrize("nels", [(6, 4), (5, 3, 4)])
def test_export_import_round_trip_with_shuffled_cells(tg, tmp_path, nels):
    prob = tg.HalfMBB(nels, (1.0,) * len(nels)) if len(nels) == 2 else tg.PointLoadCantilever(
        (6, 4, 4), (0.5, 1.0, 2.0))
    path = tmp_path / "p.inp"
    tg.write_inp(str(path), prob)
    back = tg.InpStiffness(str(path))
    assert back.nels == prob.nels and np.allclose(back.sizes, prob.sizes)
    assert np.array_equal(back.fixed_dofs, prob.fixed_dofs)
    assert np.array_equal(back.load_vector(), prob.load_vector())
    # the same mesh with its cells listed in another order and other node ids
    c = tg.parse_inp(str(path))
    rng = np.random.default_rng(0)
    cp = rng.permutation(c.cells.shape[0])
    npm = rng.permutation(c.node_coords.shape[0])      # new id of old node i is npm[i] + 1
    inv = np.argsort(npm)
    c2 = tg.InpContent(c.node_coords[inv], c.celltype, npm[c.cells[cp] - 1] + 1,
                       {k: [int(npm[m - 1] + 1) for m in v] for k, v in c.nodesets.items()}, {}, c.E, c.nu, 0.0,
                       c.nodedbcs, {int(npm[k - 1] + 1): v for k, v in c.cloads.items()}, {}, {})
    p2 = tg.InpStiffness(c2)
    assert np.array_equal(p2.fixed_dofs, prob.fixed_dofs)
    assert np.array_equal(p2.load_vector(), prob.load_vector())
    x = rng.random(prob.ncells)
    assert np.array_equal(p2.to_grid_cells(p2.to_inp_cells(x)), x)
    assert np.array_equal(p2.inp_cell_to_grid, cp)


def test_unsupported_meshes_raise(tg, tmp_path):
    bad = {
        "tri": "*Node, NSET=Nall\n1, 0, 0\n2, 1, 0\n3, 0, 1\n*Element, TYPE=CPS3, ELSET=E\n1, 1, 2, 3\n"
               "*MATERIAL, NAME=M\n*ELASTIC\n1.0, 0.3\n",
        "graded": "*Node, NSET=Nall\n1, 0, 0\n2, 1, 0\n3, 3, 0\n4, 0, 1\n5, 1, 1\n6, 3, 1\n"
                  "*Element, TYPE=CPS4, ELSET=E\n1, 1, 2, 5, 4\n2, 2, 3, 6, 5\n*MATERIAL, NAME=M\n*ELASTIC\n1.0, 0.3\n",
        "clockwise": "*Node, NSET=Nall\n1, 0, 0\n2, 1, 0\n3, 0, 1\n4, 1, 1\n"
                     "*Element, TYPE=CPS4, ELSET=E\n1, 1, 3, 4, 2\n*MATERIAL, NAME=M\n*ELASTIC\n1.0, 0.3\n",
        "prescribed": "*Node, NSET=Nall\n1, 0, 0\n2, 1, 0\n3, 0, 1\n4, 1, 1\n"
                      "*Element, TYPE=CPS4, ELSET=E\n1, 1, 2, 4, 3\n*MATERIAL, NAME=M\n*ELASTIC\n1.0, 0.3\n"
                      "*NSET, NSET=S\n1\n*BOUNDARY\nS, 1, 1, 0.5\n",
        "no_material": "*Node, NSET=Nall\n1, 0, 0\n2, 1, 0\n3, 0, 1\n4, 1, 1\n"
                       "*Element, TYPE=CPS4, ELSET=E\n1, 1, 2, 4, 3\n",
        "first_node": "*Node, NSET=Nall\n2, 0, 0\n3, 1, 0\n",
    }
    for name, text in bad.items():
        path = tmp_path / (name + ".inp")
        path.write_text(text)
        with pytest.raises(ValueError):
            tg.InpStiffness(str(path))


@pytest.mark.gpu
def test_inp_problem_solves_like_the_oracle(tg, O, tmp_path):
    """The MBB mesh read from an .inp file, solved on the GPU (FP64 PCG and FP32-IR) at
    random densities, against the oracle's direct solve of the same problem: 1e-8.  The
    file's own supports (x at node 1, x and y at node 41) leave the rotation about node 41
    free, so the beam is simply supported here instead (y at node 1)."""
    path, _ = _mbb_text(tmp_path, boundary=[["roller_support", 2], ["fixed_support", 1], ["fixed_support", 2]])
    p = tg.InpStiffness(str(path))
    g = O.rectilinear_grid(p.nels, p.sizes)
    nd, cd = O.dof_numbering(g)
    op = O.Problem(g, p.E, p.nu, 1.0, nd, cd, np.asarray(p.fixed_dofs, dtype=np.int64), p.load_vector(), -1, -1)
    st = O.fea_setup(op, xmin=1e-3, p=3.0)
    rng = np.random.default_rng(5)
    x = rng.uniform(0.2, 1.0, p.ncells)
    st.vars = x
    ud = O.direct_solve(st)
    for precision in ("fp64", "fp32_ir"):
        s = tg.FEASolver(tg.GB300Solver, p, xmin=1e-3, penalty=tg.PowerPenaltyFun(3.0), rtol=1e-11, abstol=0.0,
                         cg_max_iter=100000, precision=precision)
        s.vars = x
        s()
        assert np.linalg.norm(s.u - ud) / np.linalg.norm(ud) < 1e-8, precision
        s.close()
