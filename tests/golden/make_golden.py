"""Extract the reference's own golden vectors for the hot path into JSON fixtures.

Reads TopOpt.jl test sources AS TEXT (Julia is not available to run them) and
writes small JSON files next to this script.  Run from the repository root:

    python tests/golden/make_golden.py [/path/to/TopOpt.jl]

Sources:
  test/topopt_problems/metadata.jl:53-132  HalfMBB 2x2 coords, cells, node_dofs,
                                            cell_dofs, node_cells (1-based)
  test/topopt_problems/problems.jl:13-20   PointLoadCantilever 160x40 force_dof
  test/FEA/solvers.jl:32-59                solver-agreement case and tolerance
  test/Functions/test_common_fns.jl:32-49  compliance FD-gradient case and tolerance
  test/CheqFilters/test_filters.jl:71-73    too-small rmin throws
  test/inp_parser/MBB.inp, parser.jl:36-59  the structured CPS4 MBB mesh (described by its
                                            lattice, sets, supports, load and material) and
                                            the parser's asserted values for it
"""
import json
import os
import re
import sys

HERE = os.path.dirname(os.path.abspath(__file__))


def _matrix_after(src, name):
    m = re.search(name + r"\s*=\s*\[(.*?)\]", src, re.S)
    rows = [r.split() for r in m.group(1).strip().splitlines() if r.strip()]
    return [[int(v) for v in r] for r in rows]


def main(ref):
    meta = open(os.path.join(ref, "test/topopt_problems/metadata.jl")).read()
    coords = [[float(a), float(b)] for a, b in
              re.findall(r"\(([-\d.]+),\s*([-\d.]+)\),?\n", meta.split("coords = [")[1].split("]")[0])]
    cells = [[int(v) for v in t.split(",")] for t in
             re.findall(r"Ferrite\.Quadrilateral\(\(([\d, ]+)\)\),?\n", meta.split("cells = [")[1].split("]\n")[0])]
    node_dofs = _matrix_after(meta, r"\n    node_dofs")
    cell_dofs = _matrix_after(meta, r"\n    cell_dofs")
    node_cells = {}
    for n, body in re.findall(r"node_cells\[(\d+)\] == \[(.*?)\]\n", meta):
        node_cells[int(n)] = [[int(a), int(b)] for a, b in re.findall(r"\((\d+),\s*(\d+)\)", body)]
    out = dict(source="test/topopt_problems/metadata.jl:53-132", problem="HalfMBB((2,2),(1.0,1.0),1.0,0.3,1.0)",
               index_base=1, coords=coords, cells=cells, node_dofs=node_dofs, cell_dofs=cell_dofs,
               node_cells={str(k): v for k, v in sorted(node_cells.items())})
    with open(os.path.join(HERE, "metadata_2x2.json"), "w") as f:
        json.dump(out, f, indent=1)

    probs = open(os.path.join(ref, "test/topopt_problems/problems.jl")).read()
    m = re.search(r"PointLoadCantilever\(\((\d+), (\d+)\).*?force_dof == ([\d* ]+)\n", probs, re.S)
    nx, ny, expr = int(m.group(1)), int(m.group(2)), m.group(3)
    val = 1
    for t in expr.split("*"):
        val *= int(t)
    solv = open(os.path.join(ref, "test/FEA/solvers.jl")).read()
    ms = re.search(r"nels = \((\d+), (\d+), (\d+)\).*?force = ([-\d.]+).*?fill\(([\d.]+).*?"
                   r"solver_matrixfree\.u ≈ solver_direct\.u rtol = ([\de.-]+)", solv, re.S)
    fns = open(os.path.join(ref, "test/Functions/test_common_fns.jl")).read()
    mf = re.search(r'@testset "ComplianceFun" begin.*?nels = \((\d+), (\d+)\).*?'
                   r"for p in \(([\d., ]+)\).*?xmin=([\d.]+).*?norm\(grad2 - grad3\) <= ([\de.-]+)", fns, re.S)
    filt = open(os.path.join(ref, "test/CheqFilters/test_filters.jl")).read()
    mr = re.search(r"@test_throws ArgumentError DensityFilterFun\(solver; rmin=([\d.]+)\)", filt)
    pins = dict(
        cantilever_force_dof=dict(source="test/topopt_problems/problems.jl:13-20",
                                  nels=[nx, ny], force_dof_1based=val),
        solver_agreement=dict(source="test/FEA/solvers.jl:32-59",
                              nels=[int(ms.group(1)), int(ms.group(2)), int(ms.group(3))],
                              force=float(ms.group(4)), x=float(ms.group(5)), abstol=1e-7,
                              rtol=float(ms.group(6))),
        compliance_fd=dict(source="test/Functions/test_common_fns.jl:32-49",
                           nels=[int(mf.group(1)), int(mf.group(2))], xmin=float(mf.group(4)),
                           penalties=[float(v) for v in mf.group(3).split(",")],
                           tol=float(mf.group(5))),
        filter_too_small_rmin=dict(source="test/CheqFilters/test_filters.jl:71-73",
                                   nels=[5, 5], rmin=float(mr.group(1))),
    )
    with open(os.path.join(HERE, "reference_pins.json"), "w") as f:
        json.dump(pins, f, indent=1)
    inp_mbb(ref)
    print("wrote metadata_2x2.json, reference_pins.json and inp_mbb.json")


def inp_mbb(ref):
    """MBB.inp is a structured quad mesh: record it as its lattice (checked node by node
    and cell by cell), its node sets, *BOUNDARY and *CLOAD entries and material, and the
    values test/inp_parser/parser.jl asserts for it."""
    text = open(os.path.join(ref, "test/inp_parser/MBB.inp")).read().splitlines()
    sec, nodes, cells, nsets, bcs, cl, mat = None, [], [], {}, [], [], None
    for i, line in enumerate(text):
        if line.startswith("*"):
            sec = line
            if line.startswith("*NSET"):
                nsets[re.search(r"NSET\s*=\s*([^,\s]*)", line).group(1)] = []
            if line.startswith("*ELASTIC"):
                mat = [float(v) for v in text[i + 1].split(",")]
            continue
        v = [t.strip() for t in line.split(",") if t.strip()]
        if not v:
            continue
        if sec.startswith("*Node"):
            nodes.append([float(t) for t in v[1:]])
        elif sec.startswith("*Element"):
            cells.append([int(t) for t in v[1:]])
        elif sec.startswith("*NSET"):
            list(nsets.values())[-1].extend(int(t) for t in v)
        elif sec.startswith("*BOUNDARY"):
            bcs.append([v[0], int(v[1])])
        elif sec.startswith("*CLOAD"):
            cl.append([int(v[0]), int(v[1]), float(v[2])])
    xs = sorted({c[0] for c in nodes})
    ys = sorted({c[1] for c in nodes})
    nnx, h = len(xs), xs[1] - xs[0]
    for k, c in enumerate(nodes):   # x fastest from id 1, spacing h, origin (0, 0)
        assert c == [h * (k % nnx), h * (k // nnx)], k
    for e, c in enumerate(cells):   # x fastest, corners (n, n+1, n+1+nnx, n+nnx)
        n = 1 + e % (nnx - 1) + nnx * (e // (nnx - 1))
        assert c == [n, n + 1, n + 1 + nnx, n + nnx], e
    par = open(os.path.join(ref, "test/inp_parser/parser.jl")).read()
    blk = par.split('extract_inp(joinpath(@__DIR__, "MBB.inp"))')[1].split("extract_inp")[0]
    pins = dict(
        celltype=re.search(r'celltype == "(\w+)"', blk).group(1),
        node_coords={k: [float(a), float(b)] for k, a, b in
                     re.findall(r"node_coords\[(\d+)\] == \(([-\d.]+), ([-\d.]+)\)", blk)},
        cells={k: [int(t) for t in v.split(",")] for k, v in re.findall(r"cells\[(\d+)\] == \(([\d, ]+)\)", blk)},
        nodedbcs={k: [[int(a), float(b)] for a, b in re.findall(r"\((\d+), ([-\d.]+)\)", v)]
                  for k, v in re.findall(r'nodedbcs\["(\w+)"\] == \[(.*?)\]\n', blk)},
        cloads={k: [float(t) for t in v.split(",")] for k, v in re.findall(r"cloads\[(\d+)\] == \[([-\d., ]+)\]", blk)},
        density=float(re.search(r"density == ([-\d.]+)", blk).group(1)),
        E=float(re.search(r"\.E == ([-\d.]+)", blk).group(1)),
        nu=float(re.search(r"\.ν == ([-\d.]+)", blk).group(1)))
    out = dict(source="test/inp_parser/MBB.inp; asserted values test/inp_parser/parser.jl:36-59",
               lattice=dict(nn=[nnx, len(ys)], spacing=[h, ys[1] - ys[0]], origin=[0.0, 0.0],
                            celltype="CPS4", node_order="x fastest from 1",
                            cell_order="x fastest, corners (n, n+1, n+1+nnx, n+nnx)"),
               nsets=nsets, boundary=bcs, cload=cl, material=mat, pins=pins)
    with open(os.path.join(HERE, "inp_mbb.json"), "w") as f:
        json.dump(out, f, indent=1)


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_golden.py <TopOpt.jl checkout>")
    main(sys.argv[1])
