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
    print("wrote metadata_2x2.json and reference_pins.json")


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_golden.py <TopOpt.jl checkout>")
    main(sys.argv[1])
