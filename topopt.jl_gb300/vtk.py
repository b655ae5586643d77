"""save_mesh: the design as a VTK unstructured grid (.vtu), the output format of
TopOpt.jl's src/TopOptProblems/IO/VTK.jl:17-71.

As the reference: every node of the grid, and one cell (VTK_QUAD = 9 in 2D,
VTK_HEXAHEDRON = 12 in 3D) per element whose density is >= 0.5, its nodes in
Ferrite's local order -- (i, j), (i+1, j), (i+1, j+1), (i, j+1), on the plane z = k
then z = k + 1 -- which is VTK's order for these cells.  Coordinates are padded to
three components in 2D, as WriteVTK does.  The arrays are written inline in VTK's
XML "binary" encoding (base64 of a UInt64 byte count followed by the data).
"""
import base64

import numpy as np

VTK_QUAD, VTK_HEXAHEDRON = 9, 12


def _b64(a):
    raw = np.ascontiguousarray(a).tobytes()
    return base64.b64encode(np.uint64(len(raw)).tobytes() + raw).decode("ascii")


def _vtk_type(a):
    return {np.dtype(np.float64): "Float64", np.dtype(np.int64): "Int64", np.dtype(np.uint8): "UInt8"}[a.dtype]


def mesh_arrays(problem, vars=None):
    """(points (nnodes, 3), connectivity of the kept cells (k, 2^dim), their cell ids)."""
    dim = problem.dim
    nels = problem.nels
    nn = [n + 1 for n in nels]
    x = np.ones(problem.ncells) if vars is None else np.asarray(vars, dtype=np.float64)
    if x.shape != (problem.ncells,):
        raise ValueError("Density vector must have length equal to number of cells (%d)" % problem.ncells)
    ix, iy, iz = problem._node_grid()
    pts = np.zeros((problem.nnodes, 3))
    pts[:, 0] = ix * problem.sizes[0]
    pts[:, 1] = iy * problem.sizes[1]
    if dim == 3:
        pts[:, 2] = iz * problem.sizes[2]
    e = np.nonzero(x >= 0.5)[0]
    ex = e % nels[0]
    ey = (e // nels[0]) % nels[1]
    ez = e // (nels[0] * nels[1]) if dim == 3 else np.zeros_like(e)
    base = ex + nn[0] * (ey + nn[1] * ez)
    quad = [0, 1, 1 + nn[0], nn[0]]
    local = quad if dim == 2 else quad + [q + nn[0] * nn[1] for q in quad]
    conn = base[:, None] + np.asarray(local, dtype=np.int64)[None, :]
    return pts, conn.astype(np.int64), e


def save_mesh(filename, problem, vars=None):
    """Write `filename`.vtu (the suffix is added when missing) for `problem` with the
    densities `vars` (all ones when omitted); returns the path written."""
    pts, conn, _ = mesh_arrays(problem, vars)
    k, npc = conn.shape
    offsets = np.arange(1, k + 1, dtype=np.int64) * npc
    types = np.full(k, VTK_QUAD if problem.dim == 2 else VTK_HEXAHEDRON, dtype=np.uint8)
    path = filename if filename.endswith(".vtu") else filename + ".vtu"

    def arr(name, a, ncomp=1):
        return ('<DataArray type="%s" Name="%s" NumberOfComponents="%d" format="binary">%s</DataArray>'
                % (_vtk_type(a), name, ncomp, _b64(a)))

    with open(path, "w") as f:
        f.write('<?xml version="1.0"?>\n')
        f.write('<VTKFile type="UnstructuredGrid" version="1.0" byte_order="LittleEndian" header_type="UInt64">\n')
        f.write('<UnstructuredGrid>\n<Piece NumberOfPoints="%d" NumberOfCells="%d">\n' % (pts.shape[0], k))
        f.write("<Points>\n%s\n</Points>\n" % arr("Points", pts.astype("<f8"), 3))
        f.write("<Cells>\n%s\n%s\n%s\n</Cells>\n" % (arr("connectivity", conn.astype("<i8")),
                                                     arr("offsets", offsets.astype("<i8")),
                                                     arr("types", types)))
        f.write("</Piece>\n</UnstructuredGrid>\n</VTKFile>\n")
    return path
