"""Abaqus .inp files: import (InpStiffness) restricted to structured quad4 / hex8
grids, and export of a structured problem.

The reader follows the reference's parser section by section
(src/TopOptProblems/IO/INP/Parser/Parser.jl:61-170 and FeatureExtractors/*.jl):
``*Node, NSET=Nall`` (ids from 1, consecutive), ``*Element, TYPE=..., ELSET=...``
(consecutive ids; the element id offset is subtracted from ELSET members),
``*NSET`` / ``*ELSET`` (numbers or names of earlier sets), ``*MATERIAL`` followed by
``*ELASTIC`` (E, nu), ``*BOUNDARY`` (set, dof[, last dof[, value]]), ``*CLOAD``
(node, dof, value; repeated entries add) and ``*DLOAD`` (element, Pface, value).

InpStiffness (src/TopOptProblems/IO/INP/inpstiffness.jl:37-52) builds a problem from
the content.  The GPU kernels run structured grids only, so the mesh must be a
rectilinear lattice of CPS4 (2D) or C3D8 / C3D8R (3D) cells with uniform spacing per
axis, every lattice cell present once with the Abaqus / Ferrite corner order; anything
else -- other element types, unstructured or graded meshes, prescribed non-zero
displacements, pressure (DLOAD) loads -- raises ValueError, the reference's
ArgumentError.  The problem's vectors are in this library's reference dof numbering
(the first-touch numbering of the lattice's cells in x-fastest order); the mesh's own
numbering is available through ``inp_node_to_grid``, ``inp_cell_to_grid`` and
``to_inp_dofs``.
"""
import re
from dataclasses import dataclass, field

import numpy as np

from .topopt_api import _StructuredProblem, node_dofs

_STOP = re.compile(r"^\*[^\*]")
_NODE_HEAD = re.compile(r"\*Node\s*,\s*NSET\s*=\s*([^,]*)")
_CELL_HEAD = re.compile(r"\*Element\s*,\s*TYPE\s*=\s*([^,]*)\s*,\s*ELSET\s*=\s*([^,]*)")
_NSET_HEAD = re.compile(r"\*NSET\s*,\s*NSET\s*=\s*([^,]*)")
_ELSET_HEAD = re.compile(r"\*ELSET\s*,\s*ELSET\s*=\s*([^,]*)")
_MAT_HEAD = re.compile(r"\*MATERIAL\s*,\s*NAME\s*=\s*([^\s]*)")
_BC_HEAD = re.compile(r"\*BOUNDARY")
_CLOAD_HEAD = re.compile(r"\*CLOAD")
_DLOAD_HEAD = re.compile(r"\*DLOAD")
_NUM = r"-?\d+\.?\d*(?:[eE][-\+]?\d+)?"
_FNUM = r"[-+]?\d*\.?\d+(?:[eE][-+]?\d+)?"


@dataclass
class InpContent:
    """The parsed file (Parser.jl:24-37): node coordinates (nnodes x dim), cell type,
    cells (1-based node ids, ncells x nodes per cell), node and cell sets (1-based ids),
    E, nu, density, node boundary conditions {set: [(dof, value)]}, concentrated loads
    {node: load vector}, face sets {name: [(cell, face)]} and pressures {face set: p}."""
    node_coords: np.ndarray
    celltype: str
    cells: np.ndarray
    nodesets: dict = field(default_factory=dict)
    cellsets: dict = field(default_factory=dict)
    E: float = 0.0
    nu: float = 0.0
    density: float = 0.0
    nodedbcs: dict = field(default_factory=dict)
    cloads: dict = field(default_factory=dict)
    facesets: dict = field(default_factory=dict)
    dloads: dict = field(default_factory=dict)

    @property
    def dim(self):
        return self.node_coords.shape[1]


class _Lines:
    def __init__(self, path):
        with open(path) as f:
            self.lines = f.read().splitlines()
        self.i = 0

    def next(self):
        """The next line, or None at the end of the file."""
        if self.i >= len(self.lines):
            return None
        line = self.lines[self.i]
        self.i += 1
        return line


def _section_lines(src):
    """Lines up to the next keyword line (the reference's stopping pattern); returns
    (body lines, the keyword line or None)."""
    body = []
    while True:
        line = src.next()
        if line is None or _STOP.match(line):
            return body, line
        body.append(line)


def _parse_nodes(body):
    pat = re.compile(r"(\d+)\s*,\s*(%s)\s*,\s*(%s)\s*(?:,\s*(%s))?" % (_NUM, _NUM, _NUM))
    coords, prev = [], 0
    for line in body:
        m = pat.match(line.strip())
        if not m:
            continue
        idx = int(m.group(1))
        if not coords and idx != 1:
            raise ValueError("First node index is not 1.")
        if coords and idx != prev + 1:
            raise ValueError("Node indices are not consecutive.")
        c = [float(m.group(2)), float(m.group(3))]
        if m.group(4) is not None:
            c.append(float(m.group(4)))
        if coords and len(c) != len(coords[0]):
            raise ValueError("Nodes of different dimensions.")
        coords.append(c)
        prev = idx
    if not coords:
        raise ValueError("Failed to parse node data from first line")
    return np.asarray(coords, dtype=np.float64)


def _parse_cells(body):
    cells, first, prev = [], None, None
    for line in body:
        m = re.match(r"^(\d+)\s*,", line.strip())
        if not m:
            continue
        idx = int(m.group(1))
        nodes = [int(v) for v in re.findall(r",\s*(\d+)", line)]
        if first is None:
            first = idx
        elif idx != prev + 1:
            raise ValueError("Cell indices are not consecutive.")
        elif len(nodes) != len(cells[0]):
            raise ValueError("Cell %d has fewer nodes than it should." % idx)
        cells.append(nodes)
        prev = idx
    if not cells:
        raise ValueError("Failed to parse cell index from first line")
    return np.asarray(cells, dtype=np.int64), first - 1


def _parse_set(sets, name, body, offset=0):
    members = []
    for line in body:
        s = line.strip()
        if re.match(r"^\d+", s):
            members.extend(int(v) - offset for v in re.findall(r"(\d+)", s))
        else:
            m = re.match(r"^([^,]+)", s)
            if m and m.group(1) in sets:
                members.extend(sets[m.group(1)])
    sets[name] = members


def _parse_boundary(dbcs, body):
    for line in body:
        s = line.strip()
        m = re.match(r"([^,]+)\s*,\s*(\d)\s*,\s*(\d)\s*,\s*(\-?\d+\.\d*)", s)
        if m:
            dofs, val = range(int(m.group(2)), int(m.group(3)) + 1), float(m.group(4))
        else:
            m = re.match(r"([^,]+)\s*,\s*(\d)\s*,\s*(\d)", s)
            if m:
                dofs, val = range(int(m.group(2)), int(m.group(3)) + 1), 0.0
            else:
                m = re.match(r"([^,]+)\s*,\s*(\d)", s)
                if not m:
                    continue
                dofs, val = [int(m.group(2))], 0.0
        dbcs.setdefault(m.group(1), []).extend((d, val) for d in dofs)


def _parse_cload(cloads, body, dim):
    pat = re.compile(r"\s*(%s)\s*,\s*(%s)\s*,\s*(%s)\s*" % (_FNUM, _FNUM, _FNUM))
    for line in body:
        m = pat.match(line)
        if not m:
            continue
        node, dof, load = int(float(m.group(1))), int(float(m.group(2))), float(m.group(3))
        vec = cloads.setdefault(node, np.zeros(dim))
        vec[dof - 1] += load


def _parse_dload(dloads, facesets, body, offset):
    pat = re.compile(r"(\d+)\s*,\s*P(\d+)\s*,\s*(\-?\d+\.\d*)")
    name = "DLOAD_SET_%d" % (len(dloads) + 1)
    facesets[name] = []
    load, first = 0.0, True
    for line in body:
        m = pat.search(line)
        if not m:
            continue
        val = float(m.group(3))
        if not first and val != load:
            raise ValueError("Loads in the same DLOAD set are not equal.")
        load, first = val, False
        facesets[name].append((int(m.group(1)) - offset, int(m.group(2))))
    dloads[name] = load


def parse_inp(path):
    """Read an Abaqus .inp file into an InpContent (Parser.jl:61-170)."""
    src = _Lines(path)
    coords = celltype = cells = None
    offset = 0
    nodesets, cellsets, dbcs, cloads, facesets, dloads = {}, {}, {}, {}, {}, {}
    E = nu = None
    line = src.next()
    while line is not None:
        m = _NODE_HEAD.match(line)
        if m and m.group(1).strip() == "Nall":
            body, line = _section_lines(src)
            coords = _parse_nodes(body)
            continue
        m = _CELL_HEAD.match(line)
        if m:
            celltype = m.group(1).strip()
            body, line = _section_lines(src)
            cells, offset = _parse_cells(body)
            cellsets[m.group(2).strip()] = list(range(1, len(cells) + 1))
            continue
        m = _NSET_HEAD.match(line)
        if m:
            body, line = _section_lines(src)
            _parse_set(nodesets, m.group(1).strip(), body)
            continue
        m = _ELSET_HEAD.match(line)
        if m:
            body, line = _section_lines(src)
            _parse_set(cellsets, m.group(1).strip(), body, offset)
            continue
        if _MAT_HEAD.match(line):
            el = src.next()
            if el is None or not re.match(r"\*ELASTIC", el):
                raise ValueError("Expected *ELASTIC section in material definition")
            vals = src.next()
            m = re.search(r"(-?\d+\.?\d*)\s*,\s*(-?\d+\.?\d*)", vals or "")
            if not m:
                raise ValueError("Failed to parse Young's modulus and Poisson ratio from material data")
            E, nu = float(m.group(1)), float(m.group(2))
            line = src.next()
            continue
        if _BC_HEAD.match(line):
            body, line = _section_lines(src)
            _parse_boundary(dbcs, body)
            continue
        if _CLOAD_HEAD.match(line):
            body, line = _section_lines(src)
            _parse_cload(cloads, body, 0 if coords is None else coords.shape[1])
            continue
        if _DLOAD_HEAD.match(line):
            body, line = _section_lines(src)
            _parse_dload(dloads, facesets, body, offset)
            continue
        line = src.next()
    if coords is None:
        raise ValueError("INP file missing *Node section")
    if cells is None:
        raise ValueError("INP file missing *Element section")
    if E is None:
        raise ValueError("INP file missing *Material section")
    return InpContent(coords, celltype, cells, nodesets, cellsets, E, nu, 0.0, dbcs, cloads, facesets, dloads)


# Corner order of a lattice cell (Abaqus CPS4 / C3D8 = Ferrite Quadrilateral / Hexahedron):
# counter-clockwise in x-y, the z = k face before the z = k + 1 face.
_CORNERS = {2: [(0, 0, 0), (1, 0, 0), (1, 1, 0), (0, 1, 0)],
            3: [(0, 0, 0), (1, 0, 0), (1, 1, 0), (0, 1, 0), (0, 0, 1), (1, 0, 1), (1, 1, 1), (0, 1, 1)]}
_TYPES = {"CPS4": 2, "C3D8": 3, "C3D8R": 3}


def _lattice(values, axis):
    """Sorted distinct coordinates of one axis and their uniform spacing (or ValueError)."""
    v = np.unique(values)
    if v.size < 2:
        raise ValueError("the mesh is flat along axis %d" % axis)
    h = np.diff(v)
    tol = 1e-9 * max(1.0, float(np.max(np.abs(v))))
    if np.max(h) - np.min(h) > tol:
        raise ValueError("INP mesh is not a structured grid: axis %d spacing is not uniform" % axis)
    return v, float(np.mean(h))


class InpStiffness(_StructuredProblem):
    """A stiffness problem from an Abaqus .inp file (InpStiffness, inpstiffness.jl:37-52)
    whose mesh is a structured grid: see the module docstring for what is accepted."""

    def __init__(self, path_or_content):
        c = path_or_content if isinstance(path_or_content, InpContent) else parse_inp(path_or_content)
        self.inp_content = c
        dim = _TYPES.get(c.celltype)
        if dim is None:
            raise ValueError("InpStiffness on the GPU runs CPS4 / C3D8 structured grids; cell type %s is not "
                             "supported" % c.celltype)
        if c.dim != dim:
            raise ValueError("cell type %s needs %d-D nodes" % (c.celltype, dim))
        if c.dloads:
            raise ValueError("pressure loads (*DLOAD) are not supported on this path")
        axes = [_lattice(c.node_coords[:, a], a) for a in range(dim)]
        nels = tuple(v.size - 1 for v, _ in axes)
        sizes = tuple(h for _, h in axes)
        nn = [v.size for v, _ in axes]
        if int(np.prod(nn)) != c.node_coords.shape[0]:
            raise ValueError("INP mesh is not a structured grid: %d nodes for a %s lattice"
                             % (c.node_coords.shape[0], "x".join(map(str, nn))))
        ijk = np.stack([np.rint((c.node_coords[:, a] - axes[a][0][0]) / axes[a][1]).astype(np.int64)
                        for a in range(dim)], axis=1)
        for a in range(dim):
            if np.max(np.abs(axes[a][0][0] + ijk[:, a] * axes[a][1] - c.node_coords[:, a])) > \
                    1e-9 * max(1.0, float(np.max(np.abs(c.node_coords[:, a])))):
                raise ValueError("INP mesh is not a structured grid: a node is off the lattice")
        lin = ijk[:, 0] + nn[0] * ijk[:, 1] + (nn[0] * nn[1] * ijk[:, 2] if dim == 3 else 0)
        if np.unique(lin).size != lin.size:
            raise ValueError("INP mesh is not a structured grid: two nodes on one lattice point")
        if c.cells.shape[1] != 2 ** dim:
            raise ValueError("cells must have %d nodes" % 2 ** dim)
        cell_ijk = ijk[c.cells[:, 0] - 1]
        for k, off in enumerate(_CORNERS[dim]):
            want = cell_ijk + np.asarray(off[:dim])
            if not np.array_equal(ijk[c.cells[:, k] - 1], want):
                raise ValueError("INP mesh is not a structured grid: cells are not lattice cells in the "
                                 "Abaqus corner order")
        ecell = cell_ijk[:, 0] + nels[0] * cell_ijk[:, 1] + (nels[0] * nels[1] * cell_ijk[:, 2] if dim == 3 else 0)
        if np.unique(ecell).size != int(np.prod(nels)) or ecell.size != int(np.prod(nels)):
            raise ValueError("INP mesh is not a structured grid: its cells do not cover the lattice once")
        super().__init__(nels, sizes, c.E, c.nu, 1.0, False)
        self.inp_node_to_grid = lin
        self.inp_cell_to_grid = ecell
        fixed = []
        for name, entries in c.nodedbcs.items():
            if name not in c.nodesets:
                raise ValueError("*BOUNDARY names an unknown node set %s" % name)
            nodes = lin[np.asarray(c.nodesets[name], dtype=np.int64) - 1]
            for dof, val in entries:
                if val != 0.0:
                    raise ValueError("prescribed non-zero displacements are not supported on this path")
                if not 1 <= dof <= dim:
                    raise ValueError("*BOUNDARY dof %d outside 1..%d" % (dof, dim))
                fixed.append(self.node_dofs[nodes, dof - 1])
        self.fixed_dofs = np.unique(np.concatenate(fixed)).astype(np.int32) if fixed else np.zeros(0, np.int32)
        self._f = np.zeros(self.ndofs)
        for node, vec in c.cloads.items():
            self._f[self.node_dofs[lin[node - 1]]] += vec
        # the mesh's own first-touch dof numbering (Ferrite DofHandler over the file's cells)
        own = -np.ones(c.node_coords.shape[0], dtype=np.int64)
        order = []
        for n in c.cells.ravel() - 1:
            if own[n] < 0:
                own[n] = len(order)
                order.append(n)
        self._inp_first_touch = own

    def load_vector(self):
        return self._f.copy()

    def to_inp_dofs(self, u):
        """A dof vector of this library (reference numbering of the lattice) in the mesh's
        own first-touch numbering."""
        u = np.asarray(u)
        out = np.empty_like(u)
        for c in range(self.dim):
            out[self.dim * self._inp_first_touch + c] = u[self.node_dofs[self.inp_node_to_grid, c]]
        return out

    def to_grid_cells(self, x_inp):
        """Cell values in the file's cell order -> this library's (x-fastest) cell order."""
        out = np.empty(self.ncells)
        out[self.inp_cell_to_grid] = np.asarray(x_inp)
        return out

    def to_inp_cells(self, x_grid):
        return np.asarray(x_grid)[self.inp_cell_to_grid]


def write_inp(path, problem, *, origin=None, material="Material", loads=None):
    """Write a structured problem (nels, sizes, fixed dofs, load vector) as an Abaqus
    .inp file in the layout the reader accepts: nodes x fastest from id 1, CPS4 / C3D8
    cells in x-fastest order, one node set per constrained component, *BOUNDARY and
    *CLOAD entries."""
    dim = problem.dim
    nn = [n + 1 for n in problem.nels]
    org = np.zeros(dim) if origin is None else np.asarray(origin, dtype=np.float64)
    idx = np.arange(problem.nnodes)
    ijk = [idx % nn[0], (idx // nn[0]) % nn[1]] + ([idx // (nn[0] * nn[1])] if dim == 3 else [])
    nd = problem.node_dofs
    lines = ["*Heading", "** structured grid written by topopt.jl_gb300", "*Node, NSET=Nall"]
    for n in range(problem.nnodes):
        xs = [org[a] + ijk[a][n] * problem.sizes[a] for a in range(dim)]
        lines.append("%d, %s" % (n + 1, ", ".join(repr(float(v)) for v in xs)))
    lines.append("*Element, TYPE=%s, ELSET=Eall" % ("CPS4" if dim == 2 else "C3D8"))
    e = 0
    for k in range(problem.nels[2] if dim == 3 else 1):
        for j in range(problem.nels[1]):
            for i in range(problem.nels[0]):
                e += 1
                ids = [1 + (i + o[0]) + nn[0] * ((j + o[1]) + nn[1] * (k + o[2])) for o in _CORNERS[dim]]
                lines.append("%d, %s" % (e, ", ".join(map(str, ids))))
    lines += ["*MATERIAL, NAME=%s" % material, "*ELASTIC", "%r, %r" % (float(problem.E), float(problem.nu))]
    fixed = np.zeros(problem.ndofs, dtype=bool)
    fixed[np.asarray(problem.fixed_dofs, dtype=np.int64)] = True
    bcs = []
    for c in range(dim):
        nodes = np.nonzero(fixed[nd[:, c]])[0]
        if nodes.size:
            name = "fixed_%d" % (c + 1)
            lines.append("*NSET, NSET=%s" % name)
            for a in range(0, nodes.size, 16):
                lines.append(", ".join(str(int(v) + 1) for v in nodes[a:a + 16]))
            bcs.append("%s, %d" % (name, c + 1))
    if bcs:
        lines.append("*BOUNDARY")
        lines += bcs
    f = problem.load_vector() if loads is None else loads
    entries = []
    for n in range(problem.nnodes):
        for c in range(dim):
            v = f[nd[n, c]]
            if v != 0.0:
                entries.append("%d, %d, %r" % (n + 1, c + 1, float(v)))
    if entries:
        lines.append("*CLOAD")
        lines += entries
    lines.append("*End Step")
    with open(path, "w") as fh:
        fh.write("\n".join(lines) + "\n")
