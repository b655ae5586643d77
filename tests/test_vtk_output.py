"""save_mesh (src/TopOptProblems/IO/VTK.jl:17-71): the .vtu file read back holds every
node, one cell per element with density >= 0.5, in the oracle grid's (Ferrite's)
connectivity and coordinates, with VTK quad / hexahedron types.  Host-only code."""
import base64
import xml.etree.ElementTree as ET

import numpy as np
import pytest


def _read(path):
    root = ET.parse(path).getroot()
    piece = root.find("UnstructuredGrid/Piece")
    arrays = {}
    dt = {"Float64": "<f8", "Int64": "<i8", "UInt8": "u1"}
    for a in root.iter("DataArray"):
        raw = base64.b64decode(a.text)
        n = int(np.frombuffer(raw[:8], "<u8")[0])
        arrays[a.get("Name")] = np.frombuffer(raw[8:8 + n], dt[a.get("type")])
    return int(piece.get("NumberOfPoints")), int(piece.get("NumberOfCells")), arrays


@pytest.mark.parametrize("nels", [(10, 6), (4, 4), (4, 4, 2), (5, 3, 4)])
def test_save_mesh_round_trip(tg, O, nels, tmp_path):
    sizes = tuple(1.0 + 0.5 * i for i in range(len(nels)))
    cls = tg.PointLoadCantilever if nels[1] % 2 == 0 and (len(nels) == 2 or nels[2] % 2 == 0) else tg.HalfMBB
    if cls is tg.HalfMBB and len(nels) == 3:
        cls = tg.LoadedCantilever
        p = cls(nels, sizes, (0, 0), (0.0, -1.0, 0.0))
    else:
        p = cls(nels, sizes)
    grid = O.rectilinear_grid(nels, sizes)
    rng = np.random.default_rng(len(nels) * 10 + nels[0])
    for vars_ in (None, np.full(p.ncells, 0.7), rng.uniform(0, 1, p.ncells), np.zeros(p.ncells)):
        path = tg.save_mesh(str(tmp_path / "design"), p, vars_)
        assert path.endswith(".vtu")
        npts, ncells, a = _read(path)
        keep = np.arange(p.ncells) if vars_ is None else np.nonzero(vars_ >= 0.5)[0]
        assert npts == grid.nnodes and ncells == len(keep)
        pts = a["Points"].reshape(-1, 3)
        assert np.allclose(pts[:, :len(nels)], grid.coords, rtol=0, atol=1e-12)
        npc = 2 ** len(nels)
        assert np.array_equal(a["connectivity"].reshape(-1, npc), grid.cells[keep])
        assert np.array_equal(a["offsets"], npc * np.arange(1, ncells + 1))
        assert np.all(a["types"] == (9 if len(nels) == 2 else 12))
    with pytest.raises(ValueError):
        tg.save_mesh(str(tmp_path / "bad"), p, np.ones(p.ncells + 1))
