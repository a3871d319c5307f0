"""VTK export against what the reference's export_vtk hands to meshio
(tests/golden/vtk.npz, recorded by tests/golden/make_golden.py): the same
points, the same cells in the same node order, the same point data per load
case and the same cell data, including the thresholded design."""
import os

import numpy as np
import pytest

from topoptlab_gb300.output_designs import export_stl, export_vtk, threshold

GOLD = os.path.join(os.path.dirname(__file__), "golden", "vtk.npz")


def _read_legacy_vtk(path):
    """Minimal reader for the ASCII legacy unstructured-grid files written by
    export_vtk: returns points, cells, cell types, point and cell fields."""
    toks = open(path).read().split("\n")
    i, out = 0, {"point_data": {}, "cell_data": {}}
    section = None

    def block(n, width):
        nonlocal i
        rows = [np.array(toks[i + k].split(), dtype=float) for k in range(n)]
        i += n
        return np.array(rows).reshape(n, width)

    while i < len(toks):
        line = toks[i].split()
        i += 1
        if not line:
            continue
        key = line[0]
        if key == "POINTS":
            out["points"] = block(int(line[1]), 3)
        elif key == "CELLS":
            n = int(line[1])
            rows = [np.array(toks[i + k].split(), dtype=np.int64) for k in range(n)]
            i += n
            out["cells"] = np.array([r[1:] for r in rows])
            assert all(r[0] == len(r) - 1 for r in rows)
        elif key == "CELL_TYPES":
            out["types"] = block(int(line[1]), 1)[:, 0].astype(int)
        elif key == "POINT_DATA":
            section, npts = "point_data", int(line[1])
        elif key == "CELL_DATA":
            section, ncell = "cell_data", int(line[1])
        elif key == "SCALARS":
            i += 1                                   # LOOKUP_TABLE
            n = npts if section == "point_data" else ncell
            out[section][line[1]] = block(n, 1)
        elif key == "VECTORS":
            out[section][line[1]] = block(npts, 3)
    return out


@pytest.mark.parametrize("tag,dims", [("2d", (4, 3, None)), ("3d", (3, 2, 2))])
def test_export_vtk_matches_reference_mesh(tmp_path, tag, dims):
    g = np.load(GOLD)
    nx, ny, nz = dims
    path = export_vtk(str(tmp_path / "design"), nelx=nx, nely=ny, nelz=nz,
                      xPhys=g[f"{tag}_in_xPhys"], x=g[f"{tag}_in_x"], u=g[f"{tag}_in_u"],
                      f=g[f"{tag}_in_f"], volfrac=0.4)
    m = _read_legacy_vtk(path)
    pts = g[f"{tag}_points"]
    ndim = pts.shape[1]
    np.testing.assert_array_equal(m["points"][:, :ndim], pts)
    np.testing.assert_array_equal(m["points"][:, ndim:], 0.0)
    np.testing.assert_array_equal(m["cells"], g[f"{tag}_cells"])
    expect_type = {"quad": 9, "hexahedron": 12}[str(g[f"{tag}_celltype"])]
    assert (m["types"] == expect_type).all()
    for name in ("u0", "u1", "f0", "f1"):
        ref = g[f"{tag}_pd_{name}"]
        got = m["point_data"][name]
        np.testing.assert_array_equal(got[:, :ref.shape[1]], ref)
        np.testing.assert_array_equal(got[:, ref.shape[1]:], 0.0)
    for name in ("xPhys", "x", "xThresh"):
        np.testing.assert_array_equal(m["cell_data"][name], g[f"{tag}_cd_{name}"])


def test_threshold_volume_and_order():
    x = np.array([[0.2], [0.9], [0.5], [0.7], [0.1]])
    t = threshold(x, 0.5)                       # floor(2.5) = 2 solid elements
    np.testing.assert_array_equal(t[:, 0], [0, 1, 0, 1, 0])


def test_export_vtk_element_size(tmp_path):
    path = export_vtk(str(tmp_path / "s"), nelx=2, nely=1, nelz=None,
                      xPhys=np.ones((2, 1)), elem_size=np.array([0.5, 2.0]))
    m = _read_legacy_vtk(path)
    assert m["points"][:, 0].max() == 1.0 and m["points"][:, 1].max() == 2.0


def test_export_stl_matches_reference_triangles(tmp_path):
    """The triangles export_stl hands to meshio (output_designs.py:181-230),
    recorded with the mask flattened, facet by facet and in order."""
    g = np.load(GOLD)
    path = export_stl(str(tmp_path / "design"), nelx=4, nely=3, xPhys=g["2d_in_xPhys"],
                      volfrac=0.4)
    lines = [ln.split() for ln in open(path)]
    verts = np.array([[float(v) for v in ln[1:]] for ln in lines if ln and ln[0] == "vertex"])
    normals = np.array([[float(v) for v in ln[2:]] for ln in lines if ln and ln[0] == "facet"])
    ref = g["stl_points"][g["stl_tris"]].reshape(-1, 2)
    assert str(g["stl_celltype"]) == "triangle"
    assert verts.shape == (ref.shape[0], 3)
    np.testing.assert_array_equal(verts[:, :2], ref)
    np.testing.assert_array_equal(verts[:, 2], 0.0)
    np.testing.assert_allclose(np.abs(normals[:, 2]), 1.0)
    assert lines[0][0] == "solid" and lines[-1][0] == "endsolid"
