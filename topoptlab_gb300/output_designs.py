"""Design export for visualisation (e.g. ParaView): legacy-format VTK files of
the structured quad4 / hex8 grid with the element densities and the nodal
fields, and STL files of the thresholded 2-D design, written without meshio.

Mirrors topoptlab.output_designs (output_designs.py:7-178): the same point
coordinates (x = ex, y = nely - ey, z = ez; y counted downwards like the
node numbering), the same cell node order as the reference's ``idMat``
(quad4 (n1+1, n2+1, n2, n1), counter-clockwise; hex8 the bottom then the top
face), point data ``u{i}`` / ``f{i}`` per load case and cell data ``xPhys``,
``x``, ``xTilde`` and the thresholded ``xThresh``.  The reference writes
through meshio's legacy VTK writer; this module writes the ASCII form of the
same legacy format directly.
"""
from __future__ import annotations

from typing import Optional, Union

import numpy as np


def threshold(xPhys: np.ndarray, volfrac: float) -> np.ndarray:
    """Black and white design with the volume fraction's number of solid
    elements: the floor(volfrac * nel) densest elements are 1, the rest 0
    (output_designs.py:7-34)."""
    xPhys = np.asarray(xPhys).reshape(-1, 1)
    order = np.flip(np.argsort(xPhys[:, 0]))     # numpy's default sort, as the reference: same ties
    nsolid = int(np.floor(volfrac * xPhys.shape[0]))
    xt = np.zeros(xPhys.shape)
    xt[order[:nsolid]] = 1.0
    print("Thresholded Vol.: {0:.5f}".format(nsolid / xt.shape[0]))
    return xt


def _points(nelx: int, nely: int, nelz: Optional[int]) -> np.ndarray:
    if nelz is None:
        ex, ey = np.meshgrid(np.arange(nelx + 1), np.arange(nely + 1), indexing="ij")
        return np.column_stack((ex.ravel(), (nely - ey).ravel(), np.zeros(ex.size)))
    ez, ex, ey = np.meshgrid(np.arange(nelz + 1), np.arange(nelx + 1), np.arange(nely + 1),
                             indexing="ij")
    return np.column_stack((ex.ravel(), (nely - ey).ravel(), ez.ravel())).astype(np.float64)


def _cells(nelx: int, nely: int, nelz: Optional[int]) -> np.ndarray:
    if nelz is None:
        ex, ey = np.meshgrid(np.arange(nelx), np.arange(nely), indexing="ij")
        n1 = ((nely + 1) * ex + ey).ravel()
        n2 = ((nely + 1) * (ex + 1) + ey).ravel()
        return np.column_stack((n1 + 1, n2 + 1, n2, n1))
    ez, ex, ey = np.meshgrid(np.arange(nelz), np.arange(nelx), np.arange(nely), indexing="ij")
    plane = (nelx + 1) * (nely + 1)
    n1 = (plane * ez + (nely + 1) * ex + ey).ravel()
    n2 = (plane * ez + (nely + 1) * (ex + 1) + ey).ravel()
    n3 = n1 + plane
    n4 = n2 + plane
    return np.column_stack((n1 + 1, n2 + 1, n2, n1, n3 + 1, n4 + 1, n4, n3))


def _write_point_field(fh, name: str, v: np.ndarray, npts: int) -> None:
    comps = v.shape[0] // npts
    a = v.reshape(npts, comps)
    if comps == 1:
        fh.write(f"SCALARS {name} double 1\nLOOKUP_TABLE default\n")
        np.savetxt(fh, a, fmt="%.17g")
    else:                                   # vectors are 3-component in VTK
        b = np.zeros((npts, 3))
        b[:, :comps] = a
        fh.write(f"VECTORS {name} double\n")
        np.savetxt(fh, b, fmt="%.17g")


def export_vtk(filename: str, nelx: int, nely: int, xPhys: np.ndarray,
               nelz: Union[None, int], x: Optional[np.ndarray] = None,
               u: Optional[np.ndarray] = None, f: Optional[np.ndarray] = None,
               u_bw: Optional[np.ndarray] = None, f_bw: Optional[np.ndarray] = None,
               xTilde: Optional[np.ndarray] = None,
               elem_size: Union[None, float, np.ndarray] = None,
               volfrac: Optional[float] = None, stress_vm=None) -> str:
    """Write ``filename + ".vtk"`` (output_designs.py:36-178); returns the path."""
    pts = _points(nelx, nely, nelz)
    if elem_size is not None:
        ndim = 2 if nelz is None else 3
        h = np.full(ndim, float(elem_size)) if np.isscalar(elem_size) else \
            np.asarray(elem_size, dtype=float)
        pts[:, :ndim] *= h[None, :]
    cells = _cells(nelx, nely, nelz)
    ncell, nper = cells.shape
    vtk_type = 9 if nper == 4 else 12           # VTK_QUAD / VTK_HEXAHEDRON
    path = filename + ".vtk"
    with open(path, "w") as fh:
        fh.write("# vtk DataFile Version 4.2\ntopoptlab_gb300 design\nASCII\n"
                 "DATASET UNSTRUCTURED_GRID\n")
        fh.write(f"POINTS {pts.shape[0]} double\n")
        np.savetxt(fh, pts, fmt="%.17g")
        fh.write(f"CELLS {ncell} {ncell * (nper + 1)}\n")
        np.savetxt(fh, np.column_stack((np.full(ncell, nper), cells)), fmt="%d")
        fh.write(f"CELL_TYPES {ncell}\n")
        np.savetxt(fh, np.full(ncell, vtk_type), fmt="%d")
        fields = [("u", u), ("u_bw", u_bw), ("f", f), ("f_bw", f_bw)]
        fields = [(n, np.asarray(v).reshape(v.shape[0], -1)) for n, v in fields if v is not None]
        if fields:
            fh.write(f"POINT_DATA {pts.shape[0]}\n")
            for name, v in fields:
                for i in range(v.shape[1]):
                    _write_point_field(fh, f"{name}{i}", v[:, i], pts.shape[0])
        fh.write(f"CELL_DATA {ncell}\n")
        cell_fields = [("xPhys", xPhys), ("x", x), ("xTilde", xTilde)]
        if volfrac is not None:
            cell_fields.append(("xThresh", threshold(xPhys, volfrac)))
        if stress_vm is not None:
            cell_fields.append(("stress_vm", stress_vm))
        for name, v in cell_fields:
            if v is None:
                continue
            fh.write(f"SCALARS {name} double 1\nLOOKUP_TABLE default\n")
            np.savetxt(fh, np.asarray(v, dtype=np.float64).reshape(-1), fmt="%.17g")
    return path


def export_stl(filename: str, nelx: int, nely: int, xPhys: np.ndarray, volfrac: float) -> str:
    """Write ``filename + ".stl"`` (ASCII STL, z = 0): the thresholded 2-D
    design as two triangles per solid element, (n1+1, n2+1, n2) for every
    solid element and then (n1+1, n2, n1) for every solid element, over the
    points of export_vtk (output_designs.py:181-230).  The reference indexes
    the cells with threshold()'s (nel, 1) mask, which NumPy rejects; the mask
    is used flattened here.  Facet normals follow the vertex winding."""
    mask = threshold(xPhys, volfrac)[:, 0] == 1
    pts = _points(nelx, nely, None)
    cells = _cells(nelx, nely, None)[mask]
    tris = np.vstack((cells[:, [0, 1, 2]], cells[:, [0, 2, 3]]))
    path = filename + ".stl"
    with open(path, "w") as fh:
        fh.write("solid topoptlab_gb300\n")
        for t in tris:
            v = pts[t]
            nrm = np.cross(v[1] - v[0], v[2] - v[0])
            ln = np.linalg.norm(nrm)
            nrm = nrm / ln if ln > 0 else nrm
            fh.write("  facet normal {:.9g} {:.9g} {:.9g}\n    outer loop\n".format(*nrm))
            for p in v:
                fh.write("      vertex {:.17g} {:.17g} {:.17g}\n".format(*p))
            fh.write("    endloop\n  endfacet\n")
        fh.write("endsolid topoptlab_gb300\n")
    return path
