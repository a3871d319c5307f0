"""Compliance objective (objectives.py:7-55).

``compliance`` keeps the reference signature so driver code that passes
``obj_func=compliance`` selects the GPU's fused compliance + sensitivity
kernel; called directly it evaluates on the GPU for structured grids whose
size it infers from ``edofMat`` and the element matrix."""
from __future__ import annotations

import atexit

import numpy as np

# the context of the last grid / element matrix / SIMP parameters evaluated
# (a design loop calls compliance with the same ones every iteration)
_CTX: dict = {}


@atexit.register
def _close_contexts():
    for p in _CTX.values():
        p.close()
    _CTX.clear()


def grid_from_edofmat(edofMat, nedof):
    """(nelx, nely, nelz or None, nnode_dof) of the structured grid whose
    element-DOF matrix (the reference's numbering, elements/
    bilinear_quadrilateral.py:7-48, trilinear_hexahedron.py:7-58) is edofMat:
    element 0's corner nodes give nely (and nelx in 3-D), the element count
    the rest; element 0 and the last element are checked against them."""
    ed = np.asarray(edofMat)
    nel, ncol = ed.shape
    if ncol != nedof:
        raise ValueError(f"edofMat has {ncol} columns, the element matrix {nedof} rows")
    if ncol == 4:
        ndim, nd = 2, 1
    elif ncol == 24:
        ndim, nd = 3, 3
    elif ncol == 8:
        # quad4 with 2 DOFs per node numbers a node's DOFs consecutively
        ndim, nd = (2, 2) if ed[0, 1] == ed[0, 0] + 1 else (3, 1)
    else:
        raise ValueError(f"no structured quad4 / hex8 layout has {ncol} DOFs per element")
    node = ed[:, ::nd] // nd                     # corner node ids
    nely = int(node[0, 2]) - 1                   # corner (1, 0[, 0]) of element 0
    if nely < 1:
        raise ValueError("edofMat does not follow the structured numbering")
    if ndim == 2:
        nelx, nelz = nel // nely, None
        dims = (nelx, nely)
    else:
        nelx = int(node[0, 7]) // (nely + 1) - 1  # corner (0, 0, 1) of element 0
        if nelx < 1 or nel % (nelx * nely):
            raise ValueError("edofMat does not follow the structured numbering")
        nelz = nel // (nelx * nely)
        dims = (nelx, nely, nelz)
    if int(np.prod(dims)) != nel:
        raise ValueError("edofMat does not follow the structured numbering")
    # the last element's corners: ((z*(nelx+1)) + x)*(nely+1) + y
    ex, ey = nelx - 1, nely - 1
    ez = (nelz - 1) if ndim == 3 else 0
    corners = ([(0, 1), (1, 1), (1, 0), (0, 0)] if ndim == 2 else
               [(0, 1, 0), (1, 1, 0), (1, 0, 0), (0, 0, 0),
                (0, 1, 1), (1, 1, 1), (1, 0, 1), (0, 0, 1)])
    for k, c in enumerate(corners):
        dz = c[2] if ndim == 3 else 0
        want = ((ez + dz) * (nelx + 1) + ex + c[0]) * (nely + 1) + ey + c[1]
        if int(node[-1, k]) != want:
            raise ValueError("edofMat does not follow the structured numbering")
    return nelx, nely, nelz, nd


def compliance(xPhys, u, KE, edofMat, i, matinterpol, matinterpol_kw, obj, **kwargs):
    """obj += sum simp(xPhys) u_e^T KE u_e ; returns (obj, -u, True).

    The grid comes from ``edofMat``; ``nelx``, ``nely`` (and ``nelz``)
    keywords, when given, take precedence."""
    from .context import GpuProblem
    KE = np.ascontiguousarray(np.asarray(KE, dtype=np.float64))
    if "nelx" in kwargs:
        nelx, nely, nelz = kwargs["nelx"], kwargs["nely"], kwargs.get("nelz")
    else:
        nelx, nely, nelz, _ = grid_from_edofmat(edofMat, KE.shape[0])
    u = np.asarray(u)
    ndof = u.shape[0]
    eps = matinterpol_kw.get("eps", 1e-9)
    penal = matinterpol_kw.get("penal", 3.0)
    key = (nelx, nely, nelz, ndof, KE.tobytes(), eps, penal)
    prob = _CTX.get(key)
    if prob is None:
        for old in _CTX.values():
            old.close()
        _CTX.clear()
        prob = GpuProblem(nelx, nely, nelz, KE, np.zeros(0, np.int64), np.zeros(ndof), 0.5, 1.5,
                          precond="gb300-jacobi", eps=eps, penal=penal)
        _CTX[key] = prob
    col = u[:, i] if u.ndim == 2 else u
    val, _ = prob.compliance(np.asarray(xPhys).reshape(-1), col)
    return obj + val, -u, True
