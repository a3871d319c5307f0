"""Boundary-condition callables with the reference signature
``bcs(nelx, nely, nelz, ndof, **kw) -> (u, f, fixed, free, springs)``.

The driver also accepts the reference's own callables unchanged; these are
the ones a GPU machine without the reference package uses.

  mbb_2d                  example_bc/lin_elast.py:6-46
  cantilever_2d           example_bc/lin_elast.py:100-139
  cantilever_2d_twoloads  example_bc/lin_elast.py:141-182 (two load cases)
  cantilever_3d           example_bc/lin_elast.py:274-338
  heatplate_2d            example_bc/heat_conduction.py:5-49
"""
from __future__ import annotations

import numpy as np


def mbb_2d(nelx, nely, ndof, **kwargs):
    """Half MBB beam: x-DOFs of the left edge and the y-DOF of the bottom-right
    node fixed, unit downward load at the top-left node."""
    f = np.zeros((ndof, 1))
    u = np.zeros((ndof, 1))
    fixed = np.union1d(np.arange(0, 2 * (nely + 1), 2), np.array([ndof - 1]))
    f[1, 0] = -1.0
    return u, f, fixed, np.setdiff1d(np.arange(ndof), fixed), None


def cantilever_2d(nelx, nely, ndof, **kwargs):
    """All DOFs of the left wall fixed; unit downward load on the last DOF
    (the y-DOF of the bottom-right node)."""
    f = np.zeros((ndof, 1))
    u = np.zeros((ndof, 1))
    fixed = np.arange(0, 2 * (nely + 1))
    f[-1, 0] = -1.0
    return u, f, fixed, np.setdiff1d(np.arange(ndof), fixed), None


def cantilever_2d_twoloads(nelx, nely, ndof, **kwargs):
    """Left wall fixed; two load cases: downward unit load at the bottom-right
    node, upward unit load at the top-right node (y-DOF of node nelx*(nely+1))."""
    f = np.zeros((ndof, 2))
    u = np.zeros((ndof, 2))
    fixed = np.arange(0, 2 * (nely + 1))
    f[-1, 0] = -1.0
    f[2 * nelx * (nely + 1) + 1, 1] = 1.0
    return u, f, fixed, np.setdiff1d(np.arange(ndof), fixed), None


def cantilever_2d_wrong(nelx, nely, ndof, **kwargs):
    """cantilever_2d with the left wall's last DOF (the y-DOF of its bottom
    node) left free: fixed = 0 .. 2 nely (example_bc/lin_elast.py:230-272)."""
    f = np.zeros((ndof, 1))
    u = np.zeros((ndof, 1))
    fixed = np.arange(0, 2 * nely + 1)
    f[-1, 0] = -1.0
    return u, f, fixed, np.setdiff1d(np.arange(ndof), fixed), None


def cantilever_2d_twoloads_wrong(nelx, nely, ndof, **kwargs):
    """cantilever_2d_twoloads with fixed = 0 .. 2 nely
    (example_bc/lin_elast.py:184-228)."""
    f = np.zeros((ndof, 2))
    u = np.zeros((ndof, 2))
    fixed = np.arange(0, 2 * nely + 1)
    f[-1, 0] = -1.0
    f[2 * nelx * (nely + 1) + 1, 1] = 1.0
    return u, f, fixed, np.setdiff1d(np.arange(ndof), fixed), None


def cantilever_3d(nelx, nely, nelz, ndof, force_mode="linear", **kwargs):
    """All DOFs of the x=0 face and the z-DOFs of the z=0 plane fixed; a
    downward y-load on the bottom edge of the x=nelx face, one node per
    z-layer, linearly decreasing from 1 to 0 ("linear") or all 1 ("constant")."""
    nnx, nny, nnz = nelx + 1, nely + 1, nelz + 1
    f = np.zeros((ndof, 1))
    u = np.zeros((ndof, 1))
    z, y = np.meshgrid(np.arange(nnz), np.arange(nny), indexing="ij")
    wall = (z * nnx * nny + y).ravel()                      # nodes with x = 0
    zsym = np.arange(nnx * nny)                             # nodes with z = 0
    fixed = np.union1d(np.concatenate([3 * wall, 3 * wall + 1, 3 * wall + 2]), 3 * zsym + 2)
    if force_mode == "linear":
        load = -np.linspace(1.0, 0.0, nnz)
    elif force_mode == "constant":
        load = -1.0
    else:
        raise ValueError("force_mode must be either 'linear' or 'constant': ", force_mode)
    tip = np.arange(nnz) * nnx * nny + nelx * nny + nely    # (x=nelx, y=nely, z)
    f[3 * tip + 1, 0] = load
    return u, f, fixed, np.setdiff1d(np.arange(ndof), fixed), None


def heatplate_2d(nelx, nely, ndof, **kwargs):
    """Uniform source 0.01 on every node, T = 0 sink on the middle of the
    x = 0 edge (nodes int(nely/2 - nely/20) .. int(nely/2 + 1 + nely/20) - 1)."""
    f = np.full((ndof, 1), 0.01)
    u = np.zeros((ndof, 1))
    fixed = np.arange(int(nely / 2 - nely / 20), int(nely / 2 + 1 + nely / 20))
    return u, f, fixed, np.setdiff1d(np.arange(ndof), fixed), None


def heatplate_2d_element_source(nelx, nely, ndof, source=0.01, **kwargs):
    """heatplate_2d with a uniform volumetric source of `source` per element
    (each element's source split equally over its 4 nodes) instead of the
    reference's 0.01 per node; same T = 0 sink on the middle of the x = 0 edge."""
    u, _, fixed, free, springs = heatplate_2d(nelx, nely, ndof)
    cnt = np.zeros((nelx + 1, nely + 1))
    cnt[:-1, :-1] += 1
    cnt[1:, :-1] += 1
    cnt[:-1, 1:] += 1
    cnt[1:, 1:] += 1
    f = (0.25 * source * cnt).reshape(-1, 1)     # node (x, y) -> x*(nely+1) + y
    return u, f, fixed, free, springs
