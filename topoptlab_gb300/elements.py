"""Element DOF maps and element matrices of the structured quad4 / hex8 grids.

The element matrices are evaluated once per problem on the host (they are
inputs of the GPU path, like the reference's ``lk`` callables); the element
DOF map is generated on the GPU by ``tg_edofmat``.

Mirrors:
  create_edofMat   elements/bilinear_quadrilateral.py:7-48,
                   elements/trilinear_hexahedron.py:7-58
  lk_linear_elast_2d   elements/linear_elasticity_2d.py:69 (plane stress)
  lk_linear_elast_3d   elements/linear_elasticity_3d.py:65
  lk_poisson_2d / 3d   elements/poisson_2d.py:68, elements/poisson_3d.py:62
  lk_screened_poisson_2d / 3d   elements/screenedpoisson_2d.py:8,
                   elements/screenedpoisson_3d.py:9 (Laplacian + consistent mass)
"""
from __future__ import annotations

import itertools

import numpy as np

from . import _lib

# Reference local node order as (dx, dy[, dz]) offsets from the element's
# lowest-index node; y is the index direction (grows downward in the figures),
# so the physical y coordinate of a node is 1 - dy.
_LOCAL_2D = [(0, 1), (1, 1), (1, 0), (0, 0)]
_LOCAL_3D = [(0, 1, 0), (1, 1, 0), (1, 0, 0), (0, 0, 0),
             (0, 1, 1), (1, 1, 1), (1, 0, 1), (0, 0, 1)]


def create_edofMat(nelx: int, nely: int, nelz: int | None = None, nnode_dof: int = 1,
                   device: int = 0, **kwargs):
    """Element DOF matrix (int32, nel x 2^ndim*nnode_dof) built on the GPU.

    Returns (edofMat, n1, n2, n3, n4) like the reference; the helper index
    arrays n1..n4 (first-corner node ids) are derived from edofMat."""
    ndim = 2 if nelz is None else 3
    nel = nelx * nely * (nelz if ndim == 3 else 1)
    ncol = (4 if ndim == 2 else 8) * nnode_dof
    out = np.empty((nel, ncol), dtype=np.int32)
    lib = _lib.load()
    rc = lib.tg_edofmat(ndim, nelx, nely, 0 if nelz is None else nelz, nnode_dof,
                        out.ctypes.data_as(_lib._i32p), device)
    _lib.check(rc, None, "tg_edofmat")
    node = out[:, ::nnode_dof] // nnode_dof
    n1, n2 = node[:, 3], node[:, 2]
    if ndim == 2:
        return out, n1, n2, None, None
    return out, n1, n2, node[:, 7], node[:, 6]


def _grad_N(xi, phys_corners):
    """Gradients of multilinear shape functions on [-1,1]^d at point xi."""
    d = len(xi)
    g = np.empty((len(phys_corners), d))
    for k, c in enumerate(phys_corners):
        s = 2 * np.asarray(c) - 1
        for a in range(d):
            v = 0.5 * s[a]
            for b in range(d):
                if b != a:
                    v *= 0.5 * (1 + s[b] * xi[b])
            g[k, a] = v
    return g


def _element_matrix(ndim, l, kernel):
    local = _LOCAL_2D if ndim == 2 else _LOCAL_3D
    phys = [(c[0], 1 - c[1]) + tuple(c[2:]) for c in local]
    l = np.broadcast_to(np.asarray(l, dtype=float), (ndim,))
    gp = np.array([-1.0, 1.0]) / np.sqrt(3.0)      # 2-point Gauss, exact here
    K = 0.0
    for xi in itertools.product(gp, repeat=ndim):
        dN = _grad_N(np.array(xi), phys) * (2.0 / l)[None, :]
        K = K + kernel(dN) * np.prod(l / 2.0)
    return np.asarray(K)


def _strain_matrix(dN, ndim):
    nn = dN.shape[0]
    if ndim == 2:
        B = np.zeros((3, 2 * nn))
        B[0, 0::2] = dN[:, 0]
        B[1, 1::2] = dN[:, 1]
        B[2, 0::2] = dN[:, 1]
        B[2, 1::2] = dN[:, 0]
        return B
    B = np.zeros((6, 3 * nn))
    B[0, 0::3], B[1, 1::3], B[2, 2::3] = dN[:, 0], dN[:, 1], dN[:, 2]
    B[3, 1::3], B[3, 2::3] = dN[:, 2], dN[:, 1]
    B[4, 0::3], B[4, 2::3] = dN[:, 2], dN[:, 0]
    B[5, 0::3], B[5, 1::3] = dN[:, 1], dN[:, 0]
    return B


def lk_linear_elast_2d(E: float = 1.0, nu: float = 0.3, plane_stress: bool = True,
                       l=np.array([1.0, 1.0]), t: float = 1.0, **kwargs) -> np.ndarray:
    if plane_stress:
        D = E / (1 - nu ** 2) * np.array([[1, nu, 0], [nu, 1, 0], [0, 0, (1 - nu) / 2]])
    else:
        c = E / ((1 + nu) * (1 - 2 * nu))
        D = c * np.array([[1 - nu, nu, 0], [nu, 1 - nu, 0], [0, 0, (1 - 2 * nu) / 2]])
    return t * _element_matrix(2, l, lambda dN: _strain_matrix(dN, 2).T @ D @ _strain_matrix(dN, 2))


def lk_linear_elast_3d(E: float = 1.0, nu: float = 0.3, l=np.array([1.0, 1.0, 1.0]),
                       **kwargs) -> np.ndarray:
    """Hexahedron element matrix identical to the reference closed form, whose
    shear stiffness is C11/2 = E(1-nu)/(2(1+nu)(1-2nu)) (not mu)."""
    c11 = E * (1 - nu) / ((1 + nu) * (1 - 2 * nu))
    c12 = E * nu / ((1 + nu) * (1 - 2 * nu))
    D = np.zeros((6, 6))
    D[:3, :3] = c12
    np.fill_diagonal(D[:3, :3], c11)
    D[3:, 3:] = np.eye(3) * c11 / 2
    return _element_matrix(3, l, lambda dN: _strain_matrix(dN, 3).T @ D @ _strain_matrix(dN, 3))


def lk_poisson_2d(k: float = 1.0, l=np.array([1.0, 1.0]), t: float = 1.0, **kwargs) -> np.ndarray:
    return t * k * _element_matrix(2, l, lambda dN: dN @ dN.T)


def lk_poisson_3d(k: float = 1.0, l=np.array([1.0, 1.0, 1.0]), **kwargs) -> np.ndarray:
    return k * _element_matrix(3, l, lambda dN: dN @ dN.T)


def _mass_matrix(ndim, l):
    """Consistent scalar mass matrix int N N^T (2-point Gauss, exact here)."""
    local = _LOCAL_2D if ndim == 2 else _LOCAL_3D
    phys = [np.array((c[0], 1 - c[1]) + tuple(c[2:])) for c in local]
    l = np.broadcast_to(np.asarray(l, dtype=float), (ndim,))
    gp = np.array([-1.0, 1.0]) / np.sqrt(3.0)
    M = np.zeros((len(phys), len(phys)))
    for xi in itertools.product(gp, repeat=ndim):
        N = np.array([np.prod(0.5 * (1 + (2 * c - 1) * np.asarray(xi))) for c in phys])
        M += np.outer(N, N) * np.prod(l / 2.0)
    return M


def lk_screened_poisson_2d(k: float = 1.0, l=np.array([1.0, 1.0]), t: float = 1.0,
                           **kwargs) -> np.ndarray:
    """k * Laplacian + mass; the Helmholtz filter uses k = (rmin / (2 sqrt 3))^2."""
    return t * (k * _element_matrix(2, l, lambda dN: dN @ dN.T) + _mass_matrix(2, l))


def lk_screened_poisson_3d(k: float = 1.0, l=np.array([1.0, 1.0, 1.0]), **kwargs) -> np.ndarray:
    return k * _element_matrix(3, l, lambda dN: dN @ dN.T) + _mass_matrix(3, l)
