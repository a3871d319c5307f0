"""Element flags of simple shapes on the structured grid, for ``el_flags``
(passive / active elements).  Mirrors geometries.py (``sphere``, ``ellipse``
in 2-D, element e = ex * nely + ey; ``ball``, ``ellipsoid`` in 3-D,
e = (ez * nelx + ex) * nely + ey): shape centre and sizes in element indices,
flag ``fill_value`` inside, 0 outside.  ``ellipsoid`` keeps the reference's
test, which takes two semi-axes (the same ellipse in every z-layer)."""
from __future__ import annotations

import numpy as np


def _ij(nelx: int, nely: int):
    return np.divmod(np.arange(nelx * nely, dtype=np.int32), nely)


def sphere(nelx: int, nely: int, center, radius: float, fill_value: int = 1) -> np.ndarray:
    """Flags of the elements with (ex - cx)^2 + (ey - cy)^2 <= radius^2."""
    i, j = _ij(nelx, nely)
    flags = np.zeros(nelx * nely, dtype=np.int32)
    flags[(i - center[0]) ** 2 + (j - center[1]) ** 2 <= radius ** 2] = fill_value
    return flags


def ellipse(nelx: int, nely: int, center, ax_half_lengths, fill_value: int = 1) -> np.ndarray:
    """Flags of the elements inside the axis-aligned ellipse with semi-axes (a, b)."""
    i, j = _ij(nelx, nely)
    a, b = ax_half_lengths
    flags = np.zeros(nelx * nely, dtype=np.int32)
    flags[((i - center[0]) ** 2) / a ** 2 + ((j - center[1]) ** 2) / b ** 2 <= 1.0] = fill_value
    return flags


def _ijk(nelx: int, nely: int, nelz: int):
    k, ij = np.divmod(np.arange(nelx * nely * nelz, dtype=np.int32), nelx * nely)
    i, j = np.divmod(ij, nely)
    return i, j, k


def ball(nelx: int, nely: int, nelz: int, center, radius: float, fill_value: int = 1) -> np.ndarray:
    """Flags of the elements with |(ex, ey, ez) - center| <= radius."""
    i, j, k = _ijk(nelx, nely, nelz)
    flags = np.zeros(nelx * nely * nelz, dtype=np.int32)
    flags[(i - center[0]) ** 2 + (j - center[1]) ** 2 + (k - center[2]) ** 2 <= radius ** 2] = fill_value
    return flags


def ellipsoid(nelx: int, nely: int, nelz: int, center, ax_half_lengths,
              fill_value: int = 1) -> np.ndarray:
    """Flags of the elements inside the ellipse of semi-axes (a, b), in every
    z-layer (the reference's test; like the reference it takes exactly two
    semi-axes)."""
    i, j, _ = _ijk(nelx, nely, nelz)
    a, b = ax_half_lengths
    flags = np.zeros(nelx * nely * nelz, dtype=np.int32)
    flags[((i - center[0]) ** 2) / a ** 2 + ((j - center[1]) ** 2) / b ** 2 <= 1.0] = fill_value
    return flags
