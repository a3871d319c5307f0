"""Element flags of simple shapes on the structured 2-D grid, for ``el_flags``
(passive / active elements).  Mirrors geometries.py:6-72 (``sphere``,
``ellipse``): element e = ex * nely + ey, shape centre and sizes in element
indices, flag ``fill_value`` inside, 0 outside."""
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
