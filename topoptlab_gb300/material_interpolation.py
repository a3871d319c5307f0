"""Modified SIMP interpolation (material_interpolation.py:6-62).

These host functions identify the interpolation scheme that main passes to
the GPU (eps, penal); the GPU kernels evaluate the same formulas in FP64."""
from __future__ import annotations

import numpy as np


def simp(xPhys: np.ndarray, eps: float, penal: float, **kwargs) -> np.ndarray:
    return eps + (1 - eps) * xPhys ** penal


def simp_dx(xPhys: np.ndarray, eps: float, penal: float, **kwargs) -> np.ndarray:
    return penal * (1 - eps) * xPhys ** (penal - 1)
