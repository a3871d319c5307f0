"""Filter objects of the reference's modular filter interface, evaluated on
the GPU.

Mirrors filter/filter.py:7-94 (``TOFilter``: ``apply_filter``,
``apply_filter_dx``, ``vol_conserv``), filter/matrix_filter.py:9-99
(``MatrixFilter``) and filter/helmholtz_filter.py:16-131
(``HelmholtzFilter``).  In the reference both concrete classes leave the
abstract ``vol_conserv`` unimplemented and cannot be instantiated; here they
implement it, with the reference's arithmetic otherwise:

* ``MatrixFilter.apply_filter(x)`` and ``apply_filter_dx(dx_filtered)`` are
  both ``H (v / Hs)`` (matrix_filter.py:56-99), H the distance filter with
  weights ``max(0, rmin - |d|)`` and Hs its row sums;
* ``HelmholtzFilter.apply_filter(x)`` and ``apply_filter_dx(x_filtered,
  dx_filtered)`` are ``TF^T KF^-1 TF v`` (helmholtz_filter.py:69-131),
  2-D only like ``assemble_helmholtz_filter`` (helmholtz_filter.py:180).

Both conserve volume: ``1^T H (x / Hs) = sum(x)`` for the symmetric H, and
``KF 1 = M 1 = TF 1`` without boundary conditions gives
``1^T TF^T KF^-1 TF x = 1^T TF x = sum(x)``.  Periodic boundary conditions
(``pbc``) are not implemented on the GPU path and raise ValueError.

Each object owns a small library context on one structured grid (scalar
element matrix, Jacobi preconditioning, no loads); call ``close()`` (or use
it as a context manager) to release its device memory.
"""
from __future__ import annotations

from abc import ABC, abstractmethod
from typing import Any, Union

import numpy as np

from .context import GpuProblem
from .elements import lk_poisson_2d, lk_poisson_3d

_MODE_MATRIX = 1        # tg_filter: H (x / Hs)
_MODE_HELMHOLTZ = 6     # tg_filter: TF^T KF^-1 TF x


class TOFilter(ABC):
    """Base class of filters (filter/filter.py:7-94)."""

    @abstractmethod
    def apply_filter(self, x: np.ndarray) -> np.ndarray:
        ...

    @abstractmethod
    def apply_filter_dx(self, *args: np.ndarray) -> np.ndarray:
        ...

    @property
    @abstractmethod
    def vol_conserv(self) -> bool:
        ...


class _GpuFilter(TOFilter):
    """A filter evaluated by ``tg_filter`` on its own context."""

    _mode = _MODE_MATRIX

    def __init__(self, nelx: int, nely: int, rmin: float, nelz: Union[int, None],
                 filter_mode: str, l: Union[None, np.ndarray] = None, device: int = 0) -> None:
        ndim = 2 if nelz is None else 3
        KE = lk_poisson_2d() if ndim == 2 else lk_poisson_3d()
        nnodes = (nelx + 1) * (nely + 1) * ((nelz + 1) if ndim == 3 else 1)
        self.nel = nelx * nely * (nelz if ndim == 3 else 1)
        self._prob = GpuProblem(nelx, nely, nelz, KE, np.zeros(0, dtype=np.int64),
                                np.zeros(nnodes), 0.5, rmin, ft=1, precond="gb300-jacobi",
                                device=device, filter_mode=filter_mode, filter_l=l)

    def _apply(self, v: np.ndarray) -> np.ndarray:
        v = np.asarray(v, dtype=np.float64)
        if v.size != self.nel:
            raise ValueError(f"expected {self.nel} element values, got {v.size}")
        return self._prob.filter(v.reshape(-1), self._mode).reshape(v.shape)

    @property
    def vol_conserv(self) -> bool:
        return True

    def close(self) -> None:
        if getattr(self, "_prob", None) is not None:
            self._prob.close()
            self._prob = None

    def __enter__(self):
        return self

    def __exit__(self, *exc) -> None:
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class MatrixFilter(_GpuFilter):
    """Distance-weighted filter of Andreassen et al. (2011), 2-D and 3-D
    (filter/matrix_filter.py:9-99)."""

    _mode = _MODE_MATRIX

    def __init__(self, nelx: int, nely: int, rmin: float, nelz: Union[int, None] = None,
                 pbc: Union[bool, list, np.ndarray] = False, device: int = 0,
                 **kwargs: Any) -> None:
        if np.any(np.asarray(pbc, dtype=bool)):
            raise ValueError("periodic boundary conditions are not supported by the GPU path")
        super().__init__(nelx, nely, rmin, nelz, "matrix", device=device)

    def apply_filter(self, x: np.ndarray) -> np.ndarray:
        """H (x / Hs) (matrix_filter.py:56-73)."""
        return self._apply(x)

    def apply_filter_dx(self, dx_filtered: np.ndarray) -> np.ndarray:
        """H (dx_filtered / Hs) (matrix_filter.py:75-99)."""
        return self._apply(dx_filtered)


class HelmholtzFilter(_GpuFilter):
    """PDE filter of Lazarov and Sigmund (2011) (filter/helmholtz_filter.py:16-131):
    the screened Poisson problem with k = (rmin / (2 sqrt 3))^2 solved on the GPU."""

    _mode = _MODE_HELMHOLTZ

    def __init__(self, nelx: int, nely: int, rmin: float, nelz: Union[int, None] = None,
                 l: np.ndarray = np.array([1.0, 1.0]), device: int = 0, **kwargs: Any) -> None:
        if nelz is not None:
            # assemble_helmholtz_filter raises this for 3-D grids (helmholtz_filter.py:180)
            raise NotImplementedError("3D not yet completely implemented.")
        super().__init__(nelx, nely, rmin, nelz, "helmholtz", l=l, device=device)

    def apply_filter(self, x: np.ndarray) -> np.ndarray:
        """TF^T KF^-1 TF x (helmholtz_filter.py:69-94)."""
        return self._apply(x)

    def apply_filter_dx(self, x_filtered: np.ndarray, dx_filtered: np.ndarray) -> np.ndarray:
        """TF^T KF^-1 TF dx_filtered (helmholtz_filter.py:96-131)."""
        return self._apply(dx_filtered)
