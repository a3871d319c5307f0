"""Batches of independent designs stepped together on one GPU.

Each design is its own context (own grid, hierarchy, CUDA stream and CUDA
graphs); ``DesignBatch.step`` runs one design iteration of every design
through ``tg_step_many``, which steps them concurrently from a pool of host
threads, so small designs overlap on the GPU instead of running one after
another.  A design's results are those of stepping it alone.

``heat_plate_batch`` builds the 64-plate heat batch workload: stationary heat-plate
cooling on nelx = nely drawn uniformly from [nmin, nmax] by seed, conductivity
kmin = 1e-3 .. kmax = 1 (SIMP eps = kmin), penal 3, volfrac 0.4, rmin 1.5,
uniform source 0.01 per element, T = 0 sink on the middle 10 % of the left
edge (example_bc.heatplate_2d_element_source).
"""
from __future__ import annotations

import ctypes as C
from typing import List, Sequence

import numpy as np

from . import _lib
from .context import GpuProblem, IterResult


class DesignBatch:
    def __init__(self, problems: Sequence[GpuProblem], nthreads: int = 0):
        self.problems: List[GpuProblem] = list(problems)
        self.nthreads = nthreads
        n = len(self.problems)
        self._handles = (C.c_void_p * n)(*[p._h for p in self.problems])
        self._outs = (_lib.TgIterOut * n)()
        self._rcs = (C.c_int32 * n)()

    def __len__(self):
        return len(self.problems)

    def step(self) -> List[IterResult]:
        lib = _lib.load()
        n = len(self.problems)
        rc = lib.tg_step_many(self._handles, n, self._outs, self._rcs, self.nthreads)
        if rc != _lib.TG_OK:
            for i in range(n):
                if self._rcs[i] != _lib.TG_OK:
                    _lib.check(self._rcs[i], self.problems[i]._h, f"tg_step_many (design {i})")
        return [IterResult(*(getattr(o, k) for k, _ in _lib.TgIterOut._fields_))
                for o in self._outs]

    def close(self):
        for p in self.problems:
            p.close()


def heat_plate_sizes(n_designs: int = 64, seed: int = 0, nmin: int = 64, nmax: int = 512):
    return [int(v) for v in np.random.default_rng(seed).integers(nmin, nmax + 1, n_designs)]


def heat_plate_batch(sizes: Sequence[int], precision: str = "mixed", rtol: float = 1e-8,
                     kmin: float = 1e-3, volfrac: float = 0.4, rmin: float = 1.5,
                     penal: float = 3.0, ft: int = 1, device: int = 0, nthreads: int = 0):
    from .elements import lk_poisson_2d
    from .example_bc import heatplate_2d_element_source
    KE = lk_poisson_2d()
    probs = []
    try:
        for n in sizes:
            ndof = (n + 1) * (n + 1)
            _, f, fixed, _, _ = heatplate_2d_element_source(n, n, ndof)
            probs.append(GpuProblem(n, n, None, KE, fixed, f[:, 0], volfrac, rmin, ft=ft,
                                    eps=kmin, penal=penal, precision=precision, rtol=rtol,
                                    device=device))
    except Exception:
        for p in probs:
            p.close()
        raise
    return DesignBatch(probs, nthreads=nthreads)
