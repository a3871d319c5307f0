"""GPU mirrors of the reference's linear-solve interfaces.

``solve_lin`` keeps the signature and return value of
topoptlab.solve_linsystem.solve_lin (solve_linsystem.py:20-365):
``(solution, factorization, preconditioner)``, solution of shape
(ndof_free, nbc), one column solved after the other, non-convergence ->
RuntimeError("... did not converge ...") (:349-351), unknown names ->
ValueError (:364-365).

Two kinds of operator are accepted:
* a ``StructuredOperator`` (a ``GpuProblem`` and its densities): the
  matrix-free GMG-PCG of the structured grid (solvers "gb300-gmgpcg",
  "gb300-pcg"; the rhs lives on all DOFs, fixed ones ignored);
* an assembled SciPy sparse matrix (the reference's K[free][:, free]):
  Jacobi-preconditioned CG on the GPU in FP64 (solver "gb300-pcg" or any
  reference Krylov name; the direct-solver names use rtol 1e-12).
There is no CPU path.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import _lib
from .log_utils import EmptyLogger

_DIRECT = {"scipy-direct", "scipy-lu", "cvxopt-cholmod"}
_KRYLOV = {"scipy-cg", "scipy-bicg", "scipy-cgs", "scipy-gmres", "scipy-lgmres", "scipy-minres",
           "scipy-qmr", "scipy-tfqmr", "scipy-gcrotmk", "topoptlab-pcg", "topoptlab-cg"}


@dataclass
class StructuredOperator:
    """K(xPhys) of a GpuProblem, applied matrix-free on the GPU."""
    prob: object
    xPhys: np.ndarray

    @property
    def shape(self):
        return (self.prob.ndof, self.prob.ndof)


def _csr_pcg(K, b, x0, rtol, atol, maxiter, jacobi=True, device=0):
    import scipy.sparse as sp
    A = sp.csr_matrix(K)
    A.sort_indices()
    n = A.shape[0]
    indptr = np.ascontiguousarray(A.indptr.astype(np.int64))
    indices = np.ascontiguousarray(A.indices.astype(np.int32))
    data = _lib.f64(A.data)
    bb = _lib.f64(b).reshape(-1)
    x = np.empty(n)
    x0p = None
    if x0 is not None:
        x0a = _lib.f64(x0).reshape(-1)
        x0p = _lib.dptr(x0a)
    info = _lib.TgSolveInfo()
    lib = _lib.load()
    rc = lib.tg_csr_pcg(n, indptr.ctypes.data_as(_lib._i64p), indices.ctypes.data_as(_lib._i32p),
                        _lib.dptr(data), _lib.dptr(bb), x0p, _lib.dptr(x), float(rtol),
                        float(atol), int(maxiter), 1 if jacobi else 0, C.byref(info), device)
    return x, rc, info


def pcg(A, b, P=None, x0=None, rtol=1e-5, atol=0.0, maxiter=100000, logger=EmptyLogger(),
        **kwargs):
    """linear_solvers.pcg on the GPU for an assembled matrix: returns (x, info)
    with info = 0 when converged, the iteration count otherwise.  P is the
    Jacobi preconditioner when it is None or the string "jacobi" (a Python
    preconditioner object cannot run on the GPU)."""
    if P is not None and P != "jacobi":
        raise ValueError("the GPU pcg supports the Jacobi preconditioner only")
    x, rc, info = _csr_pcg(A, b, x0, rtol, atol, maxiter, jacobi=True)
    logger.perf(f"PCGit. {info.iters}")
    if rc == _lib.TG_OK:
        return x, 0
    if rc == _lib.TG_ENOTCONV:
        return x, max(info.iters, 1)
    raise RuntimeError(_lib.load().tg_csr_last_error().decode())


def solve_lin(K, rhs, solver, rhs0=None, solver_kw={}, factorization=None, preconditioner=None,
              preconditioner_kw={}, P=None, logger=EmptyLogger, **kwargs):
    if solver not in _DIRECT and solver not in _KRYLOV and solver not in ("gb300-gmgpcg",
                                                                           "gb300-pcg"):
        raise ValueError("Unknown solver: ", solver)
    rhs = np.asarray(rhs, dtype=np.float64)
    if rhs.ndim == 1:
        rhs = rhs[:, None]
    rtol = float(solver_kw.get("rtol", 1e-12 if solver in _DIRECT else 1e-8))
    maxiter = int(solver_kw.get("maxiter", 100000))
    sol = np.zeros(rhs.shape)
    if isinstance(K, StructuredOperator):
        for i in range(rhs.shape[1]):
            u0 = None if rhs0 is None else np.asarray(rhs0)[:, i]
            u, info = K.prob.solve(K.xPhys, rhs[:, i], u0=u0)
            sol[:, i] = u
        return sol, None, P
    for i in range(rhs.shape[1]):
        x0 = None if rhs0 is None else np.asarray(rhs0)[:, i]
        x, rc, info = _csr_pcg(K, rhs[:, i], x0, rtol, float(solver_kw.get("atol", 0.0)), maxiter)
        if rc == _lib.TG_ENOTCONV:
            raise RuntimeError("pcg iteration did not converge for bc ", i)
        if rc != _lib.TG_OK:
            raise RuntimeError(_lib.load().tg_csr_last_error().decode())
        sol[:, i] = x
    return sol, None, "jacobi"
