"""Compliance objective (objectives.py:7-55).

``compliance`` keeps the reference signature so driver code that passes
``obj_func=compliance`` selects the GPU's fused compliance + sensitivity
kernel; called directly it evaluates on the GPU for structured grids whose
size it infers from ``edofMat`` and the element matrix."""
from __future__ import annotations

import numpy as np


def compliance(xPhys, u, KE, edofMat, i, matinterpol, matinterpol_kw, obj, **kwargs):
    """obj += sum simp(xPhys) u_e^T KE u_e ; returns (obj, -u, True).

    ``nelx``, ``nely`` (and ``nelz`` in 3-D) must be passed as keywords."""
    from .context import GpuProblem
    nelx, nely, nelz = kwargs["nelx"], kwargs["nely"], kwargs.get("nelz")
    KE = np.asarray(KE, dtype=np.float64)
    ndof = u.shape[0]
    prob = GpuProblem(nelx, nely, nelz, KE, np.zeros(0, np.int64), np.zeros(ndof), 0.5, 1.5,
                      precond="gb300-jacobi", eps=matinterpol_kw.get("eps", 1e-9),
                      penal=matinterpol_kw.get("penal", 3.0))
    try:
        val, _ = prob.compliance(np.asarray(xPhys).reshape(-1), np.asarray(u)[:, i])
    finally:
        prob.close()
    return obj + val, -u, True
