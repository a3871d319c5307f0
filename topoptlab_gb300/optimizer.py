"""oc_top88 on the GPU (optimizer/optimality_criterion.py:9-79).

The bisection on the Lagrange multiplier runs as one launch per step with the
interval update done on the device (no host round trip per step)."""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib


def oc_top88(x, volfrac, dc, dv, g, el_flags=None, move=0.2, l1=0.0, l2=1e9, device=0):
    """Return (xnew, gt) exactly as the reference OC update."""
    xa = _lib.f64(x).reshape(-1)
    dca = _lib.f64(dc).reshape(-1)
    dva = _lib.f64(dv).reshape(-1)
    n = xa.shape[0]
    xnew = np.empty(n)
    gt = C.c_double()
    nsteps = C.c_int32()
    flp = None
    if el_flags is not None:
        fl = np.ascontiguousarray(np.asarray(el_flags).reshape(-1).astype(np.int8))
        flp = fl.ctypes.data_as(_lib._i8p)
    lib = _lib.load()
    rc = lib.tg_oc_raw(n, _lib.dptr(xa), _lib.dptr(dca), _lib.dptr(dva), float(g), flp,
                       float(move), float(l1), float(l2), _lib.dptr(xnew), C.byref(gt),
                       C.byref(nsteps), device)
    _lib.check(rc, None, "tg_oc_raw")
    return xnew.reshape(np.shape(x)), gt.value
