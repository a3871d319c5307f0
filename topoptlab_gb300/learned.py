"""Learned warm start for the GPU solver (no counterpart in the reference).

A 3-level 3-D convolutional encoder-decoder (16/32/64 channels, FP32) on the
multigrid level-1 node grid predicts a displacement correction y from the
filtered density, the previous displacement and its residual restricted to
the level-1 grid.  With w = P y the warm start of each solve is the
energy-optimal combination ``c1 u_prev + c2 w``; optionally w also deflates
the mixed solver's FP32 PCG (the coarse-grid correction, ``learned=
"coarse_correction"`` or ``"both"`` on the problem).  The learned start is
kept only when the residual after the solve's first cycle is below the plain
warm start's (otherwise the step falls back to plain PCG from the previous
displacement and reports ``fallback = 1``).  Training data are (features,
displacement change) pairs recorded around solver steps of any context with
the same grids (or given by the caller, ``fit``); training runs on the GPU
with the library's own kernels (forward, backward, Adam).
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib
from .context import GpuProblem

_fp = C.POINTER(C.c_float)


class LearnedWarmStart:
    def __init__(self, prob: GpuProblem, capacity: int = 256, seed: int = 0):
        self._lib = _lib.load()
        self.prob = prob
        h = C.c_void_p()
        _lib.check(self._lib.tg_cnn_create(prob._h, capacity, seed, C.byref(h)), prob._h,
                   "tg_cnn_create")
        self._h = h

    def close(self):
        if getattr(self, "_h", None):
            self._lib.tg_cnn_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, rc, what):
        _lib.check(rc, self.prob._h, what)

    # ------------------------------------------------------------------
    def info(self):
        n = C.c_int64()
        dims = (C.c_int32 * 3)()
        ns = C.c_int32()
        self._check(self._lib.tg_cnn_info(self._h, C.byref(n), dims, C.byref(ns)), "tg_cnn_info")
        return {"nparams": n.value, "grid": tuple(dims), "nsamples": ns.value}

    def record_step(self, prob: GpuProblem | None = None):
        """One design iteration of ``prob`` recorded as a training pair."""
        prob = prob or self.prob
        self._check(self._lib.tg_cnn_record_begin(self._h, prob._h), "tg_cnn_record_begin")
        it = prob.step()
        self._check(self._lib.tg_cnn_record_end(self._h, prob._h), "tg_cnn_record_end")
        return it

    def train(self, epochs: int = 20, lr: float = 1e-3, seed: int = 0) -> float:
        loss = C.c_double()
        self._check(self._lib.tg_cnn_train(self._h, epochs, lr, seed, C.byref(loss)), "tg_cnn_train")
        return loss.value

    def fit(self, x0s, targets, epochs: int = 1, lr: float = 1e-3, seed: int = 0) -> float:
        """Adam over caller-provided pairs: x0s (n, nodes, 7), targets (n, nodes, 3)."""
        g = self.info()["grid"]
        nn = g[0] * g[1] * g[2]
        x = np.ascontiguousarray(np.asarray(x0s, dtype=np.float32).reshape(-1, nn, 7))
        t = np.ascontiguousarray(np.asarray(targets, dtype=np.float32).reshape(-1, nn, 3))
        if x.shape[0] != t.shape[0]:
            raise ValueError("fit: as many targets as feature sets are needed")
        loss = C.c_double()
        self._check(self._lib.tg_cnn_fit(self._h, x.shape[0], x.ctypes.data_as(_fp),
                                         t.ctypes.data_as(_fp), epochs, lr, seed, C.byref(loss)),
                    "tg_cnn_fit")
        return loss.value

    def attach(self, prob: GpuProblem | None = None, on: bool = True):
        prob = prob or self.prob
        self._check(self._lib.tg_cnn_attach(prob._h, self._h if on else None), "tg_cnn_attach")

    def params(self) -> np.ndarray:
        n = self.info()["nparams"]
        a = np.empty(n, dtype=np.float32)
        self._check(self._lib.tg_cnn_params(self._h, 0, a.ctypes.data_as(_fp), n), "tg_cnn_params")
        return a

    def set_params(self, values) -> None:
        a = np.ascontiguousarray(np.asarray(values, dtype=np.float32).reshape(-1))
        self._check(self._lib.tg_cnn_params(self._h, 1, a.ctypes.data_as(_fp), a.shape[0]),
                    "tg_cnn_params")

    def eval(self, x0, target=None):
        """Forward (and, with a target, loss + parameter gradient) on host features."""
        g = self.info()["grid"]
        nn = g[0] * g[1] * g[2]
        x = np.ascontiguousarray(np.asarray(x0, dtype=np.float32).reshape(nn, 7))
        y = np.empty((nn, 3), dtype=np.float32)
        loss = C.c_double()
        grads = None
        tp = None
        if target is not None:
            t = np.ascontiguousarray(np.asarray(target, dtype=np.float32).reshape(nn, 3))
            tp = t.ctypes.data_as(_fp)
            grads = np.empty(self.info()["nparams"], dtype=np.float32)
        self._check(self._lib.tg_cnn_eval(self._h, x.ctypes.data_as(_fp), tp, y.ctypes.data_as(_fp),
                                          C.byref(loss),
                                          grads.ctypes.data_as(_fp) if grads is not None else None),
                    "tg_cnn_eval")
        return (y, loss.value, grads) if target is not None else y

    def infer(self, x0):
        """Forward pass as the warm start runs it (single TF32 products)."""
        g = self.info()["grid"]
        nn = g[0] * g[1] * g[2]
        x = np.ascontiguousarray(np.asarray(x0, dtype=np.float32).reshape(nn, 7))
        y = np.empty((nn, 3), dtype=np.float32)
        self._check(self._lib.tg_cnn_infer(self._h, x.ctypes.data_as(_fp), y.ctypes.data_as(_fp)),
                    "tg_cnn_infer")
        return y


def layer_spec():
    """(cin, cout) of the six convolutions, in parameter order; each layer's
    parameters are W[27][cin][cout] (tap k = (dz+1)*9 + (dx+1)*3 + (dy+1))
    followed by b[cout]."""
    return [(7, 16), (16, 32), (32, 64), (64, 32), (32, 16), (16, 3)]
