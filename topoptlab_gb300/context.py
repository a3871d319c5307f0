"""Python handle of one GPU problem context (tg_ctx of libtopopt_gb300.so)."""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import _lib

PRECISIONS = {"fp64": _lib.TG_PREC_FP64, "mixed": _lib.TG_PREC_MIXED}
PRECONDS = {"gb300-gmg": _lib.TG_PRECOND_GMG, "gb300-jacobi": _lib.TG_PRECOND_JACOBI}


@dataclass
class IterResult:
    obj: float
    vol: float
    change: float
    g: float
    rel_res: float
    pcg_iters: int
    vcycles: int
    refinements: int
    oc_steps: int
    fallback: int
    nlevels: int
    t_solve_ms: float
    t_step_ms: float
    warm_ratio: float


# parts of a learned network a problem uses once one is attached
# (tg_problem.learned bits: 1 warm start, 2 coarse-grid correction)
LEARNED_MODES = {"warm_start": _lib.TG_LEARNED_WARM_START,
                 "coarse_correction": _lib.TG_LEARNED_COARSE_CORRECTION,
                 "both": _lib.TG_LEARNED_WARM_START | _lib.TG_LEARNED_COARSE_CORRECTION}


def learned_mask(learned) -> int:
    """False / 0: none chosen (attaching a network then enables the warm
    start); True or "both": 3; "warm_start": 1; "coarse_correction": 2; or
    the bits themselves."""
    if isinstance(learned, str):
        if learned not in LEARNED_MODES:
            raise ValueError(f"Unknown learned mode: {learned}")
        return LEARNED_MODES[learned]
    if isinstance(learned, (bool, np.bool_)):
        return 3 if learned else 0
    v = int(learned)
    if v < 0 or v > 3:
        raise ValueError(f"Unknown learned mode: {learned}")
    return v


class GpuProblem:
    """Owns a tg_ctx: device state of one SIMP compliance problem.

    Arguments mirror what the reference main() derives in its set-up
    (topology_optimization.py:203-409)."""

    def __init__(self, nelx, nely, nelz, KE, fixed, f, volfrac, rmin, ft=1, eps=1e-9,
                 penal=3.0, move=0.2, el_flags=None, precond="gb300-gmg", precision="fp64",
                 nlevels=0, nsmooth=2, omega=0.6, rtol=1e-8, maxiter=2000, inner_rtol=1e-4,
                 learned=False, device=0, filter_mode="matrix", filter_l=None, unsmoothed=0,
                 nsmooth_coarse=0):
        self._lib = _lib.load()
        self.ndim = 2 if nelz is None else 3
        self.nelx, self.nely, self.nelz = nelx, nely, nelz
        self.nel = nelx * nely * (nelz if self.ndim == 3 else 1)
        KE = _lib.f64(KE)
        ne = KE.shape[0]
        if KE.shape != (ne, ne) or ne % (2 ** self.ndim):
            raise ValueError(f"element matrix of shape {KE.shape} does not fit ndim={self.ndim}")
        self.nnode_dof = ne // 2 ** self.ndim
        nn = (nelx + 1) * (nely + 1) * ((nelz + 1) if self.ndim == 3 else 1)
        self.ndof = nn * self.nnode_dof
        # f: (ndof,) or (ndof, nload) -- one column per load case, passed to
        # the library as nload vectors one after another
        f = np.asarray(f, dtype=np.float64)
        if f.ndim == 1:
            f = f[:, None]
        if f.ndim != 2 or f.shape[0] != self.ndof:
            raise ValueError(f"load vector has shape {f.shape}, expected ({self.ndof}, nload)")
        self.nload = f.shape[1]
        f = np.ascontiguousarray(f.T).reshape(-1)
        fixed = np.ascontiguousarray(np.asarray(fixed, dtype=np.int64).reshape(-1))
        if precision not in PRECISIONS:
            raise ValueError(f"Unknown precision: {precision}")
        if precond not in PRECONDS:
            raise ValueError(f"Unknown preconditioner: {precond}")
        self._keep = [KE, fixed, f]
        p = _lib.TgProblem()
        p.ndim, p.nnode_dof = self.ndim, self.nnode_dof
        p.nelx, p.nely, p.nelz = nelx, nely, 0 if nelz is None else nelz
        p.KE = _lib.dptr(KE)
        p.fixed = fixed.ctypes.data_as(_lib._i64p)
        p.nfixed = fixed.shape[0]
        p.f = _lib.dptr(f)
        p.volfrac, p.rmin, p.eps, p.penal, p.move = volfrac, rmin, eps, penal, move
        p.ft = ft
        if el_flags is not None:
            fl = np.ascontiguousarray(np.asarray(el_flags).reshape(-1).astype(np.int8))
            if fl.shape[0] != self.nel:
                raise ValueError("el_flags must have one entry per element")
            self._keep.append(fl)
            p.el_flags = fl.ctypes.data_as(_lib._i8p)
        p.precond = PRECONDS[precond]
        p.precision = PRECISIONS[precision]
        p.nlevels, p.nsmooth, p.omega = nlevels, nsmooth, omega
        p.unsmoothed = int(unsmoothed)
        p.nsmooth_coarse = int(nsmooth_coarse)
        p.rtol, p.maxiter, p.inner_rtol = rtol, maxiter, inner_rtol
        p.learned = learned_mask(learned)
        p.device = device
        p.nload = self.nload
        if filter_mode == "helmholtz":
            # screened Poisson element of the PDE filter (filter/helmholtz_filter.py:188-193)
            from .elements import lk_screened_poisson_2d, lk_screened_poisson_3d
            lkf = lk_screened_poisson_2d if self.ndim == 2 else lk_screened_poisson_3d
            l = np.ones(self.ndim) if filter_l is None else np.asarray(filter_l, dtype=float)
            KF = _lib.f64(lkf(k=(rmin / (2 * np.sqrt(3))) ** 2, l=l))
            self._keep.append(KF)
            p.filter_pde, p.KF = 1, _lib.dptr(KF)
        elif filter_mode not in ("matrix", "convolution"):
            raise ValueError(f"Unknown filter. ft: {ft} filter_mode {filter_mode}")
        h = C.c_void_p()
        rc = self._lib.tg_create(C.byref(p), C.byref(h))
        _lib.check(rc, None, "tg_create")
        self._h = h

    # ------------------------------------------------------------------
    def close(self):
        if getattr(self, "_h", None):
            self._lib.tg_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, rc, what):
        _lib.check(rc, self._h, what)

    def step(self) -> IterResult:
        out = _lib.TgIterOut()
        self._check(self._lib.tg_step(self._h, C.byref(out)), "tg_step")
        return IterResult(*(getattr(out, k) for k, _ in _lib.TgIterOut._fields_))

    def get(self, field: int, out: np.ndarray = None) -> np.ndarray:
        """Element fields: (nel,); u and f: (ndof,) for one load case, else
        (ndof, nload).  `out`: a C-contiguous float64 array of the field's
        size to copy into (for one load case), e.g. page-locked host memory,
        which the device copies into directly."""
        nodes = field in (_lib.TG_FIELD_U, _lib.TG_FIELD_F)
        n = self.ndof * self.nload if nodes else self.nel
        if out is not None:
            if nodes and self.nload > 1:
                raise ValueError("get(out=...) takes one load case")
            if (out.dtype != np.float64 or out.size != n or not out.flags["C_CONTIGUOUS"]
                    or not out.flags["WRITEABLE"]):
                raise ValueError(f"get(out=...) needs a writeable C-contiguous float64 array of {n}")
            a = out.reshape(-1)
        else:
            a = np.empty(n)
        self._check(self._lib.tg_get(self._h, field, _lib.dptr(a), n), "tg_get")
        if out is not None:
            return out
        if nodes and self.nload > 1:
            return np.ascontiguousarray(a.reshape(self.nload, self.ndof).T)
        return a

    def set(self, field: int, values) -> None:
        a = np.asarray(values, dtype=np.float64)
        if a.ndim == 2 and field in (_lib.TG_FIELD_U, _lib.TG_FIELD_F):
            a = a.T                                     # (ndof, nload) -> load cases first
        a = np.ascontiguousarray(a).reshape(-1)
        self._check(self._lib.tg_set(self._h, field, _lib.dptr(a), a.shape[0]), "tg_set")

    # unit entry points -------------------------------------------------
    def kmul(self, xPhys, u, precision="fp64"):
        x = _lib.f64(xPhys).reshape(-1)
        uu = _lib.f64(u).reshape(-1)
        y = np.empty(self.ndof)
        self._check(self._lib.tg_kmul(self._h, _lib.dptr(x), _lib.dptr(uu), _lib.dptr(y),
                                      PRECISIONS[precision]), "tg_kmul")
        return y

    def solve(self, xPhys, rhs, u0=None):
        x = _lib.f64(xPhys).reshape(-1)
        b = _lib.f64(rhs).reshape(-1)
        u = np.empty(self.ndof)
        info = _lib.TgSolveInfo()
        u0p = None
        if u0 is not None:
            u0a = _lib.f64(u0).reshape(-1)
            u0p = _lib.dptr(u0a)
        self._check(self._lib.tg_solve(self._h, _lib.dptr(x), _lib.dptr(b), u0p, _lib.dptr(u),
                                       C.byref(info)), "tg_solve")
        return u, {k: getattr(info, k) for k, _ in _lib.TgSolveInfo._fields_}

    def filter(self, x, mode, d=None):
        xa = _lib.f64(x).reshape(-1) if x is not None else None
        da = _lib.f64(d).reshape(-1) if d is not None else None
        y = np.empty(self.nel)
        self._check(self._lib.tg_filter(self._h, _lib.dptr(xa) if xa is not None else None,
                                        _lib.dptr(da) if da is not None else None,
                                        _lib.dptr(y), mode), "tg_filter")
        return y

    def compliance(self, xPhys, u):
        x = _lib.f64(xPhys).reshape(-1)
        uu = _lib.f64(u).reshape(-1)
        obj = C.c_double()
        dc = np.empty(self.nel)
        self._check(self._lib.tg_compliance(self._h, _lib.dptr(x), _lib.dptr(uu), C.byref(obj),
                                            _lib.dptr(dc)), "tg_compliance")
        return obj.value, dc

    def adjoint(self, u, rhs_adj):
        """Adjoint solve K adj = rhs_adj with the operator of the last state
        solve (step / solve) and the sensitivity simp_dx(xPhys) adj_e^T KE u_e
        of that design (topology_optimization.py:473-500): (adj, dobj, info)."""
        uu = _lib.f64(u).reshape(-1)
        rr = _lib.f64(rhs_adj).reshape(-1)
        adj = np.empty(self.ndof)
        dobj = np.empty(self.nel)
        info = _lib.TgSolveInfo()
        self._check(self._lib.tg_adjoint(self._h, _lib.dptr(uu), _lib.dptr(rr), _lib.dptr(adj),
                                         _lib.dptr(dobj), C.byref(info)), "tg_adjoint")
        return adj, dobj, {k: getattr(info, k) for k, _ in _lib.TgSolveInfo._fields_}

    def vcycle(self, xPhys, b, precision="fp64"):
        x = _lib.f64(xPhys).reshape(-1)
        bb = _lib.f64(b).reshape(-1)
        out = np.empty(self.ndof)
        self._check(self._lib.tg_vcycle(self._h, _lib.dptr(x), _lib.dptr(bb), _lib.dptr(out),
                                        PRECISIONS[precision]), "tg_vcycle")
        return out

    def levels(self):
        n = C.c_int32()
        nd = np.zeros(8, dtype=np.int64)
        self._check(self._lib.tg_levels(self._h, C.byref(n), nd.ctypes.data_as(_lib._i64p)),
                    "tg_levels")
        return n.value, nd[:n.value].tolist()

    def coarse_stencil(self, xPhys, level):
        x = _lib.f64(xPhys).reshape(-1)
        dims = [self.nelx, self.nely] + ([self.nelz] if self.ndim == 3 else [])
        nn = int(np.prod([d // 2 ** level + 1 for d in dims]))
        n = (27 if self.ndim == 3 else 9) * self.nnode_dof ** 2 * nn
        out = np.empty(n)
        self._check(self._lib.tg_coarse_stencil(self._h, _lib.dptr(x), level, _lib.dptr(out), n),
                    "tg_coarse_stencil")
        return out
