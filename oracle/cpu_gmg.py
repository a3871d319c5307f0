"""CPU FP64 geometric-multigrid PCG for 3-D hex8 elasticity at full size
(test infrastructure and the CPU baseline of the benchmark; never part of the
GPU library).

The algorithm of oracle/gmg.py -- PCG (linear_solvers.py:114-134, stopping at
||r|| < rtol ||b||) preconditioned by a V-cycle with nsmooth damped-Jacobi
sweeps (omega 0.6) before and after, zero initial guess per level, Galerkin
coarse operators Pt^T A Pt of the trilinear interpolation from the stride-2
nodes (gmg.py:148-189) masked on both sides, and an exact coarsest solve --
with the fine level matrix-free and every coarse level built element by
element and applied as a 27-point block stencil, by the OpenMP kernels of
oracle/cgmg.c.  The level count follows the GPU library's rule: coarsen while
the element counts are even and the level has more than 1200 DOFs.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "cgmg.c")
LIB = os.path.join(HERE, "libcgmg.so")

_dp = C.POINTER(C.c_double)
_u8p = C.POINTER(C.c_uint8)
_lib = None


def build(force: bool = False) -> str:
    """Compile cgmg.c with gcc and OpenMP (in place, next to the source)."""
    if force or not os.path.exists(LIB) or os.path.getmtime(LIB) < os.path.getmtime(SRC):
        tmp = LIB + ".tmp"
        subprocess.run(["gcc", "-O3", "-fopenmp", "-shared", "-fPIC", SRC, "-o", tmp], check=True)
        os.replace(tmp, LIB)
    return LIB


def _load():
    global _lib
    if _lib is None:
        lib = C.CDLL(build())
        i, d = C.c_int, C.c_double
        sig = {
            "hex8_apply": [i, i, i, _dp, _dp, _u8p, _dp, _dp, _dp, _dp, d, i, _dp],
            "hex8_dinv": [i, i, i, _dp, _dp, _u8p, _dp],
            "hex8_galerkin1": [i, i, i, _dp, _dp, _u8p, _u8p, _dp],
            "elem_galerkin": [i, i, i, _dp, _u8p, _dp],
            "elem_to_stencil": [i, i, i, _dp, _dp],
            "stencil_apply": [i, i, i, _dp, _dp, _dp, _dp, _dp, d, i],
            "stencil_dinv": [i, i, i, _dp, _dp],
            "prolong_add": [i, i, i, _u8p, _u8p, _dp, _dp],
            "restrict_": [i, i, i, _u8p, _u8p, _dp, _dp],
            "hex8_ce": [i, i, i, _dp, _dp, _dp],
            "vec_dot": [C.c_int64, _dp, _dp],
            "vec_axpby": [C.c_int64, d, _dp, d, _dp],
            "vec_scale_mul": [C.c_int64, d, _dp, _dp, _dp],
            "dense_matvec": [C.c_int64, _dp, _dp, _dp],
        }
        for name, args in sig.items():
            fn = getattr(lib, name)
            fn.argtypes = args
            fn.restype = C.c_double if name == "vec_dot" else None
        lib.cgmg_threads.argtypes = []
        lib.cgmg_threads.restype = C.c_int
        _lib = lib
    return _lib


def threads() -> int:
    """OpenMP threads of the CPU kernels (all host cores unless OMP_NUM_THREADS says otherwise)."""
    return int(_load().cgmg_threads())


def _p(a):
    return a.ctypes.data_as(_u8p if a.dtype == np.uint8 else _dp)


def node_masks(fixed, nnodes):
    """Per node: bit c set when DOF 3 node + c is fixed."""
    m = np.zeros(nnodes, dtype=np.uint8)
    fixed = np.asarray(fixed, dtype=np.int64)
    np.bitwise_or.at(m, fixed // 3, (1 << (fixed % 3)).astype(np.uint8))
    return m


def coarse_masks(m, dims):
    """Coarse node fixed components = those of the coincident fine node."""
    nx, ny, nz = dims
    return np.ascontiguousarray(m.reshape(nz + 1, nx + 1, ny + 1)[::2, ::2, ::2].ravel())


class CpuGmgSolver:
    def __init__(self, nelx, nely, nelz, KE, fixed, nlevels=0, omega=0.6, nsmooth=2):
        self.lib = _load()
        self.KE = np.ascontiguousarray(KE, dtype=np.float64)
        self.omega, self.nsmooth = omega, nsmooth
        dims = [(nelx, nely, nelz)]
        while True:
            nx, ny, nz = dims[-1]
            ndofs = 3 * (nx + 1) * (ny + 1) * (nz + 1)
            even = nx % 2 == 0 and ny % 2 == 0 and nz % 2 == 0 and min(nx, ny, nz) >= 2
            if not even or (nlevels > 0 and len(dims) >= nlevels) or \
                    (nlevels <= 0 and ndofs <= 1200):
                break
            dims.append((nx // 2, ny // 2, nz // 2))
        self.dims = dims
        self.L = len(dims)
        nn = [int(np.prod(np.array(d) + 1)) for d in dims]
        self.fix = [node_masks(fixed, nn[0])]
        for lvl in range(1, self.L):
            self.fix.append(coarse_masks(self.fix[-1], dims[lvl - 1]))
        self.n = [3 * v for v in nn]
        self.dinv = [np.zeros(k) for k in self.n]
        self.S = [None] + [np.zeros(243 * v) for v in nn[1:]]
        self.ae = [None] + [np.zeros(int(np.prod(d)) * 576) for d in dims[1:]]
        self.x = [np.zeros(k) for k in self.n]
        self.t = [np.zeros(k) for k in self.n]
        self.r = [np.zeros(k) for k in self.n]
        self.b = [np.zeros(k) for k in self.n]
        self.work = np.zeros(self.n[0])
        self.s = None

    def set_density(self, s):
        """Scale factors simp(xPhys): fine diagonal, coarse operators, coarsest inverse."""
        lib = self.lib
        self.s = np.ascontiguousarray(s, dtype=np.float64)
        d0 = self.dims[0]
        lib.hex8_dinv(*d0, _p(self.KE), _p(self.s), _p(self.fix[0]), _p(self.dinv[0]))
        for lvl in range(1, self.L):
            d = self.dims[lvl - 1]
            if lvl == 1:
                lib.hex8_galerkin1(*d, _p(self.KE), _p(self.s), _p(self.fix[0]), _p(self.fix[1]),
                                   _p(self.ae[1]))
            else:
                lib.elem_galerkin(*d, _p(self.ae[lvl - 1]), _p(self.fix[lvl]), _p(self.ae[lvl]))
            lib.elem_to_stencil(*self.dims[lvl], _p(self.ae[lvl]), _p(self.S[lvl]))
            lib.stencil_dinv(*self.dims[lvl], _p(self.S[lvl]), _p(self.dinv[lvl]))
        # coarsest: dense inverse (fixed DOFs: identity rows, then zeroed)
        lc = self.L - 1
        n = self.n[lc]
        if lc == 0:
            A = np.zeros((n, n))
            e = np.zeros(n)
            for j in range(n):
                e[:] = 0.0
                e[j] = 1.0
                col = np.zeros(n)
                lib.hex8_apply(*d0, _p(self.KE), _p(self.s), _p(self.fix[0]), _p(e), _p(col),
                               None, None, 0.0, 0, _p(self.work))
                A[:, j] = col
        else:
            A = np.zeros((n, n))
            e = np.zeros(n)
            col = np.zeros(n)
            for j in range(n):
                e[:] = 0.0
                e[j] = 1.0
                lib.stencil_apply(*self.dims[lc], _p(self.S[lc]), _p(e), _p(col), None, None,
                                  0.0, 0)
                A[:, j] = col
        fixed = np.repeat(self.fix[lc][:, None], 3, axis=1)
        fixed = ((fixed >> np.arange(3)) & 1).astype(bool).ravel()
        A[fixed, :] = 0.0
        A[:, fixed] = 0.0
        A[fixed, fixed] = 1.0
        self.Ac_inv = np.linalg.inv(A)
        self.Ac_inv[fixed, :] = 0.0
        self.Ac_inv[:, fixed] = 0.0
        self.Ac_inv = np.ascontiguousarray(self.Ac_inv)

    def _apply(self, lvl, u, y, b=None, mode=0):
        lib = self.lib
        bp = _p(b) if b is not None else None
        if lvl == 0:
            lib.hex8_apply(*self.dims[0], _p(self.KE), _p(self.s), _p(self.fix[0]), _p(u), _p(y),
                           bp, _p(self.dinv[0]), self.omega, mode, _p(self.work))
        else:
            lib.stencil_apply(*self.dims[lvl], _p(self.S[lvl]), _p(u), _p(y), bp,
                              _p(self.dinv[lvl]), self.omega, mode)

    def vcycle(self, b, x, lvl=0):
        """x = V(b) (zero initial guess)."""
        lib = self.lib
        if lvl == self.L - 1:
            lib.dense_matvec(self.n[lvl], _p(self.Ac_inv), _p(b), _p(x))
            return
        n = self.n[lvl]
        bufs = [x, self.t[lvl]]
        cur = 1
        lib.vec_scale_mul(n, self.omega, _p(self.dinv[lvl]), _p(b), _p(bufs[cur]))
        for _ in range(1, self.nsmooth):
            self._apply(lvl, bufs[cur], bufs[1 - cur], b, 2)
            cur = 1 - cur
        self._apply(lvl, bufs[cur], self.r[lvl], b, 1)
        lib.restrict_(*self.dims[lvl], _p(self.fix[lvl]), _p(self.fix[lvl + 1]), _p(self.r[lvl]),
                      _p(self.b[lvl + 1]))
        self.vcycle(self.b[lvl + 1], self.x[lvl + 1], lvl + 1)
        lib.prolong_add(*self.dims[lvl], _p(self.fix[lvl]), _p(self.fix[lvl + 1]),
                        _p(self.x[lvl + 1]), _p(bufs[cur]))
        for _ in range(self.nsmooth):
            self._apply(lvl, bufs[cur], bufs[1 - cur], b, 2)
            cur = 1 - cur
        if bufs[cur] is not x:
            x[:] = bufs[cur]

    def solve(self, f, u0=None, rtol=1e-8, maxiter=2000):
        """PCG (linear_solvers.py:114-134) for M K M u = M f from u0; returns
        (u, iterations, true relative residual)."""
        lib = self.lib
        n = self.n[0]
        fm = np.ascontiguousarray(f, dtype=np.float64).copy()
        fixed = ((np.repeat(self.fix[0][:, None], 3, axis=1) >> np.arange(3)) & 1).astype(bool).ravel()
        fm[fixed] = 0.0
        u = np.zeros(n) if u0 is None else np.ascontiguousarray(u0, dtype=np.float64).copy()
        u[fixed] = 0.0
        r = np.empty(n)
        self._apply(0, u, r, fm, 1)
        bnorm = np.sqrt(lib.vec_dot(n, _p(fm), _p(fm)))
        tol = rtol * bnorm
        z, p, q = np.zeros(n), np.zeros(n), np.empty(n)
        rho_old = 0.0
        it = 0
        while np.sqrt(lib.vec_dot(n, _p(r), _p(r))) >= tol and it < maxiter:
            self.vcycle(r, z)
            rho = lib.vec_dot(n, _p(r), _p(z))
            if it == 0:
                p[:] = z
            else:
                lib.vec_axpby(n, 1.0, _p(z), rho / rho_old, _p(p))
            self._apply(0, p, q, None, 0)
            alpha = rho / lib.vec_dot(n, _p(p), _p(q))
            lib.vec_axpby(n, alpha, _p(p), 1.0, _p(u))
            lib.vec_axpby(n, -alpha, _p(q), 1.0, _p(r))
            rho_old = rho
            it += 1
        self._apply(0, u, r, fm, 1)
        relres = np.sqrt(lib.vec_dot(n, _p(r), _p(r))) / bnorm if bnorm > 0 else 0.0
        return u, it, relres

    def element_compliance(self, u):
        ce = np.empty(int(np.prod(self.dims[0])))
        self.lib.hex8_ce(*self.dims[0], _p(self.KE), _p(np.ascontiguousarray(u)), _p(ce))
        return ce


def density_filter_3d(nelx, nely, nelz, rmin):
    """The distance filter (filter/matrix_filter.py:101-232) as shifted adds on
    the (nelz, nelx, nely) element array: apply(v) = H v; Hs = H 1."""
    R = int(np.ceil(rmin)) - 1
    taps = []
    for dz in range(-R, R + 1):
        for dx in range(-R, R + 1):
            for dy in range(-R, R + 1):
                w = max(0.0, rmin - float(np.sqrt(dx * dx + dy * dy + dz * dz)))
                if w > 0:
                    taps.append((dz, dx, dy, w))
    shape = (nelz, nelx, nely)

    def apply(v):
        a = v.reshape(shape)
        out = np.zeros(shape)
        for dz, dx, dy, w in taps:
            dst = tuple(slice(max(0, -d), n - max(0, d)) for d, n in zip((dz, dx, dy), shape))
            src = tuple(slice(max(0, d), n - max(0, -d)) for d, n in zip((dz, dx, dy), shape))
            out[dst] += w * a[src]
        return out.ravel()

    return apply, apply(np.ones(int(np.prod(shape))))


class CpuDesignLoop:
    """The design iteration of the reference loop (topology_optimization.py:
    411-673: SIMP scaling, solve, compliance + sensitivities, sensitivity and
    density filter ft=1, OC, change) on the host cores, with the CPU FP64
    GMG-PCG above as the solver (warm-started from the previous displacement)
    and the OC update of oracle/topopt.py."""

    def __init__(self, nelx, nely, nelz, KE, fixed, f, volfrac, rmin, rtol=1e-8, eps=1e-9,
                 penal=3.0):
        from . import topopt as O
        self.O = O
        self.solver = CpuGmgSolver(nelx, nely, nelz, KE, fixed)
        self.f = np.ascontiguousarray(f, dtype=np.float64)
        self.filt, self.Hs = density_filter_3d(nelx, nely, nelz, rmin)
        nel = nelx * nely * nelz
        self.x = np.full(nel, float(volfrac))
        self.xPhys = self.x.copy()
        self.u = np.zeros(self.f.shape[0])
        self.g = 0.0
        self.dv = self.filt(np.ones(nel) / self.Hs)
        self.rtol, self.eps, self.penal = rtol, eps, penal

    def step(self):
        O = self.O
        self.solver.set_density(O.simp(self.xPhys, self.eps, self.penal))
        self.u, its, rel = self.solver.solve(self.f, self.u, rtol=self.rtol)
        ce = self.solver.element_compliance(self.u)
        obj = float((O.simp(self.xPhys, self.eps, self.penal) * ce).sum())
        dc = -O.simp_dx(self.xPhys, self.eps, self.penal) * ce
        dc = self.filt(dc / self.Hs)
        xold = self.x
        self.x, self.g, _ = O.oc_top88(self.x, dc, self.dv, self.g)
        self.xPhys = self.filt(self.x) / self.Hs
        change = float(np.abs(self.x - xold).max())
        return {"obj": obj, "pcg_iters": its, "rel_res": rel, "change": change}
