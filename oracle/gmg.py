"""FP64 geometric-multigrid PCG restatement (test infrastructure only).

The reference ships a V-cycle skeleton (multigrid.py:89-154), a damped-Jacobi
smoother (linear_solvers.py:306-372), a PCG (linear_solvers.py:50-136) and a
stride-2 coarse-node selection (gmg.py:148-189), but its geometric
interpolator (gmg.py:34-146) raises on every grid and solve_lin never wires a
multigrid preconditioner (solve_linsystem.py:136).  This module is the CPU
statement of the multigrid the GPU library builds in their place:

* operators live on all DOFs with Dirichlet rows/columns zeroed:
  A_0 = M_0 K M_0  (M = diagonal 0/1 mask of free DOFs);
* prolongation P is the trilinear (bilinear) interpolation from the stride-2
  coarse nodes (the nodes create_coarse_inds selects), applied per DOF
  component, with masks on both sides: Pt = M_l P M_{l+1};
* coarse DOF fixed  <=>  the coincident fine DOF is fixed;
* Galerkin coarse operators A_{l+1} = Pt^T A_l Pt;
* V-cycle with zero initial guess on every level, nu damped-Jacobi sweeps
  before and after the coarse correction, exact coarsest solve;
* PCG exactly as linear_solvers.py:114-134 with ||r||_2 < rtol*||b||_2.

The mixed-precision cycle of the GPU library (FP32 arithmetic, BF16 element
scale factors in the fine-level smoother, coarse levels built from FP32 scale
factors, coarsest inverse in FP64) is stated here with exact FP64 arithmetic
on the same rounded inputs (round_bf16 / round_f32 of simp(x), K_build):
what remains between the two is the FP32 rounding of the arithmetic.
"""
from __future__ import annotations

import numpy as np
import scipy.sparse as sp


def _interp_1d(nf):
    """(nf+1) x (nf//2+1) linear interpolation between stride-2 nodes."""
    nc = nf // 2
    rows, cols, vals = [], [], []
    for i in range(nf + 1):
        if i % 2 == 0:
            rows.append(i), cols.append(i // 2), vals.append(1.0)
        else:
            rows += [i, i]
            cols += [i // 2, i // 2 + 1]
            vals += [0.5, 0.5]
    return sp.csr_matrix((vals, (rows, cols)), shape=(nf + 1, nc + 1))


def prolongation(dims, ndof):
    """P: coarse nodal vector -> fine nodal vector.  Node order y fastest,
    then x, then z; DOF = node*ndof + c.  dims = (nelx, nely[, nelz])."""
    Px = _interp_1d(dims[0])
    Py = _interp_1d(dims[1])
    P = sp.kron(Px, Py)                       # node index x*(ny+1)+y
    if len(dims) == 3:
        P = sp.kron(_interp_1d(dims[2]), P)   # z slowest
    return sp.kron(P, sp.identity(ndof)).tocsr()


def coarse_fixed_mask(fixed_mask, dims, ndof):
    """Coarse DOF fixed iff its coincident fine DOF is fixed."""
    nn = [d + 1 for d in dims]
    m = fixed_mask.reshape(([nn[2]] if len(dims) == 3 else []) + [nn[0], nn[1], ndof])
    if len(dims) == 3:
        return m[::2, ::2, ::2, :].ravel().copy()
    return m[::2, ::2, :].ravel().copy()


def round_bf16(a):
    """Round FP64 values to the nearest BF16 value (8 significant bits,
    ties to even), the rounding of a direct FP64 -> BF16 conversion."""
    a = np.asarray(a, dtype=np.float64)
    m, e = np.frexp(a)
    return np.ldexp(np.rint(m * 256.0) / 256.0, e)


def round_f32(a):
    return np.asarray(a, dtype=np.float32).astype(np.float64)


class Hierarchy:
    """K: the fine-level operator of the smoother and residual.  K_build (if
    given): the fine operator from which the level-1 Galerkin product is
    formed instead of K -- the mixed-precision cycle smooths with BF16
    densities on the fine level but builds the coarse levels from FP32
    densities.  coarse_ops (if given): the operators of levels 1, 2, ...
    themselves, used in place of the Galerkin products.  unsmoothed: levels
    (0 < l < nlevels - 1) the V-cycle does not smooth: their right-hand side
    is restricted on as it is and the coarser correction prolongated back
    (the GPU context's tg_problem.unsmoothed bits)."""

    def __init__(self, K, fixed_mask, dims, ndof, nlevels, omega=0.6, nsmooth=2, K_build=None,
                 coarse_ops=None, unsmoothed=(), nsmooth_coarse=None):
        self.omega, self.nsmooth = omega, nsmooth
        self.nsmooth_coarse = nsmooth if not nsmooth_coarse else nsmooth_coarse
        self.unsmoothed = set(unsmoothed)
        free = (~fixed_mask).astype(float)
        M = sp.diags(free)
        self.A = [(M @ K @ M).tocsr()]
        self.mask = [fixed_mask]
        self.P = []
        self.dims = [tuple(dims)]
        d = tuple(dims)
        Ab = self.A[0] if K_build is None else (M @ K_build @ M).tocsr()
        for _ in range(nlevels - 1):
            P = prolongation(d, ndof)
            cmask = coarse_fixed_mask(self.mask[-1], d, ndof)
            Pt = sp.diags((~self.mask[-1]).astype(float)) @ P @ sp.diags((~cmask).astype(float))
            Pt = Pt.tocsr()
            self.P.append(Pt)
            self.A.append((Pt.T @ Ab @ Pt).tocsr())
            Ab = self.A[-1]
            self.mask.append(cmask)
            d = tuple(x // 2 for x in d)
            self.dims.append(d)
        if coarse_ops is not None:
            # given operators of levels 1.. (e.g. ones built elsewhere in lower
            # precision) replace the Galerkin products
            for lvl, A in enumerate(coarse_ops, start=1):
                self.A[lvl] = sp.csr_matrix(A)
        self.Dinv = []
        for A, m in zip(self.A, self.mask):
            dg = A.diagonal().copy()
            inv = np.zeros_like(dg)
            inv[~m] = 1.0 / dg[~m]
            self.Dinv.append(inv)
        Ac = self.A[-1].toarray()
        mc = self.mask[-1]
        Ac[mc, mc] = 1.0
        self.Ac_inv = np.linalg.inv(Ac)
        self.Ac_inv[mc, :] = 0.0
        self.Ac_inv[:, mc] = 0.0

    def vcycle(self, b, lvl=0):
        if lvl == len(self.A) - 1:
            return self.Ac_inv @ b
        if lvl in self.unsmoothed:
            return self.P[lvl] @ self.vcycle(self.P[lvl].T @ b, lvl + 1)
        A, Dinv, w = self.A[lvl], self.Dinv[lvl], self.omega
        ns = self.nsmooth if lvl == 0 else self.nsmooth_coarse
        x = w * Dinv * b
        for _ in range(ns - 1):
            x = x + w * Dinv * (b - A @ x)
        r = b - A @ x
        xc = self.vcycle(self.P[lvl].T @ r, lvl + 1)
        x = x + self.P[lvl] @ xc
        for _ in range(ns):
            x = x + w * Dinv * (b - A @ x)
        return x


def pcg(A, b, precond, x0=None, rtol=1e-8, maxiter=10000):
    """linear_solvers.py:50-136 with conv. criterion res_norm (:31-48)."""
    x = np.zeros_like(b) if x0 is None else x0.copy()
    atol = rtol * np.linalg.norm(b)
    r = b - A @ x
    p = np.zeros_like(b)
    rho_prev = None
    for i in range(maxiter):
        if np.linalg.norm(r) < atol:
            return x, i
        z = precond(r)
        rho = r @ z
        p = z.copy() if i == 0 else p * (rho / rho_prev) + z
        q = A @ p
        alpha = rho / (p @ q)
        x += alpha * p
        r -= alpha * q
        rho_prev = rho
    return x, -1


def stencil_matrix(S, dims, ndof):
    """Sparse matrix of an assembled 27-point (9-point in 2-D) block stencil in
    the GPU library's expanded layout S[dir][ci][cj][node] (dir: dy fastest,
    then dx, then dz, each in {-1, 0, 1}), on the node grid of a level with
    element counts dims."""
    ndim = len(dims)
    nn = [d + 1 for d in dims]
    nnodes = int(np.prod(nn))
    nd = 27 if ndim == 3 else 9
    S = np.asarray(S).reshape(nd, ndof, ndof, nnodes)
    n = np.arange(nnodes)
    Y = n % nn[1]
    X = (n // nn[1]) % nn[0]
    Z = n // (nn[0] * nn[1]) if ndim == 3 else np.zeros_like(n)
    rows, cols, vals = [], [], []
    for d in range(nd):
        dy, dx = d % 3 - 1, (d // 3) % 3 - 1
        dz = d // 9 - 1 if ndim == 3 else 0
        ok = (X + dx >= 0) & (X + dx < nn[0]) & (Y + dy >= 0) & (Y + dy < nn[1])
        if ndim == 3:
            ok &= (Z + dz >= 0) & (Z + dz < nn[2])
        src = n[ok]
        m = ((Z[ok] + dz) * nn[0] + X[ok] + dx) * nn[1] + Y[ok] + dy
        for ci in range(ndof):
            for cj in range(ndof):
                rows.append(src * ndof + ci)
                cols.append(m * ndof + cj)
                vals.append(S[d, ci, cj, ok])
    rows, cols, vals = np.concatenate(rows), np.concatenate(cols), np.concatenate(vals)
    keep = vals != 0.0
    return sp.csr_matrix((vals[keep], (rows[keep], cols[keep])), shape=(nnodes * ndof,) * 2)
