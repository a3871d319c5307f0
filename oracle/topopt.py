"""NumPy/SciPy restatement of the reference SIMP loop (test infrastructure only).

Every function cites the reference file:line it follows (paths relative to the
topoptlab project root).  Nothing here is optimised; it is the checker.
"""
from __future__ import annotations

import numpy as np
import scipy.sparse as sp
import scipy.sparse.linalg as spla


# --------------------------------------------------------------------------
# element DOF maps   (elements/bilinear_quadrilateral.py:7-48,
#                     elements/trilinear_hexahedron.py:7-58)
# --------------------------------------------------------------------------
# local node order of the reference elements as (dx, dy[, dz]) offsets from
# the element's lowest-index node n1 = (ex, ey[, ez]); y grows downward.
CORNERS_2D = [(0, 1), (1, 1), (1, 0), (0, 0)]
CORNERS_3D = [(0, 1, 0), (1, 1, 0), (1, 0, 0), (0, 0, 0),
              (0, 1, 1), (1, 1, 1), (1, 0, 1), (0, 0, 1)]


def node_id(x, y, z, nelx, nely):
    """Node numbering: y fastest, then x, then z."""
    return (nelx + 1) * (nely + 1) * z + (nely + 1) * x + y


def edofmat(nelx, nely, nelz=None, ndof=1):
    """Element DOF matrix, element index = ez*nelx*nely + ex*nely + ey."""
    if nelz is None:
        out = np.zeros((nelx * nely, 4 * ndof), dtype=np.int32)
        for ex in range(nelx):
            for ey in range(nely):
                e = ex * nely + ey
                for k, (dx, dy) in enumerate(CORNERS_2D):
                    n = node_id(ex + dx, ey + dy, 0, nelx, nely)
                    out[e, k * ndof:(k + 1) * ndof] = n * ndof + np.arange(ndof)
        return out
    out = np.zeros((nelx * nely * nelz, 8 * ndof), dtype=np.int32)
    for ez in range(nelz):
        for ex in range(nelx):
            for ey in range(nely):
                e = ez * nelx * nely + ex * nely + ey
                for k, (dx, dy, dz) in enumerate(CORNERS_3D):
                    n = node_id(ex + dx, ey + dy, ez + dz, nelx, nely)
                    out[e, k * ndof:(k + 1) * ndof] = n * ndof + np.arange(ndof)
    return out


def edofmat_vec(nelx, nely, nelz=None, ndof=1):
    """edofmat with the elements vectorised, as the reference builds it
    (elements/bilinear_quadrilateral.py:7-48, trilinear_hexahedron.py:7-58):
    the same matrix, for grids where the per-element loop is too slow."""
    corners = CORNERS_2D if nelz is None else CORNERS_3D
    nz = 1 if nelz is None else nelz
    e = np.arange(nelx * nely * nz, dtype=np.int64)
    ez, rest = np.divmod(e, nelx * nely)
    ex, ey = np.divmod(rest, nely)
    out = np.empty((e.size, len(corners) * ndof), dtype=np.int32)
    for k, c in enumerate(corners):
        dz = c[2] if nelz is not None else 0
        n = node_id(ex + c[0], ey + c[1], ez + dz, nelx, nely)
        for d in range(ndof):
            out[:, k * ndof + d] = n * ndof + d
    return out


# --------------------------------------------------------------------------
# element matrices by 3-point Gauss quadrature (exact for these elements)
# (elements/linear_elasticity_2d.py:69-229 plane stress,
#  elements/linear_elasticity_3d.py:65-666, elements/poisson_2d.py:68-96,
#  elements/poisson_3d.py:62-147)
# --------------------------------------------------------------------------
_GP = np.array([-np.sqrt(0.6), 0.0, np.sqrt(0.6)])
_GW = np.array([5.0, 8.0, 5.0]) / 9.0


def _shape_grad(corners, xi):
    """d N_k / d xi_a for multilinear shape functions on [-1,1]^d."""
    nd = len(xi)
    g = np.zeros((len(corners), nd))
    for k, c in enumerate(corners):
        s = [2 * ci - 1 for ci in c]          # corner sign
        for a in range(nd):
            v = 0.5 * s[a]
            for b in range(nd):
                if b != a:
                    v *= 0.5 * (1 + s[b] * xi[b])
            g[k, a] = v
    return g


def _integrate(corners, l, fn):
    nd = len(l)
    nn = len(corners)
    acc = None
    for idx in np.ndindex(*(3,) * nd):
        xi = np.array([_GP[i] for i in idx])
        w = np.prod([_GW[i] for i in idx])
        # reference cell [-1,1]^d -> [0,l]^d: dx/dxi = l/2
        dN = _shape_grad(corners, xi) / (np.asarray(l) / 2.0)[None, :]
        detJ = np.prod(np.asarray(l) / 2.0)
        v = fn(dN) * w * detJ
        acc = v if acc is None else acc + v
    return acc


def _phys_corners(ndim):
    """Physical corner positions (y upward) of the reference local nodes."""
    cs = CORNERS_2D if ndim == 2 else CORNERS_3D
    return [(c[0], 1 - c[1]) + tuple(c[2:]) for c in cs]


def ke_poisson(ndim, k=1.0, l=None):
    l = np.ones(ndim) if l is None else np.asarray(l, float)
    corners = _phys_corners(ndim)
    return k * _integrate(corners, l, lambda dN: dN @ dN.T)


def _shape(corners, xi):
    """N_k(xi) for multilinear shape functions on [-1,1]^d."""
    return np.array([np.prod([0.5 * (1 + (2 * ci - 1) * xi[a]) for a, ci in enumerate(c)])
                     for c in corners])


def ke_mass(ndim, rho=1.0, l=None):
    """Consistent scalar mass matrix rho * int N N^T (elements/mass_scalar_2d.py:68-110,
    mass_scalar_3d.py), 3-point Gauss rule per axis (exact for the product)."""
    l = np.ones(ndim) if l is None else np.asarray(l, float)
    corners = _phys_corners(ndim)
    acc = np.zeros((len(corners), len(corners)))
    for idx in np.ndindex(*(3,) * ndim):
        xi = np.array([_GP[i] for i in idx])
        w = np.prod([_GW[i] for i in idx])
        N = _shape(corners, xi)
        acc += np.outer(N, N) * w * np.prod(l / 2.0)
    return rho * acc


def ke_screened_poisson(ndim, k=1.0, l=None):
    """k * Laplacian + mass (elements/screenedpoisson_2d.py:8-37, screenedpoisson_3d.py:9-40)."""
    return ke_poisson(ndim, k, l) + ke_mass(ndim, 1.0, l)


def _elastic_D(ndim, E, nu):
    if ndim == 2:   # plane stress
        return E / (1 - nu ** 2) * np.array([[1, nu, 0], [nu, 1, 0], [0, 0, (1 - nu) / 2]])
    # The reference's closed-form hexahedron matrix
    # (elements/linear_elasticity_3d.py:65-666) equals B^T D B integrated with
    # the normal-stress block of isotropic elasticity but a shear stiffness of
    # C11/2 = E(1-nu)/(2(1+nu)(1-2nu)) instead of mu = E/(2(1+nu)); a least
    # squares fit of D to the reference matrix reproduces it to 1e-31.  The
    # oracle restates that matrix as it is.
    c11 = E * (1 - nu) / ((1 + nu) * (1 - 2 * nu))
    c12 = E * nu / ((1 + nu) * (1 - 2 * nu))
    D = np.full((6, 6), 0.0)
    D[:3, :3] = c12
    D[np.arange(3), np.arange(3)] = c11
    D[np.arange(3, 6), np.arange(3, 6)] = c11 / 2
    return D


def _bmat(dN, ndim):
    nn = dN.shape[0]
    if ndim == 2:
        B = np.zeros((3, 2 * nn))
        for k in range(nn):
            B[0, 2 * k] = dN[k, 0]
            B[1, 2 * k + 1] = dN[k, 1]
            B[2, 2 * k] = dN[k, 1]
            B[2, 2 * k + 1] = dN[k, 0]
        return B
    B = np.zeros((6, 3 * nn))
    for k in range(nn):
        x, y, z = dN[k]
        B[0, 3 * k] = x
        B[1, 3 * k + 1] = y
        B[2, 3 * k + 2] = z
        B[3, 3 * k + 1], B[3, 3 * k + 2] = z, y      # yz
        B[4, 3 * k], B[4, 3 * k + 2] = z, x          # xz
        B[5, 3 * k], B[5, 3 * k + 1] = y, x          # xy
    return B


def ke_elast(ndim, E=1.0, nu=0.3, l=None):
    l = np.ones(ndim) if l is None else np.asarray(l, float)
    corners = _phys_corners(ndim)
    D = _elastic_D(ndim, E, nu)

    def f(dN):
        B = _bmat(dN, ndim)
        return B.T @ D @ B
    return _integrate(corners, l, f)


# --------------------------------------------------------------------------
# SIMP (material_interpolation.py:6-62)
# --------------------------------------------------------------------------
def simp(x, eps=1e-9, penal=3.0):
    return eps + (1 - eps) * x ** penal


def simp_dx(x, eps=1e-9, penal=3.0):
    return penal * (1 - eps) * x ** (penal - 1)


# --------------------------------------------------------------------------
# distance filter (filter/matrix_filter.py:101-232)
# --------------------------------------------------------------------------
def filter_matrix(nelx, nely, nelz, rmin):
    """H with weights max(0, rmin - r) over offsets |d_i| <= ceil(rmin)-1,
    element index ez*nelx*nely + ex*nely + ey; Hs = row sums."""
    ndim = 2 if nelz is None else 3
    dims = (nelx, nely) if ndim == 2 else (nelx, nely, nelz)
    R = int(np.ceil(rmin)) - 1
    rows, cols, vals = [], [], []
    nel = int(np.prod(dims))
    for e in range(nel):
        if ndim == 2:
            ex, ey = divmod(e, nely)
            c = (ex, ey)
        else:
            ez, rest = divmod(e, nelx * nely)
            ex, ey = divmod(rest, nely)
            c = (ex, ey, ez)
        for off in np.ndindex(*(2 * R + 1,) * ndim):
            d = [o - R for o in off]
            nb = [c[i] + d[i] for i in range(ndim)]
            if any(nb[i] < 0 or nb[i] >= dims[i] for i in range(ndim)):
                continue
            w = max(0.0, rmin - float(np.sqrt(sum(di * di for di in d))))
            j = nb[0] * nely + nb[1] + (nb[2] * nelx * nely if ndim == 3 else 0)
            rows.append(e)
            cols.append(j)
            vals.append(w)
    H = sp.csr_matrix((vals, (rows, cols)), shape=(nel, nel))
    Hs = np.asarray(H.sum(1)).ravel()
    return H, Hs


def filter_matrix_vec(nelx, nely, nelz, rmin):
    """filter_matrix with the loop over offsets only, all elements of an
    offset at once (the reference builds H the same way,
    filter/matrix_filter.py:170-231): the same entries, explicit zero
    weights included, for grids where the per-element loop is too slow."""
    ndim = 2 if nelz is None else 3
    dims = (nelx, nely) if ndim == 2 else (nelx, nely, nelz)
    R = int(np.ceil(rmin)) - 1
    nel = int(np.prod(dims))
    e = np.arange(nel, dtype=np.int64)
    if ndim == 2:
        ex, ey = np.divmod(e, nely)
        c = (ex, ey)
    else:
        ez, rest = np.divmod(e, nelx * nely)
        ex, ey = np.divmod(rest, nely)
        c = (ex, ey, ez)
    rows, cols, vals = [], [], []
    for off in np.ndindex(*(2 * R + 1,) * ndim):
        d = [o - R for o in off]
        w = max(0.0, rmin - float(np.sqrt(sum(di * di for di in d))))
        nb = [c[i] + d[i] for i in range(ndim)]
        ok = np.ones(nel, dtype=bool)
        for i in range(ndim):
            ok &= (nb[i] >= 0) & (nb[i] < dims[i])
        j = nb[0] * nely + nb[1] + (nb[2] * nelx * nely if ndim == 3 else 0)
        rows.append(e[ok])
        cols.append(j[ok])
        vals.append(np.full(int(ok.sum()), w))
    H = sp.csr_matrix((np.concatenate(vals), (np.concatenate(rows), np.concatenate(cols))),
                      shape=(nel, nel))
    Hs = np.asarray(H.sum(1)).ravel()
    return H, Hs


# --------------------------------------------------------------------------
# objective + sensitivity (objectives.py:51-55, topology_optimization.py:491-500)
# --------------------------------------------------------------------------
# --------------------------------------------------------------------------
# Helmholtz PDE filter (filter/helmholtz_filter.py:133-200; applied as in
# topology_optimization.py:554-555, 568-570, 646-647)
# --------------------------------------------------------------------------
def helmholtz_operators(nelx, nely, nelz, rmin, l=None):
    """KF (screened Poisson matrix, k = (rmin / (2 sqrt 3))^2, no boundary
    conditions) and TF (element -> node averaging, 1/2^d per element node).
    Returns (solve, TF) with solve a factorised KF."""
    ndim = 2 if nelz is None else 3
    KE = ke_screened_poisson(ndim, (rmin / (2 * np.sqrt(3))) ** 2, l)
    edof = edofmat(nelx, nely, nelz, 1)
    nel = edof.shape[0]
    nnodes = int(np.prod(np.array([nelx, nely] + ([nelz] if ndim == 3 else [])) + 1))
    KF = assemble(KE, edof, np.ones(nel), nnodes).tocsc()
    nper = edof.shape[1]
    TF = sp.coo_matrix((np.full(nel * nper, 1.0 / nper),
                        (edof.ravel(), np.repeat(np.arange(nel), nper))),
                       shape=(nnodes, nel)).tocsr()
    return spla.factorized(KF), TF


def helmholtz_apply(solve, TF, x):
    """x_filtered = TF^T KF^-1 TF x."""
    return TF.T @ solve(TF @ x)


def compliance_sens(xPhys, u, KE, edof, eps=1e-9, penal=3.0):
    ue = u[edof]
    ce = np.einsum("ei,ij,ej->e", ue, KE, ue)
    obj = float((simp(xPhys, eps, penal) * ce).sum())
    dc = -simp_dx(xPhys, eps, penal) * ce
    return obj, dc, ce


# --------------------------------------------------------------------------
# OC update (optimizer/optimality_criterion.py:9-79)
# --------------------------------------------------------------------------
def oc_top88(x, dc, dv, g, move=0.2, l1=0.0, l2=1e9, el_flags=None):
    """optimizer/optimality_criterion.py:59-79: passive elements (flag 1)
    set to 0 and active ones (flag 2) to 1 before each volume sum."""
    xnew = np.zeros_like(x)
    gt = g
    nsteps = 0
    while (l2 - l1) / (l1 + l2) > 1e-3:
        lmid = 0.5 * (l2 + l1)
        xnew[:] = np.maximum(0.0, np.maximum(
            x - move, np.minimum(1.0, np.minimum(x + move, x * np.sqrt(-dc / dv / lmid)))))
        if el_flags is not None:
            xnew[el_flags == 1] = 0.0
            xnew[el_flags == 2] = 1.0
        gt = g + np.sum(dv * (xnew - x))
        if gt > 0:
            l1 = lmid
        else:
            l2 = lmid
        nsteps += 1
    return xnew, gt, nsteps


# --------------------------------------------------------------------------
# assembly + direct solve (fem.py:141-237, solve_linsystem.py:83-87)
# --------------------------------------------------------------------------
def assemble(KE, edof, scale, ndof):
    n = edof.shape[1]
    iK = np.repeat(edof, n, axis=1).ravel()
    jK = np.tile(edof, (1, n)).ravel()
    sK = (KE[None, :, :] * scale[:, None, None]).ravel()
    return sp.coo_matrix((sK, (iK, jK)), shape=(ndof, ndof)).tocsr()


def solve_direct(K, f, free):
    u = np.zeros(K.shape[0])
    Kff = K[free][:, free].tocsc()
    u[free] = spla.spsolve(Kff, f[free])
    return u


# --------------------------------------------------------------------------
# the design loop (topology_optimization.py:411-673; OC, ft in {0, 1})
# --------------------------------------------------------------------------
def run(nelx, nely, nelz, volfrac, rmin, ft, KE, fixed, f, eps=1e-9, penal=3.0,
        nouteriter=2000, solve=None, record=(), filter_mode="matrix", el_flags=None):
    """Return dict with obj/vol/change per iteration, final x, xPhys, u.

    ``solve(K, f, free, u_prev) -> u`` defaults to the direct solve.
    ``filter_mode`` "helmholtz" replaces the distance filter by the PDE filter."""
    ndim = 2 if nelz is None else 3
    dims = (nelx, nely) if ndim == 2 else (nelx, nely, nelz)
    nel = int(np.prod(dims))
    nnode_dof = KE.shape[0] // 2 ** ndim
    ndof = nnode_dof * int(np.prod(np.array(dims) + 1))
    edof = edofmat(nelx, nely, nelz, nnode_dof)
    H, Hs = filter_matrix(nelx, nely, nelz, rmin)
    if filter_mode == "helmholtz":
        hsolve, TF = helmholtz_operators(nelx, nely, nelz, rmin)
        pde = lambda v: helmholtz_apply(hsolve, TF, v)   # noqa: E731
    free = np.setdiff1d(np.arange(ndof), fixed)
    x = volfrac * np.ones(nel)
    xPhys = x.copy()
    xold = x.copy()
    g = 0.0
    u = np.zeros(ndof)
    out = {"obj": [], "vol": [], "change": [], "g": [], "oc_steps": [], "rec": {}}
    solve = solve or (lambda K, f, free, u0: solve_direct(K, f, free))
    # several load cases (f with columns): one solve each, compliance and
    # sensitivities summed over the cases (topology_optimization.py:446-500)
    fcols = f[:, None] if f.ndim == 1 else f
    ucols = np.zeros(fcols.shape)
    for loop in range(nouteriter):
        K = assemble(KE, edof, simp(xPhys, eps, penal), ndof)
        obj, dc = 0.0, np.zeros(nel)
        for i in range(fcols.shape[1]):
            ucols[:, i] = solve(K, fcols[:, i], free, ucols[:, i])
            o_i, dc_i, ce = compliance_sens(xPhys, ucols[:, i], KE, edof, eps, penal)
            obj += o_i
            dc += dc_i
        u = ucols[:, 0] if f.ndim == 1 else ucols.copy()
        dv = np.ones(nel)
        if filter_mode == "helmholtz" and ft == 0:
            dc = pde(dc * xPhys) / np.maximum(0.001, x)
        elif filter_mode == "helmholtz" and ft == 1:
            dc = pde(dc)
            dv = pde(dv)
        elif ft == 0:
            dc = np.asarray(H @ (x * dc)) / Hs / np.maximum(0.001, x)
        elif ft == 1:
            dc = np.asarray(H @ (dc / Hs))
            dv = np.asarray(H @ (dv / Hs))
        if loop in record:
            out["rec"][loop] = dict(xPhys=xPhys.copy(), u=u.copy(), dc=dc.copy(),
                                    dv=dv.copy(), x=x.copy(), g=g)
        xold = x.copy()
        x, g, nsteps = oc_top88(x, dc, dv, g, el_flags=el_flags)
        if ft == 1 and filter_mode == "helmholtz":
            xPhys = pde(x)
        elif ft == 1:
            xPhys = np.asarray(H @ x) / Hs
        else:
            xPhys = x.copy()
        change = float(np.abs(x - xold).max())
        out["obj"].append(obj)
        out["vol"].append(float(xPhys.mean()))
        out["change"].append(change)
        out["g"].append(g)
        out["oc_steps"].append(nsteps)
        if change < 0.01:
            break
    out.update(x=x, xPhys=xPhys, u=u, final_obj=out["obj"][-1])
    return out


# --------------------------------------------------------------------------
# boundary-condition callables (example_bc/lin_elast.py:6-46, :274-338,
# example_bc/heat_conduction.py:5-49)
# --------------------------------------------------------------------------
def bc_mbb_2d(nelx, nely):
    ndof = 2 * (nelx + 1) * (nely + 1)
    fixed = np.union1d(np.arange(0, 2 * (nely + 1), 2), [ndof - 1])
    f = np.zeros(ndof)
    f[1] = -1.0
    return fixed, f


def bc_cantilever_2d(nelx, nely):
    """example_bc/lin_elast.py:100-139: left wall clamped, downward unit load
    on the last DOF (the y-DOF of the bottom-right node)."""
    ndof = 2 * (nelx + 1) * (nely + 1)
    fixed = np.arange(0, 2 * (nely + 1))
    f = np.zeros(ndof)
    f[-1] = -1.0
    return fixed, f


def bc_cantilever_2d_twoloads(nelx, nely):
    """example_bc/lin_elast.py:141-182: left wall clamped; case 0 downward unit
    load on the last DOF, case 1 upward unit load on the y-DOF of node
    nelx*(nely+1)."""
    ndof = 2 * (nelx + 1) * (nely + 1)
    fixed = np.arange(0, 2 * (nely + 1))
    f = np.zeros((ndof, 2))
    f[-1, 0] = -1.0
    f[2 * nelx * (nely + 1) + 1, 1] = 1.0
    return fixed, f


def bc_cantilever_3d(nelx, nely, nelz, force_mode="linear"):
    nn = (nelx + 1) * (nely + 1) * (nelz + 1)
    ndof = 3 * nn
    fixed = []
    for z in range(nelz + 1):
        for y in range(nely + 1):
            n = node_id(0, y, z, nelx, nely)
            fixed += [3 * n, 3 * n + 1, 3 * n + 2]
    for x in range(nelx + 1):
        for y in range(nely + 1):
            fixed.append(3 * node_id(x, y, 0, nelx, nely) + 2)
    fixed = np.unique(np.array(fixed))
    f = np.zeros(ndof)
    load = -np.linspace(1.0, 0.0, nelz + 1) if force_mode == "linear" else -np.ones(nelz + 1)
    for z in range(nelz + 1):
        f[3 * node_id(nelx, nely, z, nelx, nely) + 1] = load[z]
    return fixed, f


def bc_heatplate_2d(nelx, nely):
    ndof = (nelx + 1) * (nely + 1)
    f = np.full(ndof, 0.01)
    fixed = np.arange(int(nely / 2 - nely / 20), int(nely / 2 + 1 + nely / 20))
    return fixed, f
