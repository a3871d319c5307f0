"""GPU kernels against the CPU oracle, through the C ABI.

Tolerances: index work bit-exact; FP64 kernels within 1e-12 relative of the
oracle (summation order differs); FP32 kernels within 1e-5 relative."""
import numpy as np
import pytest

from oracle import topopt as O
from oracle import gmg as G

pytestmark = pytest.mark.gpu

CASES = [
    # (nelx, nely, nelz, kind)
    (12, 6, None, "elast"), (9, 7, None, "elast"), (10, 6, None, "poisson"),
    (6, 4, 4, "elast"), (5, 3, 4, "elast"), (8, 6, 4, "poisson"), (20, 10, 10, "elast"),
]


def _setup(nelx, nely, nelz, kind, rng, **kw):
    from topoptlab_gb300.context import GpuProblem
    ndim = 2 if nelz is None else 3
    KE = O.ke_elast(ndim) if kind == "elast" else O.ke_poisson(ndim)
    nnd = ndim if kind == "elast" else 1
    dims = (nelx, nely) if ndim == 2 else (nelx, nely, nelz)
    nel = int(np.prod(dims))
    ndof = nnd * int(np.prod(np.array(dims) + 1))
    if kind == "elast" and ndim == 2:
        fixed, f = O.bc_mbb_2d(nelx, nely)
    elif kind == "elast":
        fixed, f = O.bc_cantilever_3d(nelx, nely, nelz)
    else:
        fixed = np.arange(0, nely + 1)
        f = np.full(ndof, 0.01)
    prob = GpuProblem(nelx, nely, nelz, KE, fixed, f, 0.5, 1.5, **kw)
    x = rng.uniform(0.05, 1.0, nel)
    return prob, KE, fixed, f, x, ndof


def test_edofmat_bit_exact(gpu_lib, golden):
    from topoptlab_gb300.elements import create_edofMat
    d = golden("elements.npz")
    for k in d.files:
        if k.startswith("edof2d"):
            _, dims, nd = k.split("_")
            nx, ny = map(int, dims.split("x"))
            np.testing.assert_array_equal(create_edofMat(nx, ny, None, int(nd))[0], d[k])
        elif k.startswith("edof3d"):
            _, dims, nd = k.split("_")
            nx, ny, nz = map(int, dims.split("x"))
            np.testing.assert_array_equal(create_edofMat(nx, ny, nz, int(nd))[0], d[k])
    # a large grid against the oracle
    e, *_ = create_edofMat(40, 20, 10, 3)
    np.testing.assert_array_equal(e, O.edofmat(40, 20, 10, 3))


@pytest.mark.parametrize("nelx,nely,nelz,kind", CASES)
def test_kmul_fp64(gpu_lib, nelx, nely, nelz, kind):
    rng = np.random.default_rng(1)
    prob, KE, fixed, f, x, ndof = _setup(nelx, nely, nelz, kind, rng)
    try:
        u = rng.standard_normal(ndof)
        y = prob.kmul(x, u)
    finally:
        prob.close()
    edof = O.edofmat(nelx, nely, nelz, KE.shape[0] // (4 if nelz is None else 8))
    K = O.assemble(KE, edof, O.simp(x), ndof)
    m = np.ones(ndof)
    m[fixed] = 0.0
    yref = m * (K @ (m * u))
    np.testing.assert_allclose(y, yref, rtol=0, atol=1e-13 * np.abs(yref).max())


@pytest.mark.parametrize("nelx,nely,nelz,kind", CASES[:4])
def test_kmul_fp32(gpu_lib, nelx, nely, nelz, kind):
    rng = np.random.default_rng(2)
    prob, KE, fixed, f, x, ndof = _setup(nelx, nely, nelz, kind, rng, precision="mixed")
    try:
        u = rng.standard_normal(ndof)
        y = prob.kmul(x, u, precision="mixed")
    finally:
        prob.close()
    edof = O.edofmat(nelx, nely, nelz, KE.shape[0] // (4 if nelz is None else 8))
    K = O.assemble(KE, edof, O.simp(x), ndof)
    m = np.ones(ndof)
    m[fixed] = 0.0
    yref = m * (K @ (m * u))
    np.testing.assert_allclose(y, yref, rtol=0, atol=1e-5 * np.abs(yref).max())


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-13), ("mixed", 1e-5)])
@pytest.mark.parametrize("nelx,nely,nelz,kind", [(31, 17, 9, "elast"), (17, 32, 5, "poisson"),
                                                 (60, 60, 30, "elast")])
def test_kmul_3d_multi_tile(gpu_lib, precision, tol, nelx, nely, nelz, kind):
    """3-D grids spanning several node columns in x and y and several z chunks
    (the largest one gives every CTA more than one node plane); the oracle
    product is the element-by-element sum y = sum_e s_e KE u_e."""
    rng = np.random.default_rng(3)
    prob, KE, fixed, f, x, ndof = _setup(nelx, nely, nelz, kind, rng, precision=precision,
                                         precond="gb300-jacobi")
    try:
        u = rng.standard_normal(ndof)
        y = prob.kmul(x, u, precision=precision)
    finally:
        prob.close()
    nnd = KE.shape[0] // 8
    edof = O.edofmat(nelx, nely, nelz, nnd)
    m = np.ones(ndof)
    m[fixed] = 0.0
    ye = ((m * u)[edof] @ KE.T) * O.simp(x)[:, None]
    yref = m * np.bincount(edof.ravel(), ye.ravel(), minlength=ndof)
    np.testing.assert_allclose(y, yref, rtol=0, atol=tol * np.abs(yref).max())


@pytest.mark.parametrize("nelx,nely,nelz,rmin", [(7, 5, None, 2.4), (9, 6, None, 1.5),
                                                 (6, 5, 4, 1.5), (5, 4, 3, 2.4), (60, 20, None, 2.4)])
def test_filter_modes(gpu_lib, nelx, nely, nelz, rmin):
    rng = np.random.default_rng(3)
    ndim = 2 if nelz is None else 3
    prob, KE, fixed, f, x, ndof = _setup(nelx, nely, nelz, "elast", rng)
    prob.close()
    from topoptlab_gb300.context import GpuProblem
    prob = GpuProblem(nelx, nely, nelz, KE, fixed, f, 0.5, rmin)
    try:
        H, Hs = O.filter_matrix(nelx, nely, nelz, rmin)
        d = -rng.uniform(0.1, 1.0, x.shape[0])
        np.testing.assert_allclose(prob.filter(None, 3), Hs, rtol=1e-14)
        np.testing.assert_allclose(prob.filter(x, 0), (H @ x) / Hs, rtol=1e-13)
        np.testing.assert_allclose(prob.filter(d, 1), H @ (d / Hs), rtol=1e-13)
        np.testing.assert_allclose(prob.filter(x, 2, d), (H @ (x * d)) / Hs / np.maximum(0.001, x),
                                   rtol=1e-13)
    finally:
        prob.close()


@pytest.mark.parametrize("nelx,nely,nelz,kind", CASES)
def test_compliance_and_sensitivity(gpu_lib, nelx, nely, nelz, kind):
    rng = np.random.default_rng(4)
    prob, KE, fixed, f, x, ndof = _setup(nelx, nely, nelz, kind, rng)
    try:
        u = rng.standard_normal(ndof)
        u[fixed] = 0.0
        obj, dc = prob.compliance(x, u)
    finally:
        prob.close()
    edof = O.edofmat(nelx, nely, nelz, KE.shape[0] // (4 if nelz is None else 8))
    obj_ref, dc_ref, _ = O.compliance_sens(x, u, KE, edof)
    np.testing.assert_allclose(obj, obj_ref, rtol=1e-12)
    np.testing.assert_allclose(dc, dc_ref, rtol=1e-11, atol=1e-13 * np.abs(dc_ref).max())


@pytest.mark.parametrize("nelx,nely,nelz,kind", [(20, 8, None, "elast"), (12, 6, 4, "elast"),
                                                  (9, 7, None, "poisson")])
def test_objectives_compliance_reference_signature(gpu_lib, nelx, nely, nelz, kind):
    """objectives.compliance called as the reference calls it
    (objectives.py:7-15: no grid sizes, u with one column per load case, the
    SIMP parameters in matinterpol_kw): the grid comes from edofMat, the value
    is the oracle's, a second call reuses the context, and rhs_adj = -u."""
    from topoptlab_gb300 import objectives
    from topoptlab_gb300.material_interpolation import simp
    rng = np.random.default_rng(6)
    ndim = 2 if nelz is None else 3
    KE = O.ke_elast(ndim) if kind == "elast" else O.ke_poisson(ndim)
    nd = KE.shape[0] // (4 if ndim == 2 else 8)
    edof = O.edofmat(nelx, nely, nelz, nd)
    nel = edof.shape[0]
    ndof = nd * int(np.prod(np.array([nelx, nely] + ([nelz] if nelz else [])) + 1))
    x = rng.uniform(0.05, 1.0, nel)
    u = rng.standard_normal((ndof, 2))
    kw = {"eps": 1e-9, "penal": 3.0}
    try:
        for i in (0, 1):
            obj, rhs_adj, self_adj = objectives.compliance(x, u, KE, edof, i, simp, kw, 0.5)
            obj_ref, _, _ = O.compliance_sens(x, u[:, i], KE, edof)
            np.testing.assert_allclose(obj, 0.5 + obj_ref, rtol=1e-12)
            assert self_adj is True
            np.testing.assert_array_equal(rhs_adj, -u)
            assert len(objectives._CTX) == 1
    finally:
        for p in objectives._CTX.values():
            p.close()
        objectives._CTX.clear()


def test_oc_against_reference_steps(gpu_lib, golden):
    from topoptlab_gb300.optimizer import oc_top88
    g = golden("mbb2d_60x20.npz")
    for k in (0, 1, 2, 24, 143):
        xnew, gt = oc_top88(g[f"x_in_{k}"], 0.5, g[f"dc_{k}"], g[f"dv_{k}"], float(g[f"g_in_{k}"]))
        np.testing.assert_allclose(xnew, g[f"x_out_{k}"], atol=1e-13)
        np.testing.assert_allclose(gt, g["g"][k], rtol=1e-9, atol=1e-12)


def test_oc_passive_active_flags(gpu_lib):
    from topoptlab_gb300.optimizer import oc_top88
    rng = np.random.default_rng(5)
    n = 5000
    x = rng.uniform(0.1, 0.9, n)
    dc = -rng.uniform(0.1, 2.0, n)
    dv = np.ones(n)
    flags = rng.integers(0, 3, n).astype(np.int8)
    xnew, gt = oc_top88(x, 0.5, dc, dv, 0.0, el_flags=flags)
    assert np.all(xnew[flags == 1] == 0.0) and np.all(xnew[flags == 2] == 1.0)
    # oracle with the same flag rule (optimality_criterion.py:69-71)
    l1, l2 = 0.0, 1e9
    xr = np.zeros(n)
    while (l2 - l1) / (l1 + l2) > 1e-3:
        lmid = 0.5 * (l2 + l1)
        xr[:] = np.maximum(0.0, np.maximum(x - 0.2, np.minimum(1.0, np.minimum(x + 0.2, x * np.sqrt(-dc / dv / lmid)))))
        xr[flags == 1] = 0
        xr[flags == 2] = 1
        gtr = np.sum(dv * (xr - x))
        if gtr > 0:
            l1 = lmid
        else:
            l2 = lmid
    np.testing.assert_allclose(xnew, xr, atol=1e-13)


def test_oc_barrier_wait_runs_out(gpu_lib):
    """The one in-kernel wait of the library (the grid barrier of the
    one-launch OC bisection) is bounded.  tg_tune makes the next bisection's
    barrier wait for one block more than the grid holds -- an arrival that
    never comes -- so every block polls until its limit (about a second),
    records the error flag and leaves; the call returns TG_ETIMEOUT
    (RuntimeError).  The next call on the same device runs normally."""
    import time
    from topoptlab_gb300 import _lib
    from topoptlab_gb300.optimizer import oc_top88
    lib = _lib.load()
    rng = np.random.default_rng(9)
    n = 5000
    x = rng.uniform(0.1, 0.9, n)
    dc = -rng.uniform(0.1, 2.0, n)
    dv = np.ones(n)
    assert lib.tg_tune(_lib.TG_TUNE_OC_BARRIER_TIMEOUT, 1) == _lib.TG_OK
    t0 = time.perf_counter()
    with pytest.raises(RuntimeError, match="timed out"):
        oc_top88(x, 0.5, dc, dv, 0.0)
    assert time.perf_counter() - t0 < 60.0
    xnew, gt = oc_top88(x, 0.5, dc, dv, 0.0)
    xo, gto, _ = O.oc_top88(x, dc, dv, 0.0)
    np.testing.assert_allclose(xnew, xo, atol=1e-13)
    assert lib.tg_tune(99, 0) == _lib.TG_EINVAL


@pytest.mark.parametrize("nelx,nely,nelz,kind", [(12, 8, None, "elast"), (16, 8, None, "poisson"),
                                                 (8, 4, 4, "elast"), (16, 8, 8, "elast")])
def test_coarse_operators_are_galerkin(gpu_lib, nelx, nely, nelz, kind):
    rng = np.random.default_rng(6)
    prob, KE, fixed, f, x, ndof = _setup(nelx, nely, nelz, kind, rng, nlevels=3)
    ndim = 2 if nelz is None else 3
    dims = (nelx, nely) if ndim == 2 else (nelx, nely, nelz)
    nnd = KE.shape[0] // 2 ** ndim
    edof = O.edofmat(nelx, nely, nelz, nnd)
    K = O.assemble(KE, edof, O.simp(x), ndof)
    mask = np.zeros(ndof, bool)
    mask[fixed] = True
    h = G.Hierarchy(K, mask, dims, nnd, 3)
    try:
        for lvl in (1, 2):
            st = prob.coarse_stencil(x, lvl)
            A = h.A[lvl].toarray()
            Ad = _stencil_to_dense(st, h.dims[lvl], nnd)
            np.testing.assert_allclose(Ad, A, rtol=0, atol=1e-12 * np.abs(A).max())
    finally:
        prob.close()


def _stencil_to_dense(st, dims, nnd):
    ndim = len(dims)
    nn = [d + 1 for d in dims]
    nnodes = int(np.prod(nn))
    ndir = 3 ** ndim
    S = st.reshape(ndir, nnd, nnd, nnodes)
    A = np.zeros((nnodes * nnd, nnodes * nnd))
    for n in range(nnodes):
        y = n % nn[1]
        xx = (n // nn[1]) % nn[0]
        z = n // (nn[1] * nn[0]) if ndim == 3 else 0
        for d in range(ndir):
            dy, dx = d % 3 - 1, (d // 3) % 3 - 1
            dz = d // 9 - 1 if ndim == 3 else 0
            X, Y, Z = xx + dx, y + dy, z + dz
            if not (0 <= X < nn[0] and 0 <= Y < nn[1] and (ndim == 2 or 0 <= Z < nn[2])):
                continue
            m = (Z * nn[0] + X) * nn[1] + Y
            A[n * nnd:(n + 1) * nnd, m * nnd:(m + 1) * nnd] = S[d, :, :, n]
    return A


@pytest.mark.parametrize("nelx,nely,nelz,kind", [(12, 8, None, "elast"), (16, 16, None, "poisson"),
                                                 (8, 4, 4, "elast"), (16, 8, 8, "elast")])
def test_vcycle_matches_oracle(gpu_lib, nelx, nely, nelz, kind):
    rng = np.random.default_rng(7)
    prob, KE, fixed, f, x, ndof = _setup(nelx, nely, nelz, kind, rng, nlevels=3)
    ndim = 2 if nelz is None else 3
    dims = (nelx, nely) if ndim == 2 else (nelx, nely, nelz)
    nnd = KE.shape[0] // 2 ** ndim
    K = O.assemble(KE, O.edofmat(nelx, nely, nelz, nnd), O.simp(x), ndof)
    mask = np.zeros(ndof, bool)
    mask[fixed] = True
    h = G.Hierarchy(K, mask, dims, nnd, 3, omega=0.6, nsmooth=2)
    b = rng.standard_normal(ndof) * ~mask
    try:
        z = prob.vcycle(x, b)
    finally:
        prob.close()
    zr = h.vcycle(b)
    np.testing.assert_allclose(z, zr, rtol=0, atol=1e-10 * np.abs(zr).max())


@pytest.mark.parametrize("n", [37, 300, 1188])
@pytest.mark.parametrize("cond", [1e2, 1e6, 1e9])
def test_dense_inverse_fp64_and_double_word(gpu_lib, n, cond):
    """The coarsest-level inverse (symmetric block sweep) in FP64 and in
    double-word FP32 arithmetic (with and without the look-ahead panel)
    against LAPACK on SPD matrices of a given condition number.  Bound on the largest entry error of the inverse,
    relative to its largest entry: cond * 2^-42 for double-word (about 48
    significant bits), cond * 2^-46 for FP64 (LAPACK's own inverse is off by
    about cond * 2^-53 as well)."""
    import ctypes as C
    from topoptlab_gb300 import _lib
    lib = _lib.load()
    rng = np.random.default_rng(int(n + np.log10(cond)))
    Q, _ = np.linalg.qr(rng.standard_normal((n, n)))
    lam = np.logspace(0, -np.log10(cond), n)
    A = (Q * lam) @ Q.T
    A = 0.5 * (A + A.T)
    ref = np.linalg.inv(A)
    nrm = np.abs(ref).max()
    out = {}
    for mode, bound in ((0, 2.0 ** -46), (1, 2.0 ** -42), (2, 2.0 ** -42)):
        X = np.empty((n, n))
        rc = lib.tg_dense_inverse(_lib.dptr(np.ascontiguousarray(A)), n, _lib.dptr(X), mode, 0)
        assert rc == _lib.TG_OK, lib.tg_last_error(None)
        err = np.abs(X - ref).max() / nrm
        print(f"n={n} cond={cond:.0e} mode={mode} err={err:.3e} err/cond={err / cond:.3e}")
        assert err < cond * bound, (mode, err)
        np.testing.assert_array_equal(X, X.T)
        out[mode] = X
    # the double-word sweep with the next panel formed inside each update
    # launch (mode 1) computes the same values as separate launches (mode 2)
    np.testing.assert_array_equal(out[1], out[2])


@pytest.mark.parametrize("nlevels", [2, 3])
@pytest.mark.parametrize("nelx,nely,nelz,kind", [(16, 8, 8, "elast"), (32, 16, 16, "elast"),
                                                 (24, 16, 8, "poisson"), (8, 124, 4, "poisson")])
def test_stencil_tma_matches_register_path(gpu_lib, nlevels, nelx, nely, nelz, kind):
    """FP32 3-D coarse sweeps with TMA-staged coefficients (every coarse level
    forced onto the large-grid path) compute the same products in the same
    order as the register-path kernel: mixed V-cycles agree bit for bit."""
    from topoptlab_gb300 import _lib
    lib = _lib.load()
    rng = np.random.default_rng(19)
    prob, KE, fixed, f, x, ndof = _setup(nelx, nely, nelz, kind, rng, nlevels=nlevels,
                                         precision="mixed")
    mask = np.zeros(ndof, bool)
    mask[fixed] = True
    b = rng.standard_normal(ndof) * ~mask
    out = {}
    try:
        assert lib.tg_tune(_lib.TG_TUNE_STENCIL_SMALL_PAIRS, 0) == _lib.TG_OK
        for on in (0, 1):
            assert lib.tg_tune(_lib.TG_TUNE_STENCIL_TMA, on) == _lib.TG_OK
            out[on] = prob.vcycle(x, b, precision="mixed")
    finally:
        lib.tg_tune(_lib.TG_TUNE_STENCIL_TMA, 1)
        lib.tg_tune(_lib.TG_TUNE_STENCIL_SMALL_PAIRS, 150000)
        prob.close()
    assert np.abs(out[0]).max() > 0
    np.testing.assert_array_equal(out[1], out[0])


def _vcycle_tail(prob, x, b, precision, mode):
    from topoptlab_gb300 import _lib
    lib = _lib.load()
    assert lib.tg_tune(_lib.TG_TUNE_COARSE_TAIL, mode) == _lib.TG_OK
    try:
        return prob.vcycle(x, b, precision=precision)
    finally:
        lib.tg_tune(_lib.TG_TUNE_COARSE_TAIL, 0)


@pytest.mark.parametrize("mode", [1, 2])
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("nlevels", [3, 4])
@pytest.mark.parametrize("nelx,nely,nelz,kind", [(32, 16, None, "elast"), (32, 32, None, "poisson"),
                                                 (16, 8, 8, "elast"), (16, 16, 8, "poisson")])
def test_coarse_tail_matches_separate_kernels(gpu_lib, mode, precision, nlevels, nelx, nely, nelz,
                                              kind):
    """The V-cycle's bottom two levels as one launch (restriction into the
    last smoothed level, its sweeps, the coarsest dense solve, both
    prolongations), phases separated by a thread-block cluster's barrier
    (mode 1) or a cooperative grid's bounded barrier (mode 2), compute the
    same values in the same order as the separate kernels: the cycles agree
    bit for bit."""
    rng = np.random.default_rng(17)
    prob, KE, fixed, f, x, ndof = _setup(nelx, nely, nelz, kind, rng, nlevels=nlevels,
                                         precision=precision)
    mask = np.zeros(ndof, bool)
    mask[fixed] = True
    b = rng.standard_normal(ndof) * ~mask
    try:
        z_sep = _vcycle_tail(prob, x, b, precision, 0)
        z_tail = _vcycle_tail(prob, x, b, precision, mode)
    finally:
        prob.close()
    assert np.abs(z_sep).max() > 0
    np.testing.assert_array_equal(z_tail, z_sep)


def test_coarse_tail_barrier_wait_runs_out(gpu_lib):
    """The cooperative V-cycle bottom's grid barriers (mode 2) are bounded: tg_tune
    makes the next launch's first barrier wait for one block more than the
    grid holds, every block polls until its limit, the error flag is set and
    the call returns TG_ETIMEOUT (RuntimeError).  The barrier is reset, and
    the next cycle on the same context is the separate kernels' cycle."""
    import time
    from topoptlab_gb300 import _lib
    lib = _lib.load()
    rng = np.random.default_rng(18)
    prob, KE, fixed, f, x, ndof = _setup(16, 8, 8, "elast", rng, nlevels=3)
    mask = np.zeros(ndof, bool)
    mask[fixed] = True
    b = rng.standard_normal(ndof) * ~mask
    try:
        assert lib.tg_tune(_lib.TG_TUNE_COARSE_TAIL, 2) == _lib.TG_OK
        assert lib.tg_tune(_lib.TG_TUNE_TAIL_BARRIER_TIMEOUT, 1) == _lib.TG_OK
        t0 = time.perf_counter()
        with pytest.raises(RuntimeError, match="timed out"):
            prob.vcycle(x, b)
        assert time.perf_counter() - t0 < 60.0
        z = prob.vcycle(x, b)
        z_sep = _vcycle_tail(prob, x, b, "fp64", 0)
    finally:
        lib.tg_tune(_lib.TG_TUNE_TAIL_BARRIER_TIMEOUT, 0)
        lib.tg_tune(_lib.TG_TUNE_COARSE_TAIL, 0)
        prob.close()
    np.testing.assert_array_equal(z, z_sep)


@pytest.mark.parametrize("unsmoothed,nsmooth,nsmooth_coarse",
                         [((1,), 2, 0), ((2,), 2, 0), ((1, 2), 2, 0), ((1,), 1, 2), ((), 1, 3)])
@pytest.mark.parametrize("nelx,nely,nelz,kind", [(32, 16, None, "elast"), (16, 8, 8, "elast"),
                                                 (32, 16, 16, "elast"), (16, 16, 8, "poisson")])
def test_vcycle_unsmoothed_levels_match_oracle(gpu_lib, unsmoothed, nsmooth, nsmooth_coarse,
                                               nelx, nely, nelz, kind):
    """Levels left unsmoothed (tg_problem.unsmoothed): the cycle restricts
    their right-hand side on and prolongates the coarser correction back,
    as the oracle's Hierarchy(unsmoothed=...) does; with nsmooth_coarse, the
    coarse levels take that many sweeps (FP64, 4 levels)."""
    rng = np.random.default_rng(21)
    mask_bits = sum(1 << l for l in unsmoothed)
    prob, KE, fixed, f, x, ndof = _setup(nelx, nely, nelz, kind, rng, nlevels=4,
                                         unsmoothed=mask_bits, nsmooth=nsmooth,
                                         nsmooth_coarse=nsmooth_coarse)
    ndim = 2 if nelz is None else 3
    dims = (nelx, nely) if ndim == 2 else (nelx, nely, nelz)
    nnd = KE.shape[0] // 2 ** ndim
    K = O.assemble(KE, O.edofmat(nelx, nely, nelz, nnd), O.simp(x), ndof)
    mask = np.zeros(ndof, bool)
    mask[fixed] = True
    h = G.Hierarchy(K, mask, dims, nnd, 4, omega=0.6, nsmooth=nsmooth, unsmoothed=unsmoothed,
                    nsmooth_coarse=nsmooth_coarse)
    b = rng.standard_normal(ndof) * ~mask
    try:
        z = prob.vcycle(x, b)
    finally:
        prob.close()
    zr = h.vcycle(b)
    np.testing.assert_allclose(z, zr, rtol=0, atol=1e-10 * np.abs(zr).max())


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_solve_unsmoothed_level1_reaches_direct_solution(gpu_lib, precision):
    """One smoothing sweep (omega 0.6) on the fine level, two on levels 2-3,
    level 1 unsmoothed -- the bench's V-cycle -- still converges to the
    direct solution on a random-density design."""
    rng = np.random.default_rng(22)
    prob, KE, fixed, f, x, ndof = _setup(32, 16, 16, "elast", rng, precision=precision,
                                         rtol=1e-10, nlevels=4, nsmooth=1, omega=0.6,
                                         unsmoothed=2, nsmooth_coarse=2)
    try:
        u, info = prob.solve(x, f)
    finally:
        prob.close()
    assert info["converged"] == 1 and info["rel_res"] < 1e-10
    K = O.assemble(KE, O.edofmat(32, 16, 16, 3), O.simp(x), ndof)
    free = np.setdiff1d(np.arange(ndof), fixed)
    ud = O.solve_direct(K, f, free)
    np.testing.assert_allclose(u, ud, rtol=0, atol=1e-7 * np.abs(ud).max())


def test_unsmoothed_bits_are_checked(gpu_lib):
    rng = np.random.default_rng(23)
    for bits in (1, 1 << 3, 1 << 5):          # the fine level, the coarsest (4 levels), beyond
        with pytest.raises(ValueError, match="unsmoothed"):
            _setup(16, 8, 8, "elast", rng, nlevels=4, unsmoothed=bits)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("nelx,nely,nelz,kind", [(32, 16, None, "elast"), (32, 32, None, "poisson"),
                                                 (16, 8, 8, "elast")])
def test_solve_reaches_direct_solution(gpu_lib, precision, nelx, nely, nelz, kind):
    rng = np.random.default_rng(8)
    prob, KE, fixed, f, x, ndof = _setup(nelx, nely, nelz, kind, rng, precision=precision,
                                         rtol=1e-10)
    try:
        u, info = prob.solve(x, f)
    finally:
        prob.close()
    assert info["converged"] == 1 and info["rel_res"] < 1e-10
    nnd = KE.shape[0] // (4 if nelz is None else 8)
    K = O.assemble(KE, O.edofmat(nelx, nely, nelz, nnd), O.simp(x), ndof)
    free = np.setdiff1d(np.arange(ndof), fixed)
    ud = O.solve_direct(K, f, free)
    np.testing.assert_allclose(u, ud, rtol=0, atol=1e-7 * np.abs(ud).max())
