"""The CPU FP64 multigrid used as the benchmark's CPU baseline
(oracle/cpu_gmg.py, OpenMP kernels in oracle/cgmg.c) against the oracle's
assembled statement of the same algorithm (oracle/gmg.py) and the direct
solve.  CPU only."""
import numpy as np
import pytest

from oracle import topopt as O
from oracle import gmg as G
from oracle import cpu_gmg as CG


@pytest.mark.parametrize("dims,nlevels", [((8, 4, 4), 3), ((16, 8, 8), 3), ((12, 8, 4), 2)])
def test_vcycle_matches_assembled_oracle(dims, nlevels):
    nx, ny, nz = dims
    rng = np.random.default_rng(3)
    KE = O.ke_elast(3)
    x = rng.uniform(0.05, 1.0, nx * ny * nz)
    fixed, f = O.bc_cantilever_3d(nx, ny, nz)
    ndof = f.shape[0]
    K = O.assemble(KE, O.edofmat(nx, ny, nz, 3), O.simp(x), ndof)
    mask = np.zeros(ndof, bool)
    mask[fixed] = True
    h = G.Hierarchy(K, mask, dims, 3, nlevels)
    cs = CG.CpuGmgSolver(nx, ny, nz, KE, fixed, nlevels=nlevels)
    assert cs.L == nlevels
    cs.set_density(O.simp(x))
    b = rng.standard_normal(ndof) * ~mask
    z = np.zeros(ndof)
    cs.vcycle(b, z)
    zr = h.vcycle(b)
    np.testing.assert_allclose(z, zr, rtol=0, atol=1e-11 * np.abs(zr).max())
    # the operator itself
    y = np.zeros(ndof)
    cs._apply(0, b, y, None, 0)
    np.testing.assert_allclose(y, h.A[0] @ b, rtol=0, atol=1e-12 * np.abs(y).max())


def test_solve_matches_direct_and_levels_follow_the_gpu_rule():
    nx, ny, nz = 16, 8, 8
    rng = np.random.default_rng(4)
    KE = O.ke_elast(3)
    x = rng.uniform(0.05, 1.0, nx * ny * nz)
    fixed, f = O.bc_cantilever_3d(nx, ny, nz)
    cs = CG.CpuGmgSolver(nx, ny, nz, KE, fixed)
    assert cs.L == 2                       # 4131 DOFs -> 675 DOFs (<= 1200)
    s = O.simp(x)
    cs.set_density(s)
    u, it, rel = cs.solve(f, rtol=1e-10)
    assert it > 0 and rel < 1e-10
    K = O.assemble(KE, O.edofmat(nx, ny, nz, 3), s, f.shape[0])
    ud = O.solve_direct(K, f, np.setdiff1d(np.arange(f.shape[0]), fixed))
    np.testing.assert_allclose(u, ud, rtol=0, atol=1e-8 * np.abs(ud).max())
    _, _, ce = O.compliance_sens(x, ud, KE, O.edofmat(nx, ny, nz, 3))
    np.testing.assert_allclose(cs.element_compliance(ud), ce, rtol=0, atol=1e-12 * np.abs(ce).max())


def test_shifted_filter_equals_matrix_filter():
    nx, ny, nz, rmin = 9, 6, 5, 1.5
    apply, hs = CG.density_filter_3d(nx, ny, nz, rmin)
    H, Hs = O.filter_matrix(nx, ny, nz, rmin)
    v = np.random.default_rng(5).uniform(size=nx * ny * nz)
    np.testing.assert_allclose(apply(v), H @ v, rtol=1e-14)
    np.testing.assert_allclose(hs, Hs, rtol=1e-14)


@pytest.mark.parametrize("unsmoothed,nsmooth,nsmooth_coarse", [((1,), 1, 2), ((1, 2), 2, 0),
                                                                ((), 1, 3)])
def test_oracle_vcycle_variants_are_spd_preconditioners(unsmoothed, nsmooth, nsmooth_coarse):
    """The oracle's V-cycle with unsmoothed levels and a separate coarse sweep
    count (the GPU context's tg_problem.unsmoothed / nsmooth_coarse, which
    the GPU tests compare against it) is a symmetric positive definite
    operator, so PCG with it converges to the direct solution."""
    nx, ny, nz = 16, 8, 8
    rng = np.random.default_rng(5)
    KE = O.ke_elast(3)
    x = rng.uniform(0.05, 1.0, nx * ny * nz)
    fixed, f = O.bc_cantilever_3d(nx, ny, nz)
    ndof = f.shape[0]
    K = O.assemble(KE, O.edofmat(nx, ny, nz, 3), O.simp(x), ndof)
    mask = np.zeros(ndof, bool)
    mask[fixed] = True
    h = G.Hierarchy(K, mask, (nx, ny, nz), 3, 4, omega=0.6, nsmooth=nsmooth,
                    unsmoothed=unsmoothed, nsmooth_coarse=nsmooth_coarse)
    b1 = rng.standard_normal(ndof) * ~mask
    b2 = rng.standard_normal(ndof) * ~mask
    z1, z2 = h.vcycle(b1), h.vcycle(b2)
    assert abs(z1 @ b2 - z2 @ b1) <= 1e-10 * abs(z1 @ b2)
    assert z1 @ b1 > 0 and z2 @ b2 > 0
    A = h.A[0]
    u, it = G.pcg(A, f * ~mask, h.vcycle, rtol=1e-10, maxiter=500)
    assert it < 500
    free = np.setdiff1d(np.arange(ndof), fixed)
    ud = O.solve_direct(K, f, free)
    np.testing.assert_allclose(u, ud, rtol=0, atol=1e-7 * np.abs(ud).max())
