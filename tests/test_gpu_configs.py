"""The named 3-D workloads at full size.  The reference's direct solve is
infeasible there, so each design iteration is checked through properties that
need no reference run: the true FP64 residual of every solve, the multigrid
hierarchy that was asked for, and the compliance of two independent solvers
(plain FP64 GMG-PCG and the mixed-precision solver) on the same designs."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_cantilever_128x64x64_plain_fp64_4_levels(gpu_lib):
    """128x64x64 hex8 cantilever (524,288 elements, 1,635,075 DOFs), E=1,
    nu=0.3, volfrac 0.12, penal 3, rmin 1.5, density filter, OC; the x=0 face
    clamped (plus the z=0 symmetry plane of the reference's cantilever_3d);
    a unit total downward load spread evenly over the bottom edge line of the
    x=nelx face.  Plain FP64 matrix-free GMG-PCG with 4 levels and 2 damped
    Jacobi sweeps (omega 0.6), relative residual 1e-8."""
    from topoptlab_gb300.context import GpuProblem
    from topoptlab_gb300.elements import lk_linear_elast_3d
    from topoptlab_gb300.example_bc import cantilever_3d
    nx, ny, nz = 128, 64, 64
    ndof = 3 * (nx + 1) * (ny + 1) * (nz + 1)
    _, f, fixed, _, _ = cantilever_3d(nx, ny, nz, ndof, force_mode="constant")
    f = f[:, 0] / (nz + 1)                       # unit total load, evenly spread
    assert np.isclose(f.sum(), -1.0)
    KE = lk_linear_elast_3d()
    plain = GpuProblem(nx, ny, nz, KE, fixed, f, 0.12, 1.5, ft=1, precision="fp64",
                       nlevels=4, nsmooth=2, omega=0.6, rtol=1e-8)
    mixed = GpuProblem(nx, ny, nz, KE, fixed, f, 0.12, 1.5, ft=1, precision="mixed", rtol=1e-8)
    try:
        nlev, ndofs = plain.levels()
        assert nlev == 4 and ndofs[0] == ndof
        assert ndofs[3] == 3 * 17 * 9 * 9          # coarsest 16x8x8 elements
        for _ in range(3):
            a, b = plain.step(), mixed.step()
            assert a.rel_res <= 1e-8 and b.rel_res <= 1e-8
            # two solutions with residuals <= 1e-8 ||f|| differ in compliance by
            # at most ||u|| ||r1 - r2||, a few 1e-8 ||f|| ||u|| -- not 1e-8 f.u
            np.testing.assert_allclose(b.obj, a.obj, rtol=1e-6)
            np.testing.assert_allclose(b.vol, a.vol, rtol=1e-6)   # OC bisection tolerance
        np.testing.assert_allclose(mixed.get(0), plain.get(0), atol=1e-6)
    finally:
        plain.close()
        mixed.close()


def test_mixed_solver_200_iterations_from_random_densities(gpu_lib):
    """160x80x80 cantilever from seeded random densities U[0.05, 1], smoothed
    by the rmin=1.5 filter (the designs the warm-start network is trained on):
    every one of 200 mixed-precision design iterations reaches the FP64
    relative residual 1e-8.  On one of these designs the FP32 recurrence
    stalls; the refinement loop must restart it from the true residual."""
    from topoptlab_gb300 import _lib
    from topoptlab_gb300.context import GpuProblem
    from topoptlab_gb300.elements import lk_linear_elast_3d
    from topoptlab_gb300.example_bc import cantilever_3d
    nx, ny, nz = 160, 80, 80
    ndof = 3 * (nx + 1) * (ny + 1) * (nz + 1)
    _, f, fixed, _, _ = cantilever_3d(nx, ny, nz, ndof)
    p = GpuProblem(nx, ny, nz, lk_linear_elast_3d(), fixed, f[:, 0], 0.12, 1.5, ft=1,
                   precision="mixed", rtol=1e-8)
    try:
        x = np.random.default_rng(0).uniform(0.05, 1.0, p.nel)
        xs = p.filter(x, 0)
        p.set(_lib.TG_FIELD_X, xs)
        p.set(_lib.TG_FIELD_XPHYS, p.filter(xs, 0))
        iters = []
        for _ in range(200):
            r = p.step()
            assert r.rel_res <= 1e-8
            iters.append(r.pcg_iters)
        assert max(iters) < 1000
    finally:
        p.close()
