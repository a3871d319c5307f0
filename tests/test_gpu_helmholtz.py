"""Helmholtz PDE filter on the GPU (filter/helmholtz_filter.py:133-200 as main
applies it, topology_optimization.py:360-365, 554-555, 568-570, 646-647):
the filter against the reference's outputs on seeded fields, the reference's
full MBB runs (tests/test_compliance.py:11-12), 3-D and padded grids against
the oracle, and the constant-preservation property of the PDE filter."""
import numpy as np
import pytest

from oracle import topopt as O

pytestmark = pytest.mark.gpu

OUT = {"file": None, "display": False, "export": False, "write_log": False,
       "profile": False, "debug": 0}


def _problem(nx, ny, nz, rmin, ft=1, **kw):
    from topoptlab_gb300.context import GpuProblem
    if nz is None:
        fixed, f = O.bc_mbb_2d(nx, ny)
        KE = O.ke_elast(2)
    else:
        fixed, f = O.bc_cantilever_3d(nx, ny, nz)
        KE = O.ke_elast(3)
    return GpuProblem(nx, ny, nz, KE, fixed, f, 0.5, rmin, ft=ft, filter_mode="helmholtz",
                      rtol=1e-10, **kw)


@pytest.mark.parametrize("nx,ny,rmin,precond", [(7, 5, 2.4, "gb300-jacobi"),
                                                (12, 8, 1.5, "gb300-gmg")])
def test_filter_matches_reference(gpu_lib, golden, nx, ny, rmin, precond):
    g = golden("helmholtz.npz")
    key = f"{nx}_{ny}_{rmin}"
    x, dx = g["x_" + key], g["dx_" + key]
    prob = _problem(nx, ny, None, rmin, precond=precond)
    try:
        np.testing.assert_allclose(prob.filter(x, 6), g["y_" + key], rtol=0, atol=1e-11)
        np.testing.assert_allclose(prob.filter(x, 7, d=dx), g["dy_" + key], rtol=1e-10,
                                   atol=1e-11)
    finally:
        prob.close()


def test_filter_3d_matches_oracle_and_keeps_constants(gpu_lib):
    """3-D (the reference stops at NotImplementedError there; the oracle
    restates the same operators with the hexahedron screened Poisson element)."""
    nx, ny, nz, rmin = 8, 4, 4, 1.5
    rng = np.random.default_rng(3)
    x = rng.uniform(0.0, 1.0, nx * ny * nz)
    solve, TF = O.helmholtz_operators(nx, ny, nz, rmin)
    prob = _problem(nx, ny, nz, rmin)
    try:
        np.testing.assert_allclose(prob.filter(x, 6), O.helmholtz_apply(solve, TF, x),
                                   rtol=0, atol=1e-11)
        # K 1 = 0 and M 1 = TF 1, so constants pass unchanged
        np.testing.assert_allclose(prob.filter(np.full(x.size, 0.37), 6), 0.37, rtol=1e-11)
    finally:
        prob.close()


@pytest.mark.parametrize("ft,golden_obj", [(1, 237.59964), (0, 218.79281)])
def test_mbb_helmholtz_full_run(gpu_lib, golden, ft, golden_obj):
    """tests/test_compliance.py:11-12 at decimal=5, plus the reference's whole
    trajectory (140 / 107 design iterations) and final design."""
    from topoptlab_gb300 import main
    from topoptlab_gb300.example_bc import mbb_2d
    g = golden(f"mbb2d_60x20_helmholtz_ft{ft}.npz")
    x, obj = main(nelx=60, nely=20, volfrac=0.5, rmin=2.4, ft=ft, filter_mode="helmholtz",
                  optimizer="oc", bcs=mbb_2d, lin_solver_kw={"name": "scipy-direct"},
                  output_kw=dict(OUT))
    np.testing.assert_almost_equal(obj, golden_obj, decimal=5)
    np.testing.assert_allclose(obj, float(g["final_obj"]), rtol=1e-8)
    np.testing.assert_allclose(x[:, 0], g["final_x"], atol=1e-7)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_padded_grid_trajectory(gpu_lib, precision):
    """45x15 MBB (odd element counts: the device grid is padded) with the PDE
    density filter: 6 design iterations against the oracle."""
    from topoptlab_gb300.context import GpuProblem
    nx, ny = 45, 15
    fixed, f = O.bc_mbb_2d(nx, ny)
    KE = O.ke_elast(2)
    ref = O.run(nx, ny, None, 0.5, 2.4, 1, KE, fixed, f, nouteriter=6, filter_mode="helmholtz")
    prob = GpuProblem(nx, ny, None, KE, fixed, f, 0.5, 2.4, ft=1, filter_mode="helmholtz",
                      precision=precision, rtol=1e-12)
    try:
        res = [prob.step() for _ in range(6)]
        np.testing.assert_allclose([r.obj for r in res], ref["obj"], rtol=1e-8)
        np.testing.assert_allclose([r.vol for r in res], ref["vol"], rtol=1e-10)
        np.testing.assert_allclose(prob.get(0), ref["x"], atol=1e-8)
    finally:
        prob.close()


def test_filter_objects(gpu_lib, golden):
    """MatrixFilter / HelmholtzFilter objects (filter/matrix_filter.py:9-99,
    filter/helmholtz_filter.py:16-131): H (x / Hs) for both directions of the
    matrix filter, TF^T KF^-1 TF v for the PDE filter, volume conserved."""
    from topoptlab_gb300.filter import HelmholtzFilter, MatrixFilter
    rng = np.random.default_rng(9)
    for (nx, ny, nz, rmin) in [(9, 6, None, 1.5), (6, 5, 4, 1.5)]:
        H, Hs = O.filter_matrix(nx, ny, nz, rmin)
        x = rng.uniform(0.0, 1.0, (nx * ny * (nz or 1), 1))
        with MatrixFilter(nelx=nx, nely=ny, nelz=nz, rmin=rmin) as f:
            assert f.vol_conserv
            y = f.apply_filter(x)
            assert y.shape == x.shape
            ref = np.asarray(H @ (x[:, 0] / Hs))
            np.testing.assert_allclose(y[:, 0], ref, rtol=0, atol=1e-13)
            np.testing.assert_allclose(f.apply_filter_dx(x)[:, 0], ref, rtol=0, atol=1e-13)
            np.testing.assert_allclose(y.sum(), x.sum(), rtol=1e-12)
    g = golden("helmholtz.npz")
    for (nx, ny, rmin) in [(7, 5, 2.4), (12, 8, 1.5)]:
        key = f"{nx}_{ny}_{rmin}"
        x, dx = g["x_" + key], g["dx_" + key]
        solve, TF = O.helmholtz_operators(nx, ny, None, rmin)
        with HelmholtzFilter(nelx=nx, nely=ny, rmin=rmin) as f:
            assert f.vol_conserv
            y = f.apply_filter(x)
            np.testing.assert_allclose(y, g["y_" + key], rtol=0, atol=1e-11)
            np.testing.assert_allclose(f.apply_filter_dx(y, dx), O.helmholtz_apply(solve, TF, dx),
                                       rtol=0, atol=1e-11)
            np.testing.assert_allclose(y.sum(), x.sum(), rtol=1e-10)
