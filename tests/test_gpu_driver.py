"""The drop-in driver on the GPU against the reference's own trajectories
(fixtures made by running the reference, tests/golden/make_golden.py) and the
reference test suite's golden compliance values (tests/test_compliance.py)."""
import numpy as np
import pytest

from oracle import topopt as O

pytestmark = pytest.mark.gpu

OUT = {"file": None, "display": False, "export": False, "write_log": False,
       "profile": False, "debug": 0}


def test_mbb_density_filter_full_run(gpu_lib, golden):
    """tests/test_compliance.py:10 -- 233.71457 at decimal=5, plus the whole
    144-iteration trajectory and final design within 1e-8."""
    from topoptlab_gb300 import main
    from topoptlab_gb300.example_bc import mbb_2d
    g = golden("mbb2d_60x20.npz")
    x, obj = main(nelx=60, nely=20, volfrac=0.5, rmin=2.4, ft=1, filter_mode="matrix",
                  optimizer="oc", bcs=mbb_2d, lin_solver_kw={"name": "scipy-direct"},
                  output_kw=dict(OUT))
    np.testing.assert_almost_equal(obj, 233.71457, decimal=5)
    np.testing.assert_allclose(obj, float(g["final_obj"]), rtol=1e-8)
    np.testing.assert_allclose(x[:, 0], g["final_x"], atol=1e-8)


def test_log_file_matches_reference(gpu_lib, tmp_path):
    """The log file of main (write_log, verbosity 20) against the reference's
    own log of the same MBB run (topology_optimization.py:181-199, :669-670):
    the same lines in the same order, the set-up lines identical, each
    iteration line in the reference's format with its numbers within the
    solver tolerance (obj 1e-8 relative, vol and change 1e-9)."""
    import os
    import re
    from topoptlab_gb300 import main
    from topoptlab_gb300.example_bc import mbb_2d
    ref = open(os.path.join(os.path.dirname(__file__), "golden", "mbb2d_60x20.log")).read()
    base = str(tmp_path / "mbb")
    out = dict(OUT, write_log=True, file=base, verbosity=20)
    main(nelx=60, nely=20, volfrac=0.5, rmin=2.4, ft=1, filter_mode="matrix", optimizer="oc",
         bcs=mbb_2d, lin_solver_kw={"name": "scipy-direct"}, output_kw=out)
    ours = open(base + ".log").read().splitlines()
    theirs = ref.splitlines()
    assert len(ours) == len(theirs)
    pat = re.compile(r"^it\.: (\d+) obj\.: (-?\d+\.\d{10}) vol\.: (-?\d+\.\d{10}) "
                     r"ch\.: (-?\d+\.\d{10})$")
    for a, b in zip(ours, theirs):
        mb = pat.match(b)
        if mb is None:
            assert a == b
            continue
        ma = pat.match(a)
        assert ma is not None, a
        assert ma.group(1) == mb.group(1)
        np.testing.assert_allclose(float(ma.group(2)), float(mb.group(2)), rtol=1e-8)
        np.testing.assert_allclose(float(ma.group(3)), float(mb.group(3)), rtol=0, atol=1e-9)
        np.testing.assert_allclose(float(ma.group(4)), float(mb.group(4)), rtol=0, atol=1e-9)


def test_mbb_sensitivity_filter(gpu_lib, golden):
    """tests/test_compliance.py:9 -- 216.81366 (ft=0)."""
    from topoptlab_gb300 import main
    from topoptlab_gb300.example_bc import mbb_2d
    g = golden("mbb2d_60x20_ft0.npz")
    x, obj = main(nelx=60, nely=20, volfrac=0.5, rmin=2.4, ft=0, optimizer="oc", bcs=mbb_2d,
                  lin_solver_kw={"name": "scipy-direct"}, output_kw=dict(OUT))
    np.testing.assert_almost_equal(obj, 216.81366, decimal=5)
    np.testing.assert_allclose(x[:, 0], g["final_x"], atol=1e-7)


def test_heat_plate_trajectory(gpu_lib, golden):
    """Heat plate 40x40 (tests/test_compliance.py:91-113 set-up), first 40
    design iterations within 1e-8 of the reference's run.

    Beyond ~iteration 40 this ft=0 trajectory is chaotic: a 1e-13 relative
    perturbation of the first sensitivities grows to 1e-6 by iteration 59 (the
    CPU oracle, the reference algorithm with another summation order, ends at
    473.32 after 158 iterations against the reference's 473.73 after 130).  The
    reference's decimal=3 golden therefore pins its own rounding sequence; the
    converged value is checked against it at 3e-3 relative below."""
    from topoptlab_gb300.context import GpuProblem
    from topoptlab_gb300.elements import lk_poisson_2d
    g = golden("heat2d_40x40.npz")
    fixed, f = O.bc_heatplate_2d(40, 40)
    prob = GpuProblem(40, 40, None, lk_poisson_2d(), fixed, f, 0.4, 1.2, ft=0, rtol=1e-12)
    try:
        objs = [prob.step().obj for _ in range(40)]
    finally:
        prob.close()
    np.testing.assert_allclose(objs, g["obj"][:40], rtol=1e-8)


def test_heat_plate_converged(gpu_lib, golden):
    """tests/test_compliance.py:92 -- 473.7336997084.  The converged value of
    this chaotic ft=0 run depends on the rounding sequence (see the trajectory
    test): the CPU oracle ends 0.09% below the reference, and solver builds
    that differ from each other only in the summation order of the coarsest
    dense solve ended 0.05% and 0.10% above it.  The band is 3e-3 relative."""
    from topoptlab_gb300 import main
    from topoptlab_gb300.example_bc import heatplate_2d
    from topoptlab_gb300.elements import lk_poisson_2d
    x, obj = main(nelx=40, nely=40, volfrac=0.4, rmin=1.2, ft=0, optimizer="oc",
                  bcs=heatplate_2d, lk=lk_poisson_2d, lin_solver_kw={"name": "scipy-direct"},
                  output_kw=dict(OUT))
    np.testing.assert_allclose(obj, 473.7336997084, rtol=3e-3)
    np.testing.assert_allclose(np.mean(x), 0.4, atol=1e-3)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_cantilever_3d_trajectory(gpu_lib, golden, precision):
    """3-D cantilever (reference callable semantics), 12 iterations: compliance
    per iteration and final design within 1e-8 of the reference run."""
    from topoptlab_gb300.context import GpuProblem
    from topoptlab_gb300.elements import lk_linear_elast_3d
    g = golden("cant3d_12x6x6.npz")
    fixed, f = O.bc_cantilever_3d(12, 6, 6)
    prob = GpuProblem(12, 6, 6, lk_linear_elast_3d(), fixed, f, 0.3, 1.5, ft=1, rtol=1e-12,
                      precision=precision)
    try:
        objs = [prob.step().obj for _ in range(12)]
        x = prob.get(0)
    finally:
        prob.close()
    np.testing.assert_allclose(objs, g["obj"], rtol=1e-8)
    np.testing.assert_allclose(x, g["final_x"], atol=1e-8)


# (grid, design iterations, multigrid levels: 0 = automatic, 4 at 48x24x24)
LADDER = [(16, 8, 8, 20, 3), (32, 16, 16, 10, 4), (48, 24, 24, 2, 0)]


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("nelx,nely,nelz,nit,nlevels", LADDER)
def test_cantilever_3d_ladder(gpu_lib, golden, precision, nelx, nely, nelz, nit, nlevels):
    """The 3-D cantilever (reference cantilever_3d callable, volfrac 0.3,
    rmin 1.5, ft=1) on grids with deep multigrid hierarchies (3, 4 and 4
    levels, the last automatic): compliance of every iteration, the final design
    and -- where recorded -- the last iteration's xPhys, filtered
    sensitivities and displacement within 1e-8 of the reference's scipy-direct
    run."""
    from topoptlab_gb300.context import GpuProblem
    from topoptlab_gb300.elements import lk_linear_elast_3d
    from topoptlab_gb300 import _lib
    g = golden(f"cant3d_{nelx}x{nely}x{nelz}.npz")
    fixed, f = O.bc_cantilever_3d(nelx, nely, nelz)
    prob = GpuProblem(nelx, nely, nelz, lk_linear_elast_3d(), fixed, f, 0.3, 1.5, ft=1,
                      rtol=1e-12, precision=precision, nlevels=nlevels)
    try:
        assert prob.levels()[0] >= 3
        objs = []
        for k in range(nit):
            if k == nit - 1:
                xphys_last = prob.get(_lib.TG_FIELD_XPHYS)
            objs.append(prob.step().obj)
        x = prob.get(_lib.TG_FIELD_X)
        dc = prob.get(_lib.TG_FIELD_DC)
        u = prob.get(_lib.TG_FIELD_U)
    finally:
        prob.close()
    np.testing.assert_allclose(objs, g["obj"], rtol=1e-8)
    np.testing.assert_allclose(x, g["final_x"], atol=1e-8)
    if "xPhys_last" in g.files:
        np.testing.assert_allclose(xphys_last, g["xPhys_last"], atol=1e-8)
        np.testing.assert_allclose(dc, g["dc_last"], rtol=0, atol=1e-8 * np.abs(g["dc_last"]).max())
    if "u_last" in g.files:
        np.testing.assert_allclose(u, g["u_last"], rtol=0, atol=1e-8 * np.abs(g["u_last"]).max())


def test_teacher_forced_iteration(gpu_lib, golden):
    """Per-iteration parity: start from the reference's state at iteration 24
    (xPhys, x, g) and compare u, obj and the OC output of that iteration."""
    from topoptlab_gb300.context import GpuProblem
    from topoptlab_gb300.elements import lk_linear_elast_2d
    from topoptlab_gb300 import _lib
    g = golden("mbb2d_60x20.npz")
    fixed, f = O.bc_mbb_2d(60, 20)
    prob = GpuProblem(60, 20, None, lk_linear_elast_2d(), fixed, f, 0.5, 2.4, ft=1, rtol=1e-12)
    try:
        u, info = prob.solve(g["xPhys_24"], f)
        np.testing.assert_allclose(u, g["u_24"], rtol=0, atol=1e-9 * np.abs(g["u_24"]).max())
        obj, dc = prob.compliance(g["xPhys_24"], u)
        np.testing.assert_allclose(obj, g["obj"][24], rtol=1e-9)
    finally:
        prob.close()


def test_nonconvergence_raises(gpu_lib):
    """A PCG iteration cap that cannot be met surfaces as RuntimeError, like
    solve_linsystem.py:349-351 (failure made on the host: maxiter=1)."""
    from topoptlab_gb300.context import GpuProblem
    from topoptlab_gb300.elements import lk_linear_elast_2d
    fixed, f = O.bc_mbb_2d(32, 16)
    prob = GpuProblem(32, 16, None, lk_linear_elast_2d(), fixed, f, 0.5, 1.5, maxiter=1,
                      rtol=1e-12)
    try:
        with pytest.raises(RuntimeError, match="did not converge"):
            prob.step()
    finally:
        prob.close()


def test_nan_density_raises(gpu_lib):
    from topoptlab_gb300.context import GpuProblem
    from topoptlab_gb300.elements import lk_linear_elast_2d
    from topoptlab_gb300 import _lib
    fixed, f = O.bc_mbb_2d(16, 8)
    prob = GpuProblem(16, 8, None, lk_linear_elast_2d(), fixed, f, 0.5, 1.5)
    try:
        x = np.full(16 * 8, 0.5)
        x[3] = np.nan
        prob.set(_lib.TG_FIELD_XPHYS, x)
        with pytest.raises(RuntimeError):
            prob.step()
    finally:
        prob.close()


def test_get_into_page_locked_buffer(gpu_lib):
    """get(field, out=...) copies into the caller's array (page-locked host
    memory in the end-to-end bench) with the values of get(field); a wrong
    dtype, size or layout raises ValueError."""
    torch = pytest.importorskip("torch")
    from topoptlab_gb300.context import GpuProblem
    from topoptlab_gb300.elements import lk_linear_elast_2d
    from topoptlab_gb300 import _lib
    fixed, f = O.bc_mbb_2d(24, 12)
    prob = GpuProblem(24, 12, None, lk_linear_elast_2d(), fixed, f, 0.5, 1.5)
    try:
        prob.step()
        for field, n in ((_lib.TG_FIELD_XPHYS, 24 * 12), (_lib.TG_FIELD_U, prob.ndof)):
            buf = torch.empty(n, dtype=torch.float64, pin_memory=True).numpy()
            assert prob.get(field, out=buf) is buf
            np.testing.assert_array_equal(buf, prob.get(field))
        with pytest.raises(ValueError):
            prob.get(_lib.TG_FIELD_X, out=np.empty(24 * 12, dtype=np.float32))
        with pytest.raises(ValueError):
            prob.get(_lib.TG_FIELD_X, out=np.empty(24 * 12 + 1))
        with pytest.raises(ValueError):
            prob.get(_lib.TG_FIELD_X, out=np.empty((24 * 12, 2))[:, 0])
    finally:
        prob.close()


def test_main_exports_vtk(gpu_lib, tmp_path):
    """output_kw export / output_movie write the reference's VTK files: one per
    design iteration, named file_<iteration>, and the final design as file.vtk,
    whose xPhys cell data is the returned design's filtered density."""
    from topoptlab_gb300 import main
    from topoptlab_gb300.example_bc import mbb_2d
    name = str(tmp_path / "mbb")
    out = dict(OUT, file=name, export=True, output_movie=True)
    x, _ = main(nelx=12, nely=4, volfrac=0.5, rmin=1.5, ft=1, optimizer="oc", bcs=mbb_2d,
                nouteriter=5, output_kw=out)
    assert (tmp_path / "mbb.vtk").exists()
    assert sorted(p.name for p in tmp_path.glob("mbb_*.vtk")) == [f"mbb_{i}.vtk" for i in range(5)]
    txt = (tmp_path / "mbb.vtk").read_text()
    assert "CELLS 48 240" in txt and "POINTS 65 double" in txt
    for field in ("u0", "f0", "xPhys", "x", "xThresh"):
        assert f" {field} " in txt



def test_solver_independence(gpu_lib):
    """tests/test_solver.py:8-59 of the reference: the 10x3 MBB beam gives the
    scipy-direct compliance (decimal 3) whatever solver and preconditioner
    names are passed (they all run the GPU multigrid PCG here, to the
    caller's rtol)."""
    from topoptlab_gb300 import main
    from topoptlab_gb300.example_bc import mbb_2d
    cases_all = [("scipy-direct", None), ("scipy-cg", None), ("scipy-bicg", None),
                 ("scipy-cgs", "scipy-ilu"), ("scipy-minres", None), ("scipy-lgmres", None),
                 ("scipy-gmres", "scipy-ilu"), ("scipy-gcrotmk", None), ("scipy-cg", "scipy-ilu"),
                 ("cvxopt-cholmod", None), ("scipy-cg", "pyamg-adaptive_sa"),
                 ("scipy-cg", "pyamg-rootnode_solver"), ("scipy-cg", "pyamg-pairwise_solver"),
                 ("scipy-cg", "pyamg-smoothed_aggregation"), ("topoptlab-cg", None),
                 ("topoptlab-pcg", "scipy-ilu")]
    out = dict(OUT)
    for ft in (0, 1):
        _, obj_ref = main(nelx=10, nely=3, volfrac=0.5, rmin=2.4, ft=ft, filter_mode="matrix",
                          optimizer="oc", bcs=mbb_2d, lin_solver_kw={"name": "scipy-direct"},
                          output_kw=dict(out))
        cases = cases_all[:1] if ft == 0 else cases_all[1:]
        for solver, precond in cases:
            _, obj = main(nelx=10, nely=3, volfrac=0.5, rmin=2.4, ft=ft, filter_mode="matrix",
                          optimizer="oc", bcs=mbb_2d,
                          lin_solver_kw={"name": solver, "rtol": 1e-10, "maxiter": 10000},
                          preconditioner_kw={"name": precond}, output_kw=dict(out))
            np.testing.assert_almost_equal(obj, obj_ref, decimal=3)
