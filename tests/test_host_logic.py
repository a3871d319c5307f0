"""Host-side logic of the package that needs no GPU: element matrices,
boundary-condition callables, option mapping, the C-ABI library's exports."""
import ctypes
import os
import re

import numpy as np
import pytest

from topoptlab_gb300 import elements as E
from topoptlab_gb300 import example_bc as B
from topoptlab_gb300.topology_optimization import solver_options, main
from topoptlab_gb300 import _lib

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_element_matrices_match_reference(golden):
    d = golden("elements.npz")
    np.testing.assert_allclose(E.lk_linear_elast_2d(l=np.array([1., 1.])), d["KE_elast2d"], atol=1e-15)
    np.testing.assert_allclose(E.lk_linear_elast_3d(l=np.array([1., 1., 1.])), d["KE_elast3d"], atol=1e-15)
    np.testing.assert_allclose(E.lk_poisson_2d(l=np.array([1., 1.])), d["KE_poisson2d"], atol=1e-15)
    np.testing.assert_allclose(E.lk_poisson_3d(l=np.array([1., 1., 1.])), d["KE_poisson3d"], atol=1e-15)
    np.testing.assert_allclose(E.lk_linear_elast_2d(l=np.array([2., 1.])), d["KE_elast2d_rect"], atol=1e-15)
    np.testing.assert_allclose(E.lk_linear_elast_3d(l=np.array([1., 2., .5])), d["KE_elast3d_rect"], atol=1e-15)


def test_bc_callables_match_reference(golden):
    d = golden("elements.npz")
    for nx, ny in [(60, 20), (10, 4)]:
        u, f, fixed, free, springs = B.mbb_2d(nx, ny, 2 * (nx + 1) * (ny + 1))
        np.testing.assert_array_equal(fixed, d[f"bc_mbb2d_{nx}x{ny}_fixed"])
        np.testing.assert_array_equal(f[:, 0], d[f"bc_mbb2d_{nx}x{ny}_f"])
        assert springs is None and len(free) + len(fixed) == u.shape[0]
    for nx, ny, nz in [(12, 6, 6), (16, 8, 8)]:
        u, f, fixed, free, _ = B.cantilever_3d(nx, ny, nz, 3 * (nx + 1) * (ny + 1) * (nz + 1))
        np.testing.assert_array_equal(fixed, d[f"bc_cant3d_{nx}x{ny}x{nz}_fixed"])
        np.testing.assert_array_equal(f[:, 0], d[f"bc_cant3d_{nx}x{ny}x{nz}_f"])
    for n in [40, 64, 100]:
        u, f, fixed, free, _ = B.heatplate_2d(n, n, (n + 1) ** 2)
        np.testing.assert_array_equal(fixed, d[f"bc_heat2d_{n}_fixed"])
        np.testing.assert_array_equal(f[:, 0], d[f"bc_heat2d_{n}_f"])


def test_solver_options_mapping():
    o = solver_options({"name": "scipy-direct"}, {"name": None})
    assert o["precond"] == "gb300-gmg" and o["rtol"] == 1e-12
    o = solver_options({"name": "gb300-gmgpcg", "rtol": 1e-6},
                       {"name": "gb300-gmg", "precision": "mixed", "nlevels": 3})
    assert o["rtol"] == 1e-6 and o["precision"] == "mixed" and o["nlevels"] == 3
    o = solver_options({"name": "gb300-pcg"}, {"name": "gb300-jacobi"})
    assert o["precond"] == "gb300-jacobi"
    # the V-cycle's smoothing options pass through to the context
    o = solver_options({"name": "gb300-gmgpcg"},
                       {"name": "gb300-gmg", "nsmooth": 1, "nsmooth_coarse": 2, "unsmoothed": 2,
                        "omega": 0.6})
    assert (o["nsmooth"], o["nsmooth_coarse"], o["unsmoothed"], o["omega"]) == (1, 2, 2, 0.6)
    o = solver_options({"name": "gb300-gmgpcg"}, {"name": "gb300-gmg"})
    assert (o["nsmooth"], o["nsmooth_coarse"], o["unsmoothed"]) == (2, 0, 0)
    with pytest.raises(ValueError):
        solver_options({"name": "no-such-solver"}, {"name": None})
    with pytest.raises(ValueError):
        solver_options({"name": "gb300-gmgpcg"}, {"name": "no-such-preconditioner"})


@pytest.mark.parametrize("kw", [dict(optimizer="mma"), dict(optimizer="oc", ft=5),
                                dict(optimizer="oc", filter_mode="helmholtz", ft=-1),
                                dict(optimizer="oc", filter_mode="no-such-filter"),
                                dict(optimizer="oc", body_forces_kw={"density_coupled": 1}),
                                dict(optimizer="oc", mix=0.5)])
def test_main_rejects_unsupported_options(kw):
    """Unsupported options fail before any device work, like the reference's
    ValueError for unknown options (topology_optimization.py:262, :367)."""
    with pytest.raises(ValueError):
        main(nelx=4, nely=2, volfrac=0.5, rmin=1.5,
             output_kw={"file": None, "display": False, "export": False, "write_log": False}, **kw)


def test_learned_options_parse_and_refuse_without_parameters(tmp_path):
    """preconditioner_kw["learned"]: parameters (array, .npy path or a dict
    with a mode) pass through; True without parameters, or a network on a
    problem it does not serve, raises ValueError before any device work."""
    from topoptlab_gb300.topology_optimization import learned_network
    from topoptlab_gb300.context import learned_mask
    assert learned_network(False) == (None, 0)
    p, mode = learned_network(np.arange(5.0))
    assert p.dtype == np.float32 and p.size == 5 and mode == "warm_start"
    np.save(tmp_path / "w.npy", np.ones(7, dtype=np.float32))
    p, mode = learned_network({"params": str(tmp_path / "w.npy"), "mode": "both"})
    assert p.size == 7 and mode == "both"
    assert [learned_mask(v) for v in (False, True, "warm_start", "coarse_correction", 3)] == \
        [0, 3, 1, 2, 3]
    with pytest.raises(ValueError):
        learned_mask("no-such-mode")
    out = {"file": None, "display": False, "export": False, "write_log": False}
    with pytest.raises(ValueError, match="trained network parameters"):
        main(nelx=4, nely=2, nelz=2, volfrac=0.5, rmin=1.5, optimizer="oc", output_kw=out,
             preconditioner_kw={"name": "gb300-gmg", "precision": "mixed", "learned": True})
    with pytest.raises(ValueError, match="3-D problem"):
        main(nelx=4, nely=2, volfrac=0.5, rmin=1.5, optimizer="oc", output_kw=out,
             preconditioner_kw={"name": "gb300-gmg", "precision": "mixed",
                                "learned": np.ones(3)})


def test_main_helmholtz_3d_not_implemented():
    """assemble_helmholtz_filter raises NotImplementedError for 3-D grids
    (filter/helmholtz_filter.py:180); the drop-in does the same."""
    with pytest.raises(NotImplementedError):
        main(nelx=4, nely=2, nelz=2, volfrac=0.5, rmin=1.5, ft=1, filter_mode="helmholtz", optimizer="oc",
             output_kw={"file": None, "display": False, "export": False, "write_log": False})


def _declared_symbols():
    txt = open(os.path.join(ROOT, "include", "topopt_gb300.h")).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(tg_[a-z_0-9]+)\s*\(", txt)))


def test_header_and_binding_agree():
    assert _declared_symbols() == sorted(_lib.SIGNATURES)


def test_library_loads_and_exports_every_symbol():
    """Build the library here (nvcc cross-compiles, no GPU needed) and check
    that every declared entry point is exported; no compute call is made."""
    from topoptlab_gb300 import build as b
    path = b.build()
    lib = ctypes.CDLL(path)
    for name in _declared_symbols():
        assert hasattr(lib, name), name
    assert _lib.load().tg_abi_version() == _lib.TG_ABI_VERSION == 6


def test_header_constants_match_binding():
    """Every constant the header defines (status codes, precisions, fields,
    learned bits, tg_tune keys, the ABI version, the allocation-free entry's
    size limit) has the same value in the Python binding."""
    txt = open(os.path.join(ROOT, "include", "topopt_gb300.h")).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    vals = {}
    for body in re.findall(r"enum\s*\{(.*?)\}", txt, flags=re.S):
        for m in re.finditer(r"(TG_[A-Z0-9_]+)\s*=\s*(-?\d+)", body):
            vals[m.group(1)] = int(m.group(2))
    for m in re.finditer(r"#define\s+(TG_[A-Z0-9_]+)\s+(\d+)", txt):
        vals[m.group(1)] = int(m.group(2))
    assert len(vals) >= 29
    for name, v in vals.items():
        assert getattr(_lib, name) == v, name


@pytest.mark.parametrize("case", ["nelx0", "ke_shape", "fixed_range", "f_length", "ft", "precision",
                                  "filter_mode"])
def test_problem_arguments_rejected_before_device_work(case):
    """Invalid problem descriptions raise ValueError (TG_EINVAL) before any
    device is touched (so this runs without a GPU)."""
    from topoptlab_gb300.context import GpuProblem
    from topoptlab_gb300.elements import lk_linear_elast_2d
    KE = lk_linear_elast_2d()
    f = np.zeros(50)
    args = {"nelx0": ((0, 4, None, KE, [0], np.zeros(10)), {}),
            "ke_shape": ((4, 4, None, np.eye(7), [0], f), {}),
            "fixed_range": ((4, 4, None, KE, [10 ** 6], f), {}),
            "f_length": ((4, 4, None, KE, [0], np.zeros(7)), {}),
            "ft": ((4, 4, None, KE, [0], f), {"ft": 5}),
            "precision": ((4, 4, None, KE, [0], f), {"precision": "fp16"}),
            "filter_mode": ((4, 4, None, KE, [0], f), {"filter_mode": "no-such-filter"})}[case]
    pos, kw = args
    with pytest.raises(ValueError):
        GpuProblem(*pos, 0.5, 1.5, **kw)


# the (solver, preconditioner) pairs of the reference's tests/test_solver.py:8-24
REFERENCE_SOLVER_CASES = [("scipy-direct", None), ("scipy-cg", None), ("scipy-bicg", None),
                          ("scipy-cgs", "scipy-ilu"), ("scipy-minres", None),
                          ("scipy-lgmres", None), ("scipy-gmres", "scipy-ilu"),
                          ("scipy-gcrotmk", None), ("scipy-cg", "scipy-ilu"),
                          ("cvxopt-cholmod", None), ("scipy-cg", "pyamg-adaptive_sa"),
                          ("scipy-cg", "pyamg-rootnode_solver"),
                          ("scipy-cg", "pyamg-pairwise_solver"),
                          ("scipy-cg", "pyamg-smoothed_aggregation"), ("topoptlab-cg", None),
                          ("topoptlab-pcg", "scipy-ilu")]


@pytest.mark.parametrize("solver,precond", REFERENCE_SOLVER_CASES)
def test_reference_solver_names_map(solver, precond):
    """Every solver / preconditioner name the reference's solver test uses is
    accepted and runs the GPU multigrid PCG with the caller's tolerance."""
    o = solver_options({"name": solver, "rtol": 1e-10, "maxiter": 10000}, {"name": precond})
    assert o["precond"] == "gb300-gmg" and o["rtol"] == 1e-10 and o["maxiter"] == 10000


@pytest.mark.parametrize("nelx,nely,nelz,kind", [(60, 20, None, "elast"), (7, 5, None, "poisson"),
                                                  (12, 6, 4, "elast"), (5, 4, 3, "poisson"),
                                                  (1, 1, None, "elast"), (3, 1, 2, "poisson")])
def test_compliance_infers_grid_from_edofmat(nelx, nely, nelz, kind):
    """objectives.compliance takes the reference's signature (no grid sizes,
    objectives.py:7-15): the grid and DOFs per node come from edofMat (the
    reference numbering, pinned by the oracle's edofMat fixtures)."""
    from oracle import topopt as O
    from topoptlab_gb300.objectives import grid_from_edofmat
    ndim = 2 if nelz is None else 3
    nd = (ndim if kind == "elast" else 1)
    ed = O.edofmat(nelx, nely, nelz, nd)
    assert grid_from_edofmat(ed, ed.shape[1]) == (nelx, nely, nelz, nd)
    with pytest.raises(ValueError):
        grid_from_edofmat(ed, ed.shape[1] + 1)
    if ed.shape[0] > 1:                      # elements out of order
        with pytest.raises(ValueError):
            grid_from_edofmat(ed[::-1], ed.shape[1])
