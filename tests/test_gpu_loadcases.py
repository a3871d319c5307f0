"""Several load cases (columns of the bcs() load matrix): one solve per case
with the same hierarchy, compliance and sensitivities summed over the cases
(topology_optimization.py:446-500)."""
import numpy as np
import pytest

from oracle import topopt as O

pytestmark = pytest.mark.gpu

OUT = {"file": None, "display": False, "export": False, "write_log": False,
       "profile": False, "debug": 0}


def test_cantilever_twoloads_golden(gpu_lib):
    """tests/test_compliance.py:14 -- 510.3727841006 at decimal=5."""
    from topoptlab_gb300 import main
    from topoptlab_gb300.example_bc import cantilever_2d_twoloads
    x, obj = main(nelx=60, nely=20, volfrac=0.5, rmin=2.4, ft=0, filter_mode="matrix",
                  optimizer="oc", bcs=cantilever_2d_twoloads,
                  lin_solver_kw={"name": "scipy-direct"}, output_kw=dict(OUT))
    np.testing.assert_almost_equal(obj, 510.3727841006, decimal=5)


def test_cantilever_2d_golden(gpu_lib):
    """tests/test_compliance.py:15 -- 208.4429354360 at decimal=5."""
    from topoptlab_gb300 import main
    from topoptlab_gb300.example_bc import cantilever_2d
    x, obj = main(nelx=60, nely=20, volfrac=0.5, rmin=2.4, ft=0, filter_mode="matrix",
                  optimizer="oc", bcs=cantilever_2d,
                  lin_solver_kw={"name": "scipy-direct"}, output_kw=dict(OUT))
    np.testing.assert_almost_equal(obj, 208.4429354360, decimal=5)


@pytest.mark.parametrize("precision,rtol", [("fp64", 1e-12), ("mixed", 1e-11)])
def test_twoloads_trajectory_vs_oracle(gpu_lib, precision, rtol):
    """20 design iterations of the two-load cantilever against the oracle
    (direct solves), and the displacements of both cases."""
    from topoptlab_gb300 import _lib
    from topoptlab_gb300.context import GpuProblem
    fixed, f = O.bc_cantilever_2d_twoloads(60, 20)
    KE = O.ke_elast(2)
    ref = O.run(60, 20, None, 0.5, 2.4, 0, KE, fixed, f, nouteriter=20)
    prob = GpuProblem(60, 20, None, KE, fixed, f, 0.5, 2.4, ft=0, rtol=rtol, precision=precision)
    try:
        objs = [prob.step().obj for _ in range(20)]
        u = prob.get(_lib.TG_FIELD_U)
        x = prob.get(_lib.TG_FIELD_X)
    finally:
        prob.close()
    assert u.shape == (f.shape[0], 2)
    np.testing.assert_allclose(objs, ref["obj"], rtol=1e-8)
    np.testing.assert_allclose(x, ref["x"], atol=1e-8)
    np.testing.assert_allclose(u, ref["u"], rtol=0, atol=1e-8 * np.abs(ref["u"]).max())
