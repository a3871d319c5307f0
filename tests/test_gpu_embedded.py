"""Grids whose element counts do not halve down to a small coarsest level
(odd counts) run on a padded device grid: zero-stiffness padding elements,
fixed padding nodes, and the filter, volume, compliance and OC restricted to
the caller's elements.  The caller keeps its own numbering and gets the
reference algorithm's results (CPU oracle with a direct solve)."""
import numpy as np
import pytest

from oracle import topopt as O

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("precision,rtol", [("fp64", 1e-12), ("mixed", 1e-11)])
def test_heat_plate_65x65_embedded(gpu_lib, precision, rtol):
    """65x65 heat plate, ft=0: without padding the grid cannot be coarsened and
    its 4356-DOF fine level would be the dense coarsest level; embedded in
    66x66 it gets a 2-level hierarchy.  8 design iterations within 1e-8 of
    the oracle's trajectory."""
    from topoptlab_gb300 import _lib
    from topoptlab_gb300.context import GpuProblem
    n = 65
    fixed, f = O.bc_heatplate_2d(n, n)
    KE = O.ke_poisson(2)
    ref = O.run(n, n, None, 0.4, 1.2, 0, KE, fixed, f, nouteriter=8)
    prob = GpuProblem(n, n, None, KE, fixed, f, 0.4, 1.2, ft=0, rtol=rtol, precision=precision)
    try:
        nlev, ndofs = prob.levels()
        assert nlev >= 2 and ndofs[0] == 67 * 67 and ndofs[-1] <= 1200
        objs = [prob.step().obj for _ in range(8)]
        x = prob.get(_lib.TG_FIELD_X)
        u = prob.get(_lib.TG_FIELD_U)
    finally:
        prob.close()
    np.testing.assert_allclose(objs, ref["obj"], rtol=1e-8)
    np.testing.assert_allclose(x, ref["x"], atol=1e-8)
    np.testing.assert_allclose(u, ref["u"], rtol=0, atol=1e-8 * np.abs(ref["u"]).max())


def test_cantilever_25x13x13_embedded(gpu_lib):
    """25x13x13 hex8 cantilever, ft=1: the natural coarsest level (15,288
    DOFs) is beyond the dense solve; embedded in 28x16x16 it gets a
    hierarchy down to 8x5x5 nodes.  4 design iterations within 1e-8 of the
    oracle, and the unit entry points refuse the padded grid."""
    from topoptlab_gb300 import _lib
    from topoptlab_gb300.context import GpuProblem
    nx, ny, nz = 25, 13, 13
    fixed, f = O.bc_cantilever_3d(nx, ny, nz)
    KE = O.ke_elast(3)
    ref = O.run(nx, ny, nz, 0.3, 1.5, 1, KE, fixed, f, nouteriter=4)
    prob = GpuProblem(nx, ny, nz, KE, fixed, f, 0.3, 1.5, ft=1, rtol=1e-12)
    try:
        nlev, ndofs = prob.levels()
        assert ndofs[0] == 3 * 29 * 17 * 17 and ndofs[-1] == 3 * 8 * 5 * 5
        objs = [prob.step().obj for _ in range(4)]
        vols = [prob.get(_lib.TG_FIELD_XPHYS).mean()]
        x = prob.get(_lib.TG_FIELD_X)
        with pytest.raises(ValueError, match="padded"):
            prob.kmul(x, np.zeros(3 * 26 * 14 * 14))
    finally:
        prob.close()
    np.testing.assert_allclose(objs, ref["obj"], rtol=1e-8)
    np.testing.assert_allclose(x, ref["x"], atol=1e-8)
    np.testing.assert_allclose(vols[0], ref["vol"][-1], rtol=1e-12)
