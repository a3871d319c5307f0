"""solve_lin / pcg mirrors on the GPU against the reference's own data: the
reduced SIMP stiffness matrix K[free][:, free] of MBB iteration 25 (assembled
by the oracle from the reference's recorded densities) and the displacement
the reference's direct solve produced for it."""
import numpy as np
import pytest

from oracle import topopt as O

pytestmark = pytest.mark.gpu


def _system(golden):
    g = golden("mbb2d_60x20.npz")
    x = g["xPhys_24"]
    KE = O.ke_elast(2)
    ndof = 2 * 61 * 21
    K = O.assemble(KE, O.edofmat(60, 20, None, 2), O.simp(x), ndof)
    fixed, f = O.bc_mbb_2d(60, 20)
    free = np.setdiff1d(np.arange(ndof), fixed)
    return K[free][:, free].tocsr(), f[free], g["u_24"][free]


def test_solve_lin_assembled_matrix(gpu_lib, golden):
    from topoptlab_gb300.solve_linsystem import solve_lin
    Kff, ff, uref = _system(golden)
    sol, fact, P = solve_lin(Kff, ff[:, None], solver="scipy-direct")
    assert sol.shape == (ff.shape[0], 1)
    np.testing.assert_allclose(sol[:, 0], uref, rtol=0, atol=1e-8 * np.abs(uref).max())


def test_pcg_mirror_and_nonconvergence(gpu_lib, golden):
    from topoptlab_gb300.solve_linsystem import pcg, solve_lin
    Kff, ff, uref = _system(golden)
    x, info = pcg(Kff, ff, rtol=1e-10)
    assert info == 0
    np.testing.assert_allclose(x, uref, rtol=0, atol=1e-7 * np.abs(uref).max())
    x, info = pcg(Kff, ff, rtol=1e-10, maxiter=3)
    assert info > 0
    with pytest.raises(RuntimeError, match="did not converge"):
        solve_lin(Kff, ff[:, None], solver="topoptlab-pcg", solver_kw={"maxiter": 3})
    with pytest.raises(ValueError):
        solve_lin(Kff, ff[:, None], solver="no-such-solver")


def test_solve_lin_structured_operator(gpu_lib, golden):
    from topoptlab_gb300.context import GpuProblem
    from topoptlab_gb300.elements import lk_linear_elast_2d
    from topoptlab_gb300.solve_linsystem import StructuredOperator, solve_lin
    g = golden("mbb2d_60x20.npz")
    fixed, f = O.bc_mbb_2d(60, 20)
    prob = GpuProblem(60, 20, None, lk_linear_elast_2d(), fixed, f, 0.5, 2.4, rtol=1e-12)
    try:
        sol, _, _ = solve_lin(StructuredOperator(prob, g["xPhys_24"]), f[:, None],
                              solver="gb300-gmgpcg", solver_kw={"rtol": 1e-12})
    finally:
        prob.close()
    np.testing.assert_allclose(sol[:, 0], g["u_24"], rtol=0, atol=1e-9 * np.abs(g["u_24"]).max())
