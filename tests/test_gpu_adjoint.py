"""The adjoint path of objectives that are not self-adjoint
(topology_optimization.py:473-500): tg_adjoint solves K adj = rhs_adj with
the operator and hierarchy of the last state solve and returns the
sensitivity simp_dx(xPhys) adj_e^T KE u_e, against the oracle's direct
adjoint solve.  Tolerances: solves to a 1e-10 relative residual, results
within 1e-7 of the largest entry."""
import numpy as np
import pytest

from oracle import topopt as O

pytestmark = pytest.mark.gpu


def _oracle_sens(x, u, adj, KE, edof):
    return O.simp_dx(x) * np.einsum("ei,ij,ej->e", adj[edof], KE, u[edof])


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_compliance_adjoint_is_minus_u(gpu_lib, precision):
    """Compliance f^T u is self-adjoint: the reference skips the solve and
    uses -u as the adjoint (objectives.py:51-55).  Solving K adj = -f must
    give that -u and the compliance sensitivities."""
    from topoptlab_gb300.context import GpuProblem
    nx, ny = 32, 16
    KE = O.ke_elast(2)
    fixed, f = O.bc_mbb_2d(nx, ny)
    x = np.random.default_rng(2).uniform(0.1, 1.0, nx * ny)
    prob = GpuProblem(nx, ny, None, KE, fixed, f, 0.5, 1.5, rtol=1e-10, precision=precision)
    try:
        u, _ = prob.solve(x, f)
        adj, dobj, info = prob.adjoint(u, -f)
        obj, dc = prob.compliance(x, u)
    finally:
        prob.close()
    assert info["converged"] == 1
    np.testing.assert_allclose(adj, -u, rtol=0, atol=1e-8 * np.abs(u).max())
    np.testing.assert_allclose(dobj, dc, rtol=0, atol=1e-7 * np.abs(dc).max())


@pytest.mark.parametrize("dims", [(24, 12, None), (12, 6, 6)])
def test_displacement_objective_adjoint(gpu_lib, dims):
    """A displacement objective like the reference's var_maximization
    (objectives.py:121-157: rhs_adj = l, an indicator of output DOFs): adjoint
    solution and sensitivities against the oracle's direct solves."""
    from topoptlab_gb300.context import GpuProblem
    nx, ny, nz = dims
    ndim = 2 if nz is None else 3
    KE = O.ke_elast(ndim)
    fixed, f = (O.bc_mbb_2d(nx, ny) if ndim == 2 else O.bc_cantilever_3d(nx, ny, nz))
    ndof = f.shape[0]
    rng = np.random.default_rng(3)
    x = rng.uniform(0.1, 1.0, int(np.prod([d for d in dims if d])))
    l = np.zeros(ndof)
    l[rng.choice(np.setdiff1d(np.arange(ndof), fixed), 3, replace=False)] = -1.0
    prob = GpuProblem(nx, ny, nz, KE, fixed, f, 0.5, 1.5, rtol=1e-10)
    try:
        u, _ = prob.solve(x, f)
        adj, dobj, info = prob.adjoint(u, l)
    finally:
        prob.close()
    edof = O.edofmat(nx, ny, nz, ndim)
    K = O.assemble(KE, edof, O.simp(x), ndof)
    free = np.setdiff1d(np.arange(ndof), fixed)
    ud = O.solve_direct(K, f, free)
    ad = O.solve_direct(K, l, free)
    np.testing.assert_allclose(u, ud, rtol=0, atol=1e-7 * np.abs(ud).max())
    np.testing.assert_allclose(adj, ad, rtol=0, atol=1e-7 * np.abs(ad).max())
    dref = _oracle_sens(x, ud, ad, KE, edof)
    np.testing.assert_allclose(dobj, dref, rtol=0, atol=1e-7 * np.abs(dref).max())
