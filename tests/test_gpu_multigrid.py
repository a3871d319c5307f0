"""The production multigrid kernels against the oracle, through the C ABI.

Coarse levels with at least 150,000 (node, DOF) rows run the row-plane
stencil kernel (k_stencil_apply), smaller ones the small-grid kernel; only
the 1M-element workloads reach the first at their defaults.  tg_tune sets
the switch-over to 0 here, so the row-plane kernel runs every level of
grids the oracle handles in seconds, with deep hierarchies (4 levels at
32x16x16).

The mixed-precision V-cycle (FP32 arithmetic, BF16 scale factors in the
fine-level smoother, coarse levels built in FP32 from FP32 scale factors,
FP64 coarsest inverse) is checked in two parts:
  * every FP32 coarse stencil against the exact Galerkin operator of the
    FP32-rounded scale factors (oracle.gmg.round_f32), within 1e-5 of the
    largest coefficient (FP32 summation of the products);
  * the cycle against the oracle cycle evaluated exactly on the GPU's own
    coarse stencils and the BF16-rounded fine operator
    (oracle.gmg.round_bf16), within 1e-5 of the largest entry: what remains
    is the FP32 rounding of the sweeps and transfers.
The cycle against the fully exact oracle is looser than either part on
ill-conditioned coarse problems: on the 64x32 MBB beam (coarsest condition
number ~4e3) the FP32 construction error of the coarse operators moves the
coarse correction by ~4e-4 of the largest entry, on the 3-D cantilevers by
~1e-6.  FP64 cycles match the exact oracle within 1e-10."""
import numpy as np
import pytest

from oracle import topopt as O
from oracle import gmg as G

pytestmark = pytest.mark.gpu

GRIDS = [
    # (nelx, nely, nelz, kind, nlevels)
    (16, 8, 8, "elast", 3), (32, 16, 16, "elast", 4), (24, 16, 8, "elast", 3),
    (64, 32, None, "elast", 4), (48, 48, None, "poisson", 4),
]


@pytest.fixture
def row_plane_kernel(gpu_lib):
    from topoptlab_gb300 import _lib
    lib = _lib.load()
    assert lib.tg_tune(_lib.TG_TUNE_STENCIL_SMALL_PAIRS, 0) == _lib.TG_OK
    yield
    assert lib.tg_tune(_lib.TG_TUNE_STENCIL_SMALL_PAIRS, 150000) == _lib.TG_OK


def _case(nelx, nely, nelz, kind, nlevels, precision, seed):
    from topoptlab_gb300.context import GpuProblem
    rng = np.random.default_rng(seed)
    ndim = 2 if nelz is None else 3
    KE = O.ke_elast(ndim) if kind == "elast" else O.ke_poisson(ndim)
    nnd = ndim if kind == "elast" else 1
    dims = (nelx, nely) if ndim == 2 else (nelx, nely, nelz)
    ndof = nnd * int(np.prod(np.array(dims) + 1))
    if kind == "elast" and ndim == 2:
        fixed, f = O.bc_mbb_2d(nelx, nely)
    elif kind == "elast":
        fixed, f = O.bc_cantilever_3d(nelx, nely, nelz)
    else:
        fixed = np.arange(0, nely + 1)
        f = np.full(ndof, 0.01)
    prob = GpuProblem(nelx, nely, nelz, KE, fixed, f, 0.5, 1.5, nlevels=nlevels,
                      precision=precision)
    x = rng.uniform(0.05, 1.0, int(np.prod(dims)))
    mask = np.zeros(ndof, bool)
    mask[fixed] = True
    b = rng.standard_normal(ndof) * ~mask
    edof = O.edofmat(nelx, nely, nelz, nnd)
    return prob, KE, edof, x, b, mask, dims, nnd, ndof


def _oracle_cycle(KE, edof, x, mask, dims, nnd, ndof, nlevels, mixed, coarse_ops=None):
    s = O.simp(x)
    if not mixed:
        K = O.assemble(KE, edof, s, ndof)
        return G.Hierarchy(K, mask, dims, nnd, nlevels)
    K16 = O.assemble(KE, edof, G.round_bf16(s), ndof)
    K32 = O.assemble(KE, edof, G.round_f32(s), ndof)
    return G.Hierarchy(K16, mask, dims, nnd, nlevels, K_build=K32, coarse_ops=coarse_ops)


def _run(grid, precision, seed):
    nelx, nely, nelz, kind, nlevels = grid
    prob, KE, edof, x, b, mask, dims, nnd, ndof = _case(nelx, nely, nelz, kind, nlevels,
                                                        precision, seed)
    try:
        assert prob.levels()[0] == nlevels
        z = prob.vcycle(x, b, precision=precision)
        ops = None
        if precision == "mixed":
            ops = [G.stencil_matrix(prob.coarse_stencil(x, lvl), [d // 2 ** lvl for d in dims], nnd)
                   for lvl in range(1, nlevels)]
    finally:
        prob.close()
    h = _oracle_cycle(KE, edof, x, mask, dims, nnd, ndof, nlevels, precision == "mixed")
    if ops is None:
        return z, h.vcycle(b)
    for lvl, A in enumerate(ops, start=1):
        Ar = h.A[lvl]
        err = abs(A - Ar).max()
        assert err <= 1e-5 * abs(Ar).max(), (lvl, err / abs(Ar).max())
    hg = _oracle_cycle(KE, edof, x, mask, dims, nnd, ndof, nlevels, True, coarse_ops=ops)
    return z, hg.vcycle(b)


@pytest.mark.parametrize("grid", GRIDS)
def test_row_plane_stencil_vcycle_fp64(row_plane_kernel, grid):
    z, zr = _run(grid, "fp64", 21)
    np.testing.assert_allclose(z, zr, rtol=0, atol=1e-10 * np.abs(zr).max())


@pytest.mark.parametrize("grid", GRIDS)
def test_row_plane_stencil_vcycle_mixed(row_plane_kernel, grid):
    z, zr = _run(grid, "mixed", 22)
    np.testing.assert_allclose(z, zr, rtol=0, atol=1e-5 * np.abs(zr).max())


@pytest.mark.parametrize("grid", GRIDS)
def test_small_grid_stencil_vcycle_mixed(gpu_lib, grid):
    z, zr = _run(grid, "mixed", 23)
    np.testing.assert_allclose(z, zr, rtol=0, atol=1e-5 * np.abs(zr).max())
