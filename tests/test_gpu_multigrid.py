"""The production multigrid kernels against the oracle, through the C ABI.

Coarse levels with at least 150,000 (node, DOF) rows run the row-plane
stencil kernel (k_stencil_apply), smaller ones the small-grid kernel; only
the 1M-element workloads reach the first at their defaults.  tg_tune sets
the switch-over to 0 here, so the row-plane kernel runs every level of
grids the oracle handles in seconds, with deep hierarchies (4 levels at
32x16x16).

The mixed-precision V-cycle (FP32 arithmetic, BF16 scale factors in the
fine-level smoother, coarse levels built from FP32 scale factors, FP64
coarsest inverse) is compared with the oracle cycle evaluated exactly on
the same rounded scale factors (oracle.gmg.round_bf16 / round_f32): what
separates them is the FP32 rounding of the arithmetic, bounded by the
tolerance 2e-4 of the largest entry (FP64 cycles: 1e-10)."""
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


def _oracle_cycle(KE, edof, x, mask, dims, nnd, ndof, nlevels, mixed):
    s = O.simp(x)
    if not mixed:
        K = O.assemble(KE, edof, s, ndof)
        return G.Hierarchy(K, mask, dims, nnd, nlevels)
    K16 = O.assemble(KE, edof, G.round_bf16(s), ndof)
    K32 = O.assemble(KE, edof, G.round_f32(s), ndof)
    return G.Hierarchy(K16, mask, dims, nnd, nlevels, K_build=K32)


def _run(grid, precision, seed):
    nelx, nely, nelz, kind, nlevels = grid
    prob, KE, edof, x, b, mask, dims, nnd, ndof = _case(nelx, nely, nelz, kind, nlevels,
                                                        precision, seed)
    try:
        assert prob.levels()[0] == nlevels
        z = prob.vcycle(x, b, precision=precision)
    finally:
        prob.close()
    h = _oracle_cycle(KE, edof, x, mask, dims, nnd, ndof, nlevels, precision == "mixed")
    return z, h.vcycle(b)


@pytest.mark.parametrize("grid", GRIDS)
def test_row_plane_stencil_vcycle_fp64(row_plane_kernel, grid):
    z, zr = _run(grid, "fp64", 21)
    np.testing.assert_allclose(z, zr, rtol=0, atol=1e-10 * np.abs(zr).max())


@pytest.mark.parametrize("grid", GRIDS)
def test_row_plane_stencil_vcycle_mixed(row_plane_kernel, grid):
    z, zr = _run(grid, "mixed", 22)
    np.testing.assert_allclose(z, zr, rtol=0, atol=2e-4 * np.abs(zr).max())


@pytest.mark.parametrize("grid", GRIDS)
def test_small_grid_stencil_vcycle_mixed(gpu_lib, grid):
    z, zr = _run(grid, "mixed", 23)
    np.testing.assert_allclose(z, zr, rtol=0, atol=2e-4 * np.abs(zr).max())
