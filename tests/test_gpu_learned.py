"""Learned warm start on the GPU: forward pass and parameter gradient against
the CPU oracle (oracle/cnn.py, float64 autograd), training on solver-generated
pairs, the fallback rule, and what the trained network gains.

Tolerances: the GPU network runs in FP32 -- outputs within 1e-4 and
gradients within 2e-3 of the largest magnitude; solutions within the 1e-8
FP64 residual of the solver."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

from oracle import topopt as O


def _problem(nx, ny, nz, seed=None, **kw):
    from topoptlab_gb300.context import GpuProblem
    from topoptlab_gb300.elements import lk_linear_elast_3d
    fixed, f = O.bc_cantilever_3d(nx, ny, nz)
    prob = GpuProblem(nx, ny, nz, lk_linear_elast_3d(), fixed, f, 0.3, 1.5, precision="mixed",
                      rtol=1e-8, **kw)
    if seed is not None:
        from topoptlab_gb300 import _lib
        rng = np.random.default_rng(seed)
        x = rng.uniform(0.05, 1.0, nx * ny * nz)
        H, Hs = O.filter_matrix(nx, ny, nz, 1.5)
        xs = np.asarray(H @ x) / Hs
        prob.set(_lib.TG_FIELD_X, xs)
        prob.set(_lib.TG_FIELD_XPHYS, np.asarray(H @ xs) / Hs)
    return prob


def test_forward_and_gradient_match_oracle(gpu_lib):
    torch = pytest.importorskip("torch")
    from topoptlab_gb300.learned import LearnedWarmStart
    from oracle import cnn as N
    prob = _problem(16, 8, 8)
    net = LearnedWarmStart(prob, capacity=1, seed=3)
    try:
        info = net.info()
        grid = info["grid"]
        nn = grid[0] * grid[1] * grid[2]
        rng = np.random.default_rng(5)
        p = (rng.standard_normal(info["nparams"]) * 0.05).astype(np.float32)
        net.set_params(p)
        x0 = rng.standard_normal((nn, 7)).astype(np.float32)
        t = rng.standard_normal((nn, 3)).astype(np.float32)
        y, loss, g = net.eval(x0, t)
    finally:
        net.close()
        prob.close()
    loss_ref, g_ref, y_ref = N.loss_and_grad(p.astype(np.float64), x0, t, grid)
    np.testing.assert_allclose(y, y_ref, rtol=0, atol=1e-4 * np.abs(y_ref).max())
    np.testing.assert_allclose(loss, loss_ref, rtol=1e-4)
    np.testing.assert_allclose(g, g_ref, rtol=0, atol=2e-3 * np.abs(g_ref).max())


def test_tf32_inference_matches_oracle(gpu_lib):
    """The warm start's forward pass uses single TF32 products (10-bit operand
    mantissas, FP32 accumulation) instead of the split FP32-level ones: its
    output stays within 1e-2 of the largest output of the FP32 oracle, while
    the split pass (tg_cnn_eval) is within 1e-4."""
    pytest.importorskip("torch")
    from topoptlab_gb300.learned import LearnedWarmStart
    from oracle import cnn as N
    prob = _problem(16, 8, 8)
    net = LearnedWarmStart(prob, capacity=1, seed=3)
    try:
        info = net.info()
        grid = info["grid"]
        nn = grid[0] * grid[1] * grid[2]
        rng = np.random.default_rng(7)
        p = (rng.standard_normal(info["nparams"]) * 0.05).astype(np.float32)
        net.set_params(p)
        x0 = rng.standard_normal((nn, 7)).astype(np.float32)
        t = rng.standard_normal((nn, 3)).astype(np.float32)
        y_tf32 = net.infer(x0)
        y_split = net.eval(x0)
    finally:
        net.close()
        prob.close()
    _, _, y_ref = N.loss_and_grad(p.astype(np.float64), x0, t, grid)
    scale = np.abs(y_ref).max()
    np.testing.assert_allclose(y_split, y_ref, rtol=0, atol=1e-4 * scale)
    np.testing.assert_allclose(y_tf32, y_ref, rtol=0, atol=1e-2 * scale)


def test_training_fallback_and_gain(gpu_lib):
    """Train on pairs from optimisation runs started at seeded random
    densities, then run the same design iterations with and without the
    network: compliance agrees to the solver tolerance, the fallback flag is
    reported, and the PCG iteration counts of both runs are compared."""
    from topoptlab_gb300.learned import LearnedWarmStart
    nx, ny, nz = 32, 16, 16
    gen = _problem(nx, ny, nz, seed=1)
    net = LearnedWarmStart(gen, capacity=48, seed=0)
    try:
        for _ in range(24):
            net.record_step()
        loss = net.train(epochs=1, lr=1e-3, seed=0)
        loss2 = net.train(epochs=30, lr=1e-3, seed=1)
        assert np.isfinite(loss) and loss2 < loss
        # same run with and without the network
        base = _problem(nx, ny, nz)
        its_base = [base.step() for _ in range(12)]
        base.close()
        learned = _problem(nx, ny, nz)
        # the network is tied to the context it was created for: transfer the
        # trained weights to a network of the new context
        net2 = LearnedWarmStart(learned, capacity=0, seed=0)
        net2.set_params(net.params())
        net2.attach(learned)
        its_l = [learned.step() for _ in range(12)]
        net2.close()
        learned.close()
    finally:
        net.close()
        gen.close()
    ob = np.array([s.obj for s in its_base])
    ol = np.array([s.obj for s in its_l])
    np.testing.assert_allclose(ol, ob, rtol=1e-6)
    assert all(s.rel_res < 1e-8 for s in its_l)
    assert all(s.fallback in (0, 1) for s in its_l)
    pb = sum(s.pcg_iters for s in its_base[1:])
    pl = sum(s.pcg_iters for s in its_l[1:])
    print(f"PCG iterations, iterations 2-12: plain warm start {pb}, learned {pl}; "
          f"fallbacks {sum(s.fallback for s in its_l[1:])}/11")
