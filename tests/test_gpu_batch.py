"""A batch of heat plates of uneven sizes (odd sizes run on padded device
grids) stepped concurrently through tg_step_many: every design's results
equal those of stepping it alone, and the mixed-precision batch agrees with
the plain FP64 batch per design at the 1e-8 FP64 residual."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_heat_plate_batch_concurrent_equals_single_and_fp64(gpu_lib):
    from topoptlab_gb300.batch import heat_plate_batch, heat_plate_sizes
    sizes = heat_plate_sizes(6, seed=1, nmin=20, nmax=90)
    assert any(n % 2 for n in sizes)
    mixed = heat_plate_batch(sizes, precision="mixed", nthreads=4)
    plain = heat_plate_batch(sizes, precision="fp64")
    single = heat_plate_batch(sizes, precision="mixed")
    try:
        for _ in range(3):
            rm, rp = mixed.step(), plain.step()
            rs = [p.step() for p in single.problems]          # one after another
            for a, b, s in zip(rm, rp, rs):
                assert a.rel_res <= 1e-8 and b.rel_res <= 1e-8
                assert a.obj == s.obj and a.pcg_iters == s.pcg_iters
                np.testing.assert_allclose(a.obj, b.obj, rtol=1e-7)
        for pm, ps in zip(mixed.problems, single.problems):
            np.testing.assert_array_equal(pm.get(0), ps.get(0))
    finally:
        mixed.close()
        plain.close()
        single.close()


def test_element_source_load(gpu_lib):
    """0.01 per element, split over the element's 4 nodes: total 0.01 * nel."""
    from topoptlab_gb300.example_bc import heatplate_2d, heatplate_2d_element_source
    u, f, fixed, free, _ = heatplate_2d_element_source(10, 10, 121)
    _, _, fixed_ref, _, _ = heatplate_2d(10, 10, 121)
    assert np.isclose(f.sum(), 0.01 * 100)
    assert f[0, 0] == 0.0025 and f[12, 0] == 0.01
    np.testing.assert_array_equal(fixed, fixed_ref)
