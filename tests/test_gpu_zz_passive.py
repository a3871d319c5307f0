"""Passive elements through the drop-in driver (tests/test_passive.py:8-34 of
the reference): the 60x20 cantilever with a passive disc, ft=0."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

OUT = {"file": None, "display": False, "export": False, "write_log": False,
       "profile": False, "debug": 0}


def test_passive_disc_cantilever(gpu_lib, golden):
    from topoptlab_gb300 import main
    from topoptlab_gb300.example_bc import cantilever_2d
    from topoptlab_gb300.geometries import sphere
    g = golden("cant2d_60x20_passive.npz")
    flags = sphere(nelx=60, nely=20, center=(60 / 3 - 1, 20 / 2 - 1), radius=20 / 3)
    x, obj = main(nelx=60, nely=20, volfrac=0.5, rmin=2.4, ft=0, el_flags=flags,
                  filter_mode="matrix", optimizer="oc", bcs=cantilever_2d,
                  lin_solver_kw={"name": "scipy-direct"}, output_kw=dict(OUT))
    np.testing.assert_almost_equal(obj, 221.9720563724, decimal=2)
    np.testing.assert_allclose(obj, float(g["final_obj"]), rtol=1e-8)
    np.testing.assert_allclose(x[:, 0], g["final_x"], atol=1e-7)
    assert np.all(x[flags == 1, 0] == 0.0)
