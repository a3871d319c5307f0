"""Filter objects of the reference's modular interface (filter/filter.py:7-94):
the abstract base and the argument checks need no GPU."""
import numpy as np
import pytest

from topoptlab_gb300.filter import HelmholtzFilter, MatrixFilter, TOFilter


def test_tofilter_is_abstract():
    with pytest.raises(TypeError):
        TOFilter()


def test_matrix_filter_rejects_periodic_boundaries():
    with pytest.raises(ValueError):
        MatrixFilter(nelx=6, nely=4, rmin=1.5, pbc=True)
    with pytest.raises(ValueError):
        MatrixFilter(nelx=6, nely=4, rmin=1.5, pbc=np.array([True, False]))


def test_helmholtz_filter_is_2d_like_the_reference():
    """assemble_helmholtz_filter raises NotImplementedError for 3-D
    (filter/helmholtz_filter.py:180)."""
    with pytest.raises(NotImplementedError):
        HelmholtzFilter(nelx=4, nely=4, rmin=1.5, nelz=4)
