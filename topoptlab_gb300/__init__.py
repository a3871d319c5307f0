"""GB300 (sm_103a) implementation of topoptlab's SIMP compliance loop.

The per-iteration hot path (matrix-free K.u, GMG-PCG in FP64 or mixed
precision, compliance + sensitivities, distance filter, OC update) runs in
hand-written CUDA kernels of libtopopt_gb300.so, reached through a C ABI
(include/topopt_gb300.h).  ``main`` is a drop-in for
topoptlab.topology_optimization.main.
"""
from .topology_optimization import main
from .context import GpuProblem
from .filter import HelmholtzFilter, MatrixFilter, TOFilter

__all__ = ["main", "GpuProblem", "MatrixFilter", "HelmholtzFilter", "TOFilter"]
