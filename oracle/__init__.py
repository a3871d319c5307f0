"""CPU oracle for the SIMP compliance loop -- TEST INFRASTRUCTURE ONLY.

This package restates, in NumPy/SciPy, the reference topoptlab algorithm for
the per-iteration SIMP compliance-minimisation loop on structured quad4/hex8
grids, plus the FP64 geometric-multigrid PCG and the small CNN that the GPU
library adds.  It exists to check the CUDA library, never to stand in for it:
only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline
leg may import it.  The product package (``topoptlab_gb300``) never imports
anything from here and fails loudly when its CUDA library is missing.

Pinning: ``tests/test_oracle_golden.py`` checks every function here against
fixtures generated by running the reference itself
(``tests/golden/make_golden.py``) -- edofMat, KE, filter matrices, boundary
conditions and whole optimisation trajectories.  The GMG-PCG and the CNN have
no counterpart in the reference; their parity is anchored on the FP64 residual
and on the reference direct-solve trajectories.
"""
