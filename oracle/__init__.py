"""FP64 NumPy oracle of the Global-Flow-Transport render + advect hot path.

TEST INFRASTRUCTURE ONLY.  This package restates, on the CPU in float64, the
semantics of the reference's CUDA ops (phitest/render/cuda/src/*.cu.cc) and of
the Python composition around them (phitest/render/{renderer,lighting,
data_structures}.py).  It is imported only by ``tests/``, by
``__graft_entry__.smoke()`` (as the checker) and by ``bench.py``'s CPU-baseline
legs.  The product (the CUDA library and its Python wrappers) never imports it.

Parity is pinned against outputs of the reference's own CUDA kernels, compiled
from the reference sources by ``oracle/ref/build_ref.sh`` and run on a GB300 by
``tests/golden/make_golden.py``; the resulting fixtures live in
``tests/golden/*.npz`` and ``tests/test_oracle_golden.py`` checks this oracle
against them.

Modules:
  sampling   -- trilinear / nearest / min / max fetches, boundaries, mips, LOD
  transforms -- IDX <-> NDC <-> VS <-> OS chains incl. linear depth
  blend      -- blend functors and the depth reduce-blend op (+ adjoint)
  raymarch   -- fused raymarch op (+ adjoint, exact and reference-normalised)
  resample   -- SampleGridTransform / SampleGridLut ops (+ adjoints)
  advect     -- staggered -> centred, SL / MacCormack / MC_SMOOTH (+ adjoint)
  render     -- light grid, shadow pass, render_density composition
"""
