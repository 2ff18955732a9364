"""CPU oracle for the differentiable grid operators -- TEST INFRASTRUCTURE ONLY.

This package restates, in NumPy, the arithmetic of the reference's CUDA
operator layer (``phitest/render/cuda/src``): the trilinear / nearest /
min / max / quadratic samplers, the coordinate transforms, the blend
functions, the LUT and transform resample operators with their registered
gradients, the fused raymarch and its gradient, the depth reduce-blend and
the Python-composed MacCormack advection of density and MAC velocity.

Every function cites the reference file:line it follows.  Two gradient
semantics are provided: ``"exact"`` (the true adjoint of the forward,
checkable by finite differences) and ``"reference"`` (the reference's
sample-count / sample-weight normalised scatter, including its BORDER-mode
backward sampling positions).

Parity pin: the sampler, blend, transform, LUT-resample, transform-resample,
raymarch and reduce-blend arithmetic is checked against golden vectors that
``tests/golden/make_golden.py`` produced by compiling the reference's own
device code on the host (``oracle/refharness``).  The elementwise MacCormack
composition lives in TensorFlow in the reference and is not pinned that way;
it is restated from ``phitest/render/data_structures.py:1690-1737``.

Only ``tests/``, ``__graft_entry__.smoke()`` and the ``cpu_baseline`` leg of
``bench.py`` may import this package, and only as the checker / CPU
baseline -- never as a product code path.
"""

from . import core, ops, advect  # noqa: F401
