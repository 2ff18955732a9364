"""GB300-native differentiable grid operators of Neural-Global-Transport's
reconstruction loop: frustum / LUT grid resampling, emission-absorption
raymarch and depth blend, and semi-Lagrangian / MacCormack advection of
density and MAC-staggered velocity, each with forward and backward kernels
written for sm_103a behind a C-ABI library (``libngt_ops.so``).

The package directory is ``neural-global-transport_gb300``; it is imported
under the name ``ngt_gb300`` (see ``__graft_entry__.load_package``).
"""
from . import scene, synthetic  # noqa: F401

__all__ = ["scene", "synthetic"]
