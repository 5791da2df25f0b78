"""GB300-native render + advect hot path of Global-Flow-Transport.

``gft.ops`` exposes the reference's op set (RaymarchGridTransform,
SampleGridTransform, SampleGridLut, LodTransform, ReduceGridBlend and their
gradients) plus the fused advection, all backed by libgft.so (hand-written
sm_103a CUDA behind a C ABI, include/gft.h).
"""
from . import _lib  # noqa: F401

__all__ = ['ops', 'synthetic']
