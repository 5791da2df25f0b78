"""Drop-in replacement of phitest/render/cuda/ops_loader.py.

The reference loads three TensorFlow op libraries (ops_loader.py:11-12, :55-56,
:65-66) and registers their gradients (:14-31, :35-51, :57-60, :67-83).  Here
the same op handles are backed by libgft.so through gft.ops; each forward op is
a torch.autograd.Function whose backward is the matching gradient op, so the
registered-gradient behaviour is the same.
"""
from types import SimpleNamespace

from gft import ops as _ops

sampling_ops = SimpleNamespace(
    sample_grid_transform=_ops.sample_grid_transform,
    sample_grid_transform_grad=_ops.sample_grid_transform_grad,
    sample_grid_lut=_ops.sample_grid_lut,
    sample_grid_lut_grad=_ops.sample_grid_lut_grad,
    lod_transform=_ops.lod_transform,
)
sample_grid_transform = sampling_ops.sample_grid_transform
sample_grid_lut = sampling_ops.sample_grid_lut

blending_ops = SimpleNamespace(
    reduce_grid_blend=_ops.reduce_grid_blend,
    reduce_grid_blend_grad=_ops.reduce_grid_blend_grad,
)
reduce_grid_blend = blending_ops.reduce_grid_blend

raymarching_ops = SimpleNamespace(
    raymarch_grid_transform=_ops.raymarch_grid_transform,
    raymarch_grid_transform_grad=_ops.raymarch_grid_transform_grad,
)
raymarch_grid_transform = raymarching_ops.raymarch_grid_transform
