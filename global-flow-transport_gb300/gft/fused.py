"""Fused kernels for the glue of the render + advect step (libgft.so
gft_transmittance / gft_light_compose / gft_image_loss and their gradients).

Each function is an autograd op equal to a composition of tensor ops of the
reference's renderer; ``gft.pipeline`` uses them in its batched mode and keeps
the plain tensor composition in its plain mode.
"""
import numpy as np
import torch

from . import _lib
from . import ops
from .ops import _cuda, _p, _stream, _workspace


def _shape(t):
    return _lib.i64(t.shape)


class _Transmittance(torch.autograd.Function):
    @staticmethod
    def forward(ctx, x):
        lib = _lib.load()
        out = torch.empty_like(x)
        with torch.cuda.device(x.device):
            _lib.check(lib.gft_transmittance(_p(x), _shape(x), _p(out), _stream(x.device)), 'Transmittance')
        ctx.save_for_backward(out)
        return out

    @staticmethod
    def backward(ctx, g):
        (out,) = ctx.saved_tensors
        lib = _lib.load()
        g = g.contiguous()
        gx = torch.empty_like(out)
        with torch.cuda.device(out.device):
            _lib.check(lib.gft_transmittance_grad(_p(out), _p(g), _shape(out), _p(gx), _stream(out.device)),
                       'TransmittanceGrad')
        return gx


def transmittance(x):
    """exp(-exclusive depth sum) of a [N, D, H, W, 1] grid: equals
    exp(-cat([0, reduce_grid_blend(x, 'BEER_LAMBERT', keep_dims=True)[:, :-1]], 1))."""
    x = _cuda(x, 'input')
    if x.dim() != 5 or x.shape[4] != 1:
        raise _lib.GftInvalidArgument('expected [N, D, H, W, 1], got %s' % (tuple(x.shape),))
    return _Transmittance.apply(x)


class _LightCompose(torch.autograd.Function):
    @staticmethod
    def forward(ctx, d, tr, color, ambient, scale, brick):
        lib = _lib.load()
        if brick:
            out = torch.empty((d.shape[0], ops.brick_cells(d.shape[1:4]), 4), dtype=torch.float32, device=d.device)
        else:
            out = torch.empty(tuple(d.shape[:4]) + (4,), dtype=torch.float32, device=d.device)
        layout = ops.LAYOUT_BRICK if brick else 0
        with torch.cuda.device(d.device):
            _lib.check(lib.gft_light_compose(_p(d), _p(tr), _p(color), _shape(d), float(ambient), float(scale),
                                             layout, _p(out), _stream(d.device)), 'LightCompose')
        ctx.save_for_backward(d, tr, color)
        ctx.k = (float(ambient), float(scale), layout)
        return out

    @staticmethod
    def backward(ctx, g):
        d, tr, color = ctx.saved_tensors
        ambient, scale, layout = ctx.k
        lib = _lib.load()
        g = g.contiguous()
        gd = torch.empty_like(d)
        gt = torch.empty_like(tr)
        with torch.cuda.device(d.device):
            _lib.check(lib.gft_light_compose_grad(_p(d), _p(tr), _p(color), _shape(d), ambient, scale, layout,
                                                  _p(g), _p(gd), _p(gt), _stream(d.device)), 'LightComposeGrad')
        return gd, gt, None, None, None, None


def light_compose(density, transmittance, light_color, ambient, scale, brick=False):
    """cat([density * (transmittance * light_color + ambient), density], -1) * scale
    for density, transmittance [N, D, H, W, 1] and light_color [D, H, W, 3] or
    [1, D, H, W, 3] (constant: no gradient).  ``brick``: the result in the
    raymarch's 2x2x2 brick layout, [N, brick_cells(D, H, W), 4], for
    ops.raymarch_grid_transform_bricked."""
    d = _cuda(density, 'density')
    tr = _cuda(transmittance, 'transmittance')
    color = _cuda(light_color, 'light_color')
    if d.dim() != 5 or d.shape[4] != 1 or tuple(tr.shape) != tuple(d.shape):
        raise _lib.GftInvalidArgument('density and transmittance must both be [N, D, H, W, 1]')
    if color.numel() != int(np.prod(d.shape[1:4])) * 3 or color.shape[-1] != 3:
        raise _lib.GftInvalidArgument('light_color must be [D, H, W, 3]')
    return _LightCompose.apply(d, tr, color.detach(), ambient, scale, bool(brick))


TONEMAP = {'NONE': 0, 'CLIP_NEGATIVE': 1, 'SATURATE': 2, 'NORMALIZE': 3}


class _ImageLoss(torch.autograd.Function):
    @staticmethod
    def forward(ctx, img, target, bkg, tonemap):
        lib = _lib.load()
        npix = img.numel() // 4
        loss = torch.empty((), dtype=torch.float32, device=img.device)
        ws = _workspace(lib.gft_image_loss_workspace_size(npix), img.device)
        with torch.cuda.device(img.device):
            _lib.check(lib.gft_image_loss_tonemap(_p(img), _p(target), _p(bkg), npix, tonemap, _p(loss), _p(ws),
                                                  ws.numel(), _stream(img.device)), 'ImageLoss')
        ctx.save_for_backward(img, target, ws)
        ctx.bkg = bkg
        ctx.tonemap = tonemap
        return loss

    @staticmethod
    def backward(ctx, g):
        img, target, ws = ctx.saved_tensors
        lib = _lib.load()
        gi = torch.empty_like(img)
        g = g.contiguous()
        with torch.cuda.device(img.device):
            _lib.check(lib.gft_image_loss_tonemap_grad(_p(img), _p(target), _p(ctx.bkg), img.numel() // 4,
                                                       ctx.tonemap, _p(g), _p(gi), _p(ws), ws.numel(),
                                                       _stream(img.device)), 'ImageLossGrad')
        return gi, None, None, None


def image_loss(image, target, background, tonemap='NONE'):
    """mean((tone(image[..., :3] + background * exp(-image[..., 3:])) - target) ** 2)
    for image [..., 4], target [..., 3] and a background colour of 3 floats
    (host values; a CUDA tensor is copied to the host, which a CUDA-graph
    capture does not allow).  tonemap: the renderer's tonemapping, 'NONE',
    'CLIP_NEGATIVE', 'SATURATE' or 'NORMALIZE' (over all pixels of the call)."""
    img = _cuda(image, 'image')
    tgt = _cuda(target, 'target')
    if img.shape[-1] != 4 or tuple(tgt.shape) != tuple(img.shape[:-1]) + (3,):
        raise _lib.GftInvalidArgument('image must be [..., 4] and target [..., 3] of the same pixels')
    tm = str(tonemap).upper()
    if tm not in TONEMAP:
        raise _lib.GftInvalidArgument('unknown tonemapping %r' % (tonemap,))
    if isinstance(background, torch.Tensor):
        background = background.detach().cpu().numpy()
    bkg = np.ascontiguousarray(np.asarray(background, dtype=np.float32).reshape(3))
    return _ImageLoss.apply(img, tgt, bkg, TONEMAP[tm])


def transmittance_check(x, tr, column_stride=1, out=None):
    """FP64 recomputation of transmittance(x) on every column_stride-th
    column: a device float64 tensor [max |tr - tr64|, max |tr64|]
    (written into ``out`` when given, e.g. a slice of a buffer a captured
    step reads back)."""
    x = _cuda(x, 'input')
    tr = _cuda(tr, 'output')
    if x.shape != tr.shape or x.dim() != 5 or x.shape[4] != 1:
        raise _lib.GftInvalidArgument('expected two [N, D, H, W, 1] grids, got %s and %s'
                                      % (tuple(x.shape), tuple(tr.shape)))
    res = out if out is not None else torch.empty(2, dtype=torch.float64, device=x.device)
    lib = _lib.load()
    with torch.cuda.device(x.device):
        _lib.check(lib.gft_transmittance_check(_p(x), _p(tr), _shape(x), int(column_stride), _p(res),
                                               _stream(x.device)), 'TransmittanceCheck')
    return res
