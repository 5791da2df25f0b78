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


def _compose(d, tr, color, ambient, scale, brick, bf16=False):
    lib = _lib.load()
    dt = torch.bfloat16 if bf16 else torch.float32
    if brick:
        out = torch.empty((d.shape[0], ops.brick_cells(d.shape[1:4]), 4), dtype=dt, device=d.device)
    else:
        out = torch.empty(tuple(d.shape[:4]) + (4,), dtype=dt, device=d.device)
    layout = (ops.LAYOUT_BRICK if brick else 0) | (1 if bf16 else 0)  # | GFT_DTYPE_BF16
    with torch.cuda.device(d.device):
        _lib.check(lib.gft_light_compose(_p(d), _p(tr), _p(color), _shape(d), float(ambient), float(scale),
                                         layout, _p(out), _stream(d.device)), 'LightCompose')
    return out


def _compose_grad(d, tr, color, ambient, scale, brick, g):
    lib = _lib.load()
    g = g.contiguous()
    gd = torch.empty_like(d)
    gt = torch.empty_like(tr)
    layout = ops.LAYOUT_BRICK if brick else 0
    with torch.cuda.device(d.device):
        _lib.check(lib.gft_light_compose_grad(_p(d), _p(tr), _p(color), _shape(d), float(ambient), float(scale),
                                              layout, _p(g), _p(gd), _p(gt), _stream(d.device)), 'LightComposeGrad')
    return gd, gt


def _compose_factored(d, tr, fall, rgb, ambient, scale, bf16):
    lib = _lib.load()
    dt = torch.bfloat16 if bf16 else torch.float32
    out = torch.empty((d.shape[0], ops.brick_cells(d.shape[1:4]), 4), dtype=dt, device=d.device)
    layout = ops.LAYOUT_BRICK | (1 if bf16 else 0)  # | GFT_DTYPE_BF16
    with torch.cuda.device(d.device):
        _lib.check(lib.gft_light_compose_factored(_p(d), _p(tr), _p(fall), _p(rgb), _shape(d), float(ambient),
                                                  float(scale), layout, _p(out), _stream(d.device)),
                   'LightComposeFactored')
    return out


def compose_projection(rgb, ambient, scale):
    """The 8 floats projecting a 4-channel raymarch gradient onto the two sums
    the factored composition's adjoint reads (gft_light_compose_projection)."""
    lib = _lib.load()
    rgb = np.ascontiguousarray(np.asarray(rgb, dtype=np.float32).reshape(3))
    proj = np.zeros(8, np.float32)
    _lib.check(lib.gft_light_compose_projection(_p(rgb), float(ambient), float(scale), _p(proj)), 'ComposeProjection')
    return proj


def _compose_factored_grad_cameras(d, tr, fall, ncam, g2p, wsum):
    lib = _lib.load()
    gd = torch.empty_like(d)
    gt = torch.empty_like(tr)
    with torch.cuda.device(d.device):
        _lib.check(lib.gft_light_compose_factored_grad_cameras(_p(d), _p(tr), _p(fall), _shape(d), int(ncam), _p(g2p),
                                                               _p(wsum), _p(gd), _p(gt), _stream(d.device)),
                   'LightComposeFactoredGradCameras')
    return gd, gt


def _compose_factored_grad(d, tr, fall, g2):
    lib = _lib.load()
    g2 = g2.contiguous()
    gd = torch.empty_like(d)
    gt = torch.empty_like(tr)
    with torch.cuda.device(d.device):
        _lib.check(lib.gft_light_compose_factored_grad(_p(d), _p(tr), _p(fall), _shape(d), ops.LAYOUT_BRICK, _p(g2),
                                                       _p(gd), _p(gt), _stream(d.device)), 'LightComposeFactoredGrad')
    return gd, gt


class _ComposeRaymarch(torch.autograd.Function):
    """light_compose(brick=True) followed by the bricked raymarch, as one
    autograd op: the composition writes the raymarch input directly in its
    storage type (bf16 or fp32), and the raymarch's fp32 gradient reaches the
    composition's adjoint without being rounded to the storage type.

    With a factored light (rgb not None: color is the per-voxel falloff, the
    light colour falloff x rgb) the raymarch adjoint accumulates only the two
    projections of its 4-channel gradient that the composition's adjoint
    reads (gft_raymarch_grid_transform_grad_projected): half the reduction
    bytes (the deterministic adjoint: two integer sums per cell instead of
    four)."""

    @staticmethod
    def forward(ctx, d, tr, color, rgb, ambient, scale, grid, M, V, P, F, out_shape, boundary, blend, storage_dtype):
        bf16 = storage_dtype == torch.bfloat16
        if rgb is None:
            xs = _compose(d, tr, color, ambient, scale, True, bf16)
        else:
            xs = _compose_factored(d, tr, color, rgb, ambient, scale, bf16)
        need = ctx.needs_input_grad[0] or ctx.needs_input_grad[1]
        # a factored light's reference-normalised adjoint sums the weights in
        # its own pass: no weight pass ahead
        ctx.camera_sums = rgb is not None and ops.camera_sums_active()
        y, samples = ops._raymarch_forward_ctx(ctx, xs, need, M, V, P, F, out_shape, ops.FILTER['LINEAR'], boundary,
                                               blend, True, grid, weights_pass=not ctx.camera_sums)
        ctx.save_for_backward(d, tr, color, xs, y, samples)
        ctx.k = (float(ambient), float(scale))
        ctx.rgb = rgb
        ctx.args = (M, V, P, F, out_shape, ops.FILTER['LINEAR'], boundary, blend, True, grid)
        ctx.mark_non_differentiable(xs)
        ctx.set_materialize_grads(False)  # no zero-filled gradient for the stored input
        return y, xs

    @staticmethod
    def backward(ctx, dy, _dxs):
        d, tr, color, xs, y, samples = ctx.saved_tensors
        if dy is None:
            dy = torch.zeros_like(y)
        if ctx.rgb is None:
            g = ops._raymarch_backward_ctx(ctx, xs, y, samples, dy, *ctx.args)
            gd, gt = _compose_grad(d, tr, color, ctx.k[0], ctx.k[1], True, g)
        else:
            proj = compose_projection(ctx.rgb, *ctx.k)
            if ctx.camera_sums and ops.camera_sums_active():
                g2p, wsum = ops._raymarch_backward_ctx(ctx, xs, y, samples, dy, *ctx.args, projection=proj,
                                                       camera_sums=True)
                ncam = g2p.shape[0] // d.shape[0]
                gd, gt = _compose_factored_grad_cameras(d, tr, color, ncam, g2p, wsum)
                return (gd, gt) + (None,) * 13
            g2 = ops._raymarch_backward_ctx(ctx, xs, y, samples, dy, *ctx.args, projection=proj)
            gd, gt = _compose_factored_grad(d, tr, color, g2)
        return (gd, gt) + (None,) * 13


def render_bricked(density, transmittance, light_color, ambient, scale, matrix_m, matrix_v, matrix_p,
                   frustum_params, output_shape, boundary='BORDER', blending_mode='BEER_LAMBERT', storage_dtype=None):
    """raymarch_grid_transform_bricked(light_compose(density, transmittance,
    light_color, ambient, scale, brick=True), density's grid, ...) in one
    autograd op; with storage_dtype=torch.bfloat16 the composition writes the
    raymarch input in bf16 directly.  light_color: a [D, H, W, 3] colour grid,
    or a factored light (falloff [D, H, W, 1], rgb of 3 host floats) whose
    colour is falloff * rgb (a point or spot light; the adjoint then
    accumulates two channels instead of four).  Returns (images
    [1, V, H, W, 4], the raymarch input as stored: [1, brick_cells, 4], no
    gradient)."""
    d = _cuda(density, 'density')
    tr = _cuda(transmittance, 'transmittance')
    if d.dim() != 5 or d.shape[4] != 1 or tuple(tr.shape) != tuple(d.shape):
        raise _lib.GftInvalidArgument('density and transmittance must both be [N, D, H, W, 1]')
    nvox = int(np.prod(d.shape[1:4]))
    if isinstance(light_color, (tuple, list)):
        if len(light_color) != 2:
            raise _lib.GftInvalidArgument('a factored light is (falloff [D, H, W, 1], rgb [3])')
        color = _cuda(light_color[0], 'falloff')
        rgb = light_color[1]
        if isinstance(rgb, torch.Tensor):
            rgb = rgb.detach().cpu().numpy()
        rgb = np.ascontiguousarray(np.asarray(rgb, dtype=np.float32).reshape(3))
        if color.numel() != nvox or color.shape[-1] != 1:
            raise _lib.GftInvalidArgument('falloff must be [D, H, W, 1]')
    else:
        color = _cuda(light_color, 'light_color')
        rgb = None
        if color.numel() != nvox * 3 or color.shape[-1] != 3:
            raise _lib.GftInvalidArgument('light_color must be [D, H, W, 3]')
    if storage_dtype not in (None, torch.float32, torch.bfloat16):
        raise _lib.GftInvalidArgument('storage_dtype must be float32 or bfloat16')
    grid = tuple(int(v) for v in d.shape[1:4])
    return _ComposeRaymarch.apply(d, tr, color.detach(), rgb, ambient, scale, grid, matrix_m, matrix_v, matrix_p,
                                  frustum_params, ops._shape3(output_shape), ops._enum(ops.BOUNDARY, boundary, 'boundary'),
                                  ops._enum(ops.BLEND, blending_mode, 'blending_mode'), storage_dtype)


class _LightCompose(torch.autograd.Function):
    @staticmethod
    def forward(ctx, d, tr, color, ambient, scale, brick):
        out = _compose(d, tr, color, ambient, scale, brick)
        ctx.save_for_backward(d, tr, color)
        ctx.k = (float(ambient), float(scale), bool(brick))
        return out

    @staticmethod
    def backward(ctx, g):
        d, tr, color = ctx.saved_tensors
        ambient, scale, brick = ctx.k
        gd, gt = _compose_grad(d, tr, color, ambient, scale, brick, g)
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
