"""PyTorch-facing ops over libgft.so with the reference op signatures.

Each forward op mirrors one TensorFlow op of the reference
(phitest/render/cuda/ops_loader.py:11-85): same argument names, attribute
strings and output layouts; the gradient ops are registered as the autograd
backward exactly as ops_loader.py registers them with TF.  Tensors are CUDA
tensors (NDHWC, fp32, or bf16 storage where noted); matrices and frustum
parameters are host arrays as in the reference (HostMemory inputs).
"""
import ctypes

import numpy as np
import torch

from . import _lib

FILTER = {'NEAREST': 0, 'LINEAR': 1, 'MIN': 2, 'MAX': 3}
BOUNDARY = {'BORDER': 0, 'CLAMP': 1, 'WRAP': 2}
MIP = {'NONE': 0, 'NEAREST': 1, 'LINEAR': 2}
BLEND = {'BEER_LAMBERT': 0, 'BEER_LAMBERT_EXCLUSIVE': 1, 'ALPHA': 2, 'ALPHA_ADDITIVE': 3, 'ADDITIVE': 4}
COORD = {'TRANSFORM_LINDEPTH': 0, 'TRANSFORM_LINDEPTH_REVERSE': 1, 'TRANSFORM': 3, 'TRANSFORM_REVERSE': 4}
GRAD = {'REFERENCE': 0, 'EXACT': 1}
KNOB_WEIGHTS_PIPELINE = 5  # GFT_KNOB_WEIGHTS_PIPELINE
CLAMP = {'NONE': 0, 'MC_SMOOTH': 1, 'NEGATIVE': 2}

_state = {'grad_mode': 'REFERENCE', 'side_weights': True, 'sample_store': True, 'sample_pool': 0.25,
          'deterministic': False, 'camera_sums': False}
DETERMINISTIC = 0x400  # GFT_GRAD_DETERMINISTIC
CAMERA_SUMS = 0x800  # GFT_GRAD_CAMERA_SUMS


def set_raymarch_camera_sums(enabled):
    """The reference-normalised adjoint of the fused render with a factored
    light (gft.fused.render_bricked) in one pass: per camera the projected
    value sums and the weight sums from the same walk over the samples, the
    division per voxel afterwards (gft.h GFT_GRAD_CAMERA_SUMS), instead of a
    separate weight pass before a normalised scatter.  Off by default: the
    one-pass scatter does both reductions and is slower than the weight pass
    running beside the forward kernels plus the normalised scatter (cfg5
    step 9.00 against 8.61 ms)."""
    _state['camera_sums'] = bool(enabled)


def camera_sums_active():
    """Whether a fused render's reference-normalised adjoint uses per-camera
    sums now (then no weight pass runs ahead of it)."""
    return _state['camera_sums'] and _state['grad_mode'] == 'REFERENCE' and not _state['deterministic']


def set_deterministic(enabled):
    """Deterministic gradients of the raymarch and advection ops: their
    scatters add fixed-point integers instead of floats (gft.h
    GFT_GRAD_DETERMINISTIC), so repeated backward passes give bit-identical
    gradients.  Raymarch: BEER_LAMBERT or ADDITIVE blending."""
    _state['deterministic'] = bool(enabled)


def is_deterministic():
    return _state['deterministic']


class deterministic:
    """Context manager switching deterministic gradients on (or off)."""

    def __init__(self, enabled=True):
        self.enabled = bool(enabled)

    def __enter__(self):
        self.prev = _state['deterministic']
        _state['deterministic'] = self.enabled

    def __exit__(self, *a):
        _state['deterministic'] = self.prev


def _scatter_gmode():
    """grad_mode of the raymarch and advection gradient calls."""
    return GRAD[get_grad_mode()] | (DETERMINISTIC if _state['deterministic'] else 0)


def set_grad_mode(mode):
    """'REFERENCE' (default): gradients normalised like the reference ops;
    'EXACT': true adjoints of the forward ops."""
    mode = mode.upper()
    if mode not in GRAD:
        raise ValueError(mode)
    _state['grad_mode'] = mode


def get_grad_mode():
    return _state['grad_mode']


class side_stream_weights:
    """Context manager: whether a differentiable raymarch forward starts its
    gradient's weight pass on a side stream (default) or leaves it to the
    backward.  Disable it where a forward's backward may never run, e.g. the
    first forward of a checkpointed segment (which the backward recomputes)."""

    def __init__(self, enabled):
        self.enabled = bool(enabled)

    def __enter__(self):
        self.prev = _state['side_weights']
        _state['side_weights'] = self.enabled

    def __exit__(self, *a):
        _state['side_weights'] = self.prev


class grad_mode:
    """Context manager switching the gradient mode."""

    def __init__(self, mode):
        self.mode = mode

    def __enter__(self):
        self.prev = get_grad_mode()
        set_grad_mode(self.mode)

    def __exit__(self, *a):
        set_grad_mode(self.prev)


def _enum(table, v, what):
    if isinstance(v, bytes):
        v = v.decode()
    if isinstance(v, str):
        key = v.upper()
        if key not in table:
            raise _lib.GftInvalidArgument('invalid %s %r' % (what, v))
        return table[key]
    return int(v)


def _host(x, tail):
    if isinstance(x, torch.Tensor):
        x = x.detach().cpu().numpy()
    a = np.ascontiguousarray(np.asarray(x, dtype=np.float32))
    if a.shape == tail:
        a = a[None]
    if a.shape[1:] != tail:
        raise _lib.GftInvalidArgument('expected shape %s or (K,)+%s, got %s' % (tail, tail, a.shape))
    return a


def _mats(m):
    a = _host(m, (4, 4))
    return a, a.shape[0]


def _frustum(f):
    a = _host(f, (6,))
    return a, a.shape[0]


def _p(a):
    if a is None:
        return None
    if isinstance(a, np.ndarray):
        return a.ctypes.data_as(ctypes.c_void_p)
    return ctypes.c_void_p(a.data_ptr())


def _cuda(t, name, dtypes=(torch.float32,)):
    if not isinstance(t, torch.Tensor) or not t.is_cuda:
        raise _lib.GftInvalidArgument('%s must be a CUDA tensor' % name)
    if t.dtype not in dtypes:
        raise _lib.GftInvalidArgument('%s must have dtype in %s, got %s' % (name, dtypes, t.dtype))
    return t.contiguous()


def _dtype_code(t):
    return 1 if t.dtype == torch.bfloat16 else 0


def _stream(dev):
    return ctypes.c_void_p(torch.cuda.current_stream(dev).cuda_stream)


def _workspace(nbytes, dev):
    return torch.empty(max(int(nbytes), 1), dtype=torch.uint8, device=dev)


def _shape3(s):
    s = [int(v) for v in (s.tolist() if isinstance(s, (np.ndarray, torch.Tensor)) else s)]
    if len(s) != 3:
        raise _lib.GftInvalidArgument('Invalid output_shape')
    return s


def _storage(x, storage_dtype):
    if storage_dtype is None or storage_dtype == x.dtype:
        return x
    return x.to(storage_dtype)


# ------------------------------------------------------------------ raymarch
LAYOUT_BRICK = 0x10  # GFT_LAYOUT_BRICK


def brick_cells(dhw):
    """Cells of one batch slice of a D x H x W grid in the raymarch's 2x2x2
    brick layout (GFT_LAYOUT_BRICK)."""
    D, H, W = (int(v) for v in dhw)
    return ((D + 1) // 2) * ((H + 1) // 2) * ((W + 1) // 2) * 8


def to_bricks(x):
    """[N, D, H, W, C] rows -> [N, brick_cells((D, H, W)), C] 2x2x2 bricks (the
    cells outside the grid are 0)."""
    N, D, H, W, C = x.shape
    xp = torch.nn.functional.pad(x, (0, 0, 0, W % 2, 0, H % 2, 0, D % 2))
    Dp, Hp, Wp = xp.shape[1:4]
    xb = xp.reshape(N, Dp // 2, 2, Hp // 2, 2, Wp // 2, 2, C).permute(0, 1, 3, 5, 2, 4, 6, 7)
    return xb.reshape(N, -1, C).contiguous()


def from_bricks(xb, grid_shape):
    """Inverse of to_bricks for a grid of shape (D, H, W)."""
    D, H, W = (int(v) for v in grid_shape)
    N, C = xb.shape[0], xb.shape[-1]
    Bz, By, Bx = (D + 1) // 2, (H + 1) // 2, (W + 1) // 2
    x = xb.reshape(N, Bz, By, Bx, 2, 2, 2, C).permute(0, 1, 4, 2, 5, 3, 6, 7).reshape(N, 2 * Bz, 2 * By, 2 * Bx, C)
    return x[:, :D, :H, :W].contiguous()


def _grid5(x, grid):
    """The logical [N, D, H, W, C] shape and the dtype code of a raymarch input:
    NDHWC rows (grid None) or bricks of a D x H x W grid ([N, cells, C])."""
    if grid is None:
        return tuple(x.shape), _dtype_code(x)
    return (x.shape[0],) + tuple(int(v) for v in grid) + (x.shape[-1],), _dtype_code(x) | LAYOUT_BRICK


def set_raymarch_sample_store(enabled, pool_fraction=None):
    """The differentiable raymarch stores the samples its forward blends and
    its backward reads them instead of re-sampling the grid (default on).  The
    store holds the samples that can be non-zero, in a pool sized at
    ``pool_fraction`` (default 0.25) of every sample the cameras could store;
    samples beyond it are re-sampled by the backward.  The store lives from
    the forward to the backward."""
    _state['sample_store'] = bool(enabled)
    if pool_fraction is not None:
        f = float(pool_fraction)
        if not 0.0 <= f <= 1.0:
            raise ValueError('pool_fraction must lie in [0, 1]')
        _state['sample_pool'] = f



def stored_sample_count(samples, shape5, nv, out_shape, separate=True):
    """Samples with a non-zero ballot bit in a store a forward filled (stored,
    or re-sampled by the backward where the pool was full)."""
    D, H, W = out_shape
    pairs = shape5[0] * (nv if separate else 1)
    cells = pairs * ((W + 7) // 8) * ((H + 15) // 16) * D * 128
    words = samples.view(torch.uint8)[256:256 + cells // 8].cpu().numpy()  # after the pool counter
    return int(np.unpackbits(words).sum())


def sample_pool_cells(samples):
    """Pool cells the forward's warps took (in chunks of 256; chunk requests
    past the pool's end included)."""
    return int(samples.view(torch.uint8)[:8].view(torch.int64).item())


def _samples_buffer(shape5, nv, out_shape, separate, device, pool_fraction=None):
    lib = _lib.load()
    args = (_lib.i64(shape5), nv, _lib.i32(out_shape), int(separate))
    full = lib.gft_raymarch_grid_transform_samples_size(*args)
    meta = lib.gft_raymarch_grid_transform_samples_min_size(*args)
    f = _state['sample_pool'] if pool_fraction is None else float(pool_fraction)
    return _workspace(meta + int((full - meta) * f) // 256 * 256, device)


def _raymarch_fwd(x, M, V, P, F, out_shape, interp, boundary, blend, separate, grid=None, samples=None):
    """samples: a sample store (_samples_buffer) the forward fills."""
    lib = _lib.load()
    D, H, W = out_shape
    Mh, nm = _mats(M)
    Vh, nv = _mats(V)
    Ph, npj = _mats(P)
    Fh, nf = _frustum(F)
    if not (nv == npj == nf):
        raise _lib.GftInvalidArgument('camera batch size mismatch')
    shape5, code = _grid5(x, grid)
    N, C = shape5[0], shape5[4]
    out = torch.empty((N, nv if separate else 1, H, W, C), dtype=torch.float32, device=x.device)
    with torch.cuda.device(x.device):
        if samples is None:
            st = lib.gft_raymarch_grid_transform(_p(x), code, _lib.i64(shape5), _p(Mh), nm, _p(Vh), _p(Ph),
                                                 _p(Fh), nv, _lib.i32(out_shape), interp, boundary, blend,
                                                 int(separate), _p(out), _stream(x.device))
        else:
            st = lib.gft_raymarch_grid_transform_store(_p(x), code, _lib.i64(shape5), _p(Mh), nm, _p(Vh), _p(Ph),
                                                       _p(Fh), nv, _lib.i32(out_shape), interp, boundary, blend,
                                                       int(separate), _p(out), _p(samples), samples.numel(),
                                                       _stream(x.device))
    _lib.check(st, 'RaymarchGridTransform')
    return out


WEIGHTS_READY = 0x100  # GFT_GRAD_WEIGHTS_READY


def _raymarch_weights(x_shape, device, M, V, P, F, out_shape, boundary, separate, det=False):
    """Pass 1 of the reference-normalised raymarch gradient (per-camera
    reciprocal weight sums; det: the deterministic adjoint's integer sums in
    its workspace layout) for an input of ``x_shape`` into a new workspace,
    on the current stream."""
    lib = _lib.load()
    Mh, nm = _mats(M)
    Vh, nv = _mats(V)
    Ph, _ = _mats(P)
    Fh, _ = _frustum(F)
    shape = _lib.i64(x_shape)
    gmode = GRAD['REFERENCE'] | (DETERMINISTIC if det else 0)
    ws = _workspace(lib.gft_raymarch_grid_transform_grad_workspace_size(shape, nv, int(separate), gmode), device)
    with torch.cuda.device(device):
        st = lib.gft_raymarch_grid_transform_grad_weights_mode(shape, _p(Mh), nm, _p(Vh), _p(Ph), _p(Fh), nv,
                                                               _lib.i32(out_shape), boundary, int(separate), gmode,
                                                               _p(ws), ws.numel(), _stream(device))
    _lib.check(st, 'RaymarchGridTransformGrad weights')
    return ws


_side_streams = {}


def _side_stream(dev):
    s = _side_streams.get(dev.index)
    if s is None:
        s = _side_streams[dev.index] = torch.cuda.Stream(dev)
    return s


def _raymarch_weights_async(x_shape, device, M, V, P, F, out_shape, boundary, separate, det=False):
    """Launches the geometry-only weight pass on a side stream forked from the
    current one, so that it overlaps the rest of the forward pass (the pass is
    bound by L2 reductions, the forward kernels by issue and L1); returns the
    workspace and the event the backward waits on.  Fork and join are stream
    waits, so a CUDA-graph capture records the two branches."""
    cur = torch.cuda.current_stream(device)
    side = _side_stream(device)
    side.wait_stream(cur)
    with torch.cuda.stream(side):
        ws = _raymarch_weights(x_shape, device, M, V, P, F, out_shape, boundary, separate, det)
        ev = torch.cuda.Event()
        ev.record(side)
    return ws, ev


_prefetched = {}
_weight_cache = {'enabled': False, 'max': 4, 'entries': {}}


def set_raymarch_weight_cache(enabled, max_entries=4):
    """Static camera rigs: keep the reference-normalised raymarch gradient's
    per-camera weight sums (a function of the cameras, the grid shape, the
    image size and the boundary mode only) across calls and reuse them when
    exactly the same geometry comes back, instead of recomputing them in every
    backward.  Off by default.  Entries are keyed by the matrix and frustum
    values, so changed cameras are recomputed; each entry holds one float per
    voxel and camera (75 MB at 128x227x128 and 5 views), at most
    ``max_entries`` are kept.  An entry is filled on the current stream outside
    CUDA-graph capture and the stream is synchronised once then."""
    _weight_cache['enabled'] = bool(enabled)
    _weight_cache['max'] = max(1, int(max_entries))
    if not enabled:
        _weight_cache['entries'].clear()


def _cached_weights(shape5, device, M, V, P, F, out_shape, boundary, separate):
    """The cached weight workspace for this geometry, filling it if allowed;
    None when the cache is off or a capture is running and the entry is new."""
    if not _weight_cache['enabled']:
        return None
    key = _weights_key(shape5, M, V, P, F, out_shape, boundary, separate, device)
    ent = _weight_cache['entries']
    if key in ent:
        return ent[key]
    if torch.cuda.is_current_stream_capturing():
        return None
    ws = _raymarch_weights(shape5, device, M, V, P, F, out_shape, boundary, separate)
    torch.cuda.current_stream(device).synchronize()
    if len(ent) >= _weight_cache['max']:
        ent.pop(next(iter(ent)))
    ent[key] = ws
    return ws


def _weights_key(x_shape, M, V, P, F, out_shape, boundary, separate, device, det=False):
    return (tuple(int(v) for v in x_shape), _mats(M)[0].tobytes(), _mats(V)[0].tobytes(), _mats(P)[0].tobytes(),
            _frustum(F)[0].tobytes(), tuple(int(v) for v in out_shape), int(boundary), bool(separate),
            _cuda_device(device).index, bool(det))


def _cuda_device(device):
    """torch.device with an explicit index (``'cuda'`` means the current device)."""
    dev = torch.device('cuda') if device is None else torch.device(device)
    return dev if dev.index is not None else torch.device('cuda', torch.cuda.current_device())


def prefetch_raymarch_weights(input_shape, matrix_m, matrix_v, matrix_p, frustum_params, output_shape,
                              boundary='BORDER', separate_camera_batch=True, device=None, for_camera_sums=False):
    """Starts the first, geometry-only pass of the reference-normalised
    raymarch gradient (the per-camera weight sums) on a side stream now, so
    that it overlaps whatever the caller runs before the raymarch.  The next
    differentiable raymarch_grid_transform with the same input shape, device
    and geometry takes it over; until then it holds one float per voxel and
    camera.  Under CUDA-graph capture that raymarch and its backward must be
    captured too (they join the side stream).  for_camera_sums: the raymarch
    is a fused render with a factored light, whose adjoint sums the weights
    itself while camera_sums_active(); nothing is started then."""
    det = _state['deterministic']  # (then the integer sums of the deterministic adjoint)
    if _lib.load().gft_get_knob(KNOB_WEIGHTS_PIPELINE) == 1 and not det:
        return  # the gradient call computes them, beside its scatter
    if for_camera_sums and camera_sums_active():
        return  # the fused render's adjoint sums the weights itself
    dev = _cuda_device(device)
    out_shape = _shape3(output_shape)
    b = _enum(BOUNDARY, boundary, 'boundary')
    key = _weights_key(input_shape, matrix_m, matrix_v, matrix_p, frustum_params, out_shape, b,
                       separate_camera_batch, dev, det)
    if not det and _weight_cache['enabled'] and key in _weight_cache['entries']:
        return
    _prefetched[key] = _raymarch_weights_async(tuple(input_shape), dev, matrix_m, matrix_v, matrix_p, frustum_params,
                                               out_shape, b, bool(separate_camera_batch), det)


def _raymarch_bwd(x, y, dy, M, V, P, F, out_shape, interp, boundary, blend, separate, gmode, weights=None,
                  grid=None, samples=None, projection=None, camera_sums=False):
    """projection (8 host floats, bricked 4-channel x): the gradient
    accumulated projected onto two channels, [N, cells, 2].  camera_sums
    (with projection, REFERENCE): per pair the unnormalised projected sums
    [pairs, cells, 2] and the workspace holding the pairs' weight sums, as
    (sums, workspace)."""
    lib = _lib.load()
    Mh, nm = _mats(M)
    Vh, nv = _mats(V)
    Ph, _ = _mats(P)
    Fh, _ = _frustum(F)
    shape5, code = _grid5(x, grid)
    shape = _lib.i64(shape5)
    gshape = x.shape if projection is None else tuple(x.shape[:-1]) + (2,)
    if camera_sums:
        gshape = (shape5[0] * (nv if separate else 1),) + tuple(x.shape[1:-1]) + (2,)
        weights = None
    grad = torch.empty(gshape, dtype=torch.float32, device=x.device)
    if weights is not None and (gmode & ~DETERMINISTIC) == GRAD['REFERENCE']:
        ws = weights
        gmode = gmode | WEIGHTS_READY
    else:
        ws = _workspace(lib.gft_raymarch_grid_transform_grad_workspace_size(shape, nv, int(separate), gmode),
                        x.device)
    with torch.cuda.device(x.device):
        if projection is not None:
            proj = np.ascontiguousarray(np.asarray(projection, dtype=np.float32).reshape(8))
            st = lib.gft_raymarch_grid_transform_grad_projected(
                _p(x), code, shape, _p(y), _p(dy), _p(Mh), nm, _p(Vh), _p(Ph), _p(Fh), nv, _lib.i32(out_shape),
                interp, boundary, blend, int(separate), gmode | (CAMERA_SUMS if camera_sums else 0),
                _p(samples) if samples is not None else None, samples.numel() if samples is not None else 0,
                _p(proj), _p(grad), _p(ws), ws.numel(), _stream(x.device))
        elif samples is None:
            st = lib.gft_raymarch_grid_transform_grad(_p(x), code, shape, _p(y), _p(dy), _p(Mh), nm, _p(Vh),
                                                      _p(Ph), _p(Fh), nv, _lib.i32(out_shape), interp, boundary,
                                                      blend, int(separate), gmode, _p(grad), _p(ws), ws.numel(),
                                                      _stream(x.device))
        else:
            st = lib.gft_raymarch_grid_transform_grad_stored(_p(x), code, shape, _p(y), _p(dy), _p(Mh), nm, _p(Vh),
                                                             _p(Ph), _p(Fh), nv, _lib.i32(out_shape), interp,
                                                             boundary, blend, int(separate), gmode, _p(samples),
                                                             samples.numel(), _p(grad), _p(ws), ws.numel(),
                                                             _stream(x.device))
    _lib.check(st, 'RaymarchGridTransformGrad')
    return (grad, ws) if camera_sums else grad


def _raymarch_forward_ctx(ctx, xs, need_grad, M, V, P, F, out_shape, interp, boundary, blend, separate, grid,
                          weights_pass=True):
    """Forward of a differentiable raymarch of the storage-typed input xs:
    starts the reference normalisation's weight pass (cached, prefetched or on
    a side stream; not with weights_pass False, for an adjoint that sums the
    weights itself) into ctx.weights and returns (output, sample store)."""
    shape5 = _grid5(xs, grid)[0]
    ctx.weights = None
    det = _state['deterministic']
    if need_grad and weights_pass and get_grad_mode() == 'REFERENCE' and interp == FILTER['LINEAR']:
        cached = None if det else _cached_weights(shape5, xs.device, M, V, P, F, out_shape, boundary, separate)
        if cached is not None:
            ctx.weights = (cached, None)
        elif _state['side_weights'] and (det or _lib.load().gft_get_knob(KNOB_WEIGHTS_PIPELINE) != 1):
            # (with the pipeline knob the float gradient call computes the
            # weight sums itself, beside its scatter; the deterministic
            # adjoint's integer sums also run ahead)
            key = _weights_key(shape5, M, V, P, F, out_shape, boundary, separate, xs.device, det)
            ctx.weights = _prefetched.pop(key, None) or _raymarch_weights_async(shape5, xs.device, M, V, P, F,
                                                                                out_shape, boundary, separate, det)
    ctx.weights_det = det
    samples = None
    if need_grad and interp == FILTER['LINEAR'] and _state['sample_store']:
        samples = _samples_buffer(shape5, _mats(V)[1], out_shape, separate, xs.device)
    y = _raymarch_fwd(xs, M, V, P, F, out_shape, interp, boundary, blend, separate, grid=grid, samples=samples)
    return y, samples


def _raymarch_backward_ctx(ctx, xs, y, samples, dy, M, V, P, F, out_shape, interp, boundary, blend, separate, grid,
                           projection=None, camera_sums=False):
    """The fp32 input gradient of a raymarch run by _raymarch_forward_ctx
    (projected onto two channels with ``projection``; per-camera sums and
    weight sums with ``camera_sums``)."""
    ws = None
    if ctx.weights is not None:
        ws, ev = ctx.weights
        if ev is not None:
            torch.cuda.current_stream(xs.device).wait_event(ev)
        if getattr(ctx, 'weights_det', False) != _state['deterministic']:
            ws = None  # summed for the other mode: the gradient call sums its own
    g = _raymarch_bwd(xs, y, _cuda(dy, 'output_grad'), M, V, P, F, out_shape, interp, boundary, blend, separate,
                      _scatter_gmode(), weights=ws, grid=grid, samples=samples, projection=projection,
                      camera_sums=camera_sums)
    ctx.weights = None
    return g


class _Raymarch(torch.autograd.Function):
    @staticmethod
    def forward(ctx, x, M, V, P, F, out_shape, interp, boundary, blend, separate, storage_dtype, grid=None):
        xs = _storage(x, storage_dtype)
        y, samples = _raymarch_forward_ctx(ctx, xs, ctx.needs_input_grad[0], M, V, P, F, out_shape, interp,
                                           boundary, blend, separate, grid)
        # a saved tensor, so that checkpointing drops and recomputes it
        ctx.save_for_backward(xs, y, samples)
        ctx.args = (M, V, P, F, out_shape, interp, boundary, blend, separate, grid)
        ctx.in_dtype = x.dtype
        return y

    @staticmethod
    def backward(ctx, dy):
        xs, y, samples = ctx.saved_tensors
        g = _raymarch_backward_ctx(ctx, xs, y, samples, dy, *ctx.args)
        return (g.to(ctx.in_dtype),) + (None,) * 11


def raymarch_grid_transform(input, matrix_m, matrix_v, matrix_p, frustum_params, output_shape,
                            interpolation='LINEAR', boundary='BORDER', blending_mode='BEER_LAMBERT',
                            keep_dims=False, separate_camera_batch=True, storage_dtype=None):
    """RaymarchGridTransform: [N,D,H,W,C] -> [N,V,H,W,C] ([N,V,1,H,W,C] with keep_dims).
    ``storage_dtype=torch.bfloat16`` stores the sampled grid in bf16 (fp32 math)."""
    x = _cuda(input, 'input', (torch.float32, torch.bfloat16))
    if x.dim() != 5 or x.shape[4] > 4:
        raise _lib.GftInvalidArgument('Invalid input shape (NDHWC): %s' % (tuple(x.shape),))
    out_shape = _shape3(output_shape)
    y = _Raymarch.apply(x, matrix_m, matrix_v, matrix_p, frustum_params, out_shape,
                        _enum(FILTER, interpolation, 'interpolation'), _enum(BOUNDARY, boundary, 'boundary'),
                        _enum(BLEND, blending_mode, 'blending_mode'), bool(separate_camera_batch), storage_dtype)
    return y.unsqueeze(2) if keep_dims else y


def raymarch_grid_transform_bricked(input, grid_shape, matrix_m, matrix_v, matrix_p, frustum_params, output_shape,
                                    boundary='BORDER', blending_mode='BEER_LAMBERT', keep_dims=False,
                                    separate_camera_batch=True, storage_dtype=None):
    """raymarch_grid_transform (LINEAR) of a grid of logical shape
    [N, *grid_shape, C] stored in the 2x2x2 brick layout, input
    [N, brick_cells(grid_shape), C] (e.g. gft.fused.light_compose(brick=True));
    its gradient comes back in the same layout.  The bricks put the corner
    gathers of a warp's neighbouring rays into fewer cache lines."""
    x = _cuda(input, 'input', (torch.float32, torch.bfloat16))
    grid = _shape3(grid_shape)
    if x.dim() != 3 or x.shape[1] != brick_cells(grid) or x.shape[2] > 4:
        raise _lib.GftInvalidArgument('bricked input must be [N, brick_cells(grid_shape), C], got %s'
                                      % (tuple(x.shape),))
    out_shape = _shape3(output_shape)
    y = _Raymarch.apply(x, matrix_m, matrix_v, matrix_p, frustum_params, out_shape, FILTER['LINEAR'],
                        _enum(BOUNDARY, boundary, 'boundary'), _enum(BLEND, blending_mode, 'blending_mode'),
                        bool(separate_camera_batch), storage_dtype, tuple(grid))
    return y.unsqueeze(2) if keep_dims else y


def raymarch_grid_transform_grad(input, output, output_grad, matrix_m, matrix_v, matrix_p, frustum_params,
                                 output_shape, interpolation='LINEAR', boundary='BORDER',
                                 blending_mode='BEER_LAMBERT', keep_dims=False, separate_camera_batch=True):
    """RaymarchGridTransformGrad (raymarch_grid.cc:56-76)."""
    x = _cuda(input, 'input', (torch.float32, torch.bfloat16))
    y = _cuda(output, 'output')
    dy = _cuda(output_grad, 'output_grad')
    if keep_dims:
        y, dy = y.squeeze(2), dy.squeeze(2)
    if tuple(y.shape) != tuple(dy.shape):
        raise _lib.GftInvalidArgument('Shapes of output grid and output gradients must match')
    return _raymarch_bwd(x, y.contiguous(), dy.contiguous(), matrix_m, matrix_v, matrix_p, frustum_params,
                         _shape3(output_shape), _enum(FILTER, interpolation, 'interpolation'),
                         _enum(BOUNDARY, boundary, 'boundary'), _enum(BLEND, blending_mode, 'blending_mode'),
                         bool(separate_camera_batch), _scatter_gmode())


# ------------------------------------------------------------------ raymarch, uneven camera batches
def _shapes3(shapes, nv):
    s = [[int(v) for v in (sh.tolist() if isinstance(sh, (np.ndarray, torch.Tensor)) else sh)] for sh in shapes]
    if len(s) != nv or any(len(v) != 3 or min(v) < 1 for v in s):
        raise _lib.GftInvalidArgument('output_shapes must hold one positive (depth, height, width) per camera')
    return s


def _raymarch_multi_weights(x_shape, device, M, V, P, F, shapes, boundary):
    lib = _lib.load()
    Mh, nm = _mats(M)
    Vh, nv = _mats(V)
    Ph, _ = _mats(P)
    Fh, _ = _frustum(F)
    shape = _lib.i64(x_shape)
    ws = _workspace(lib.gft_raymarch_grid_transform_multi_grad_workspace_size(shape, nv, GRAD['REFERENCE']), device)
    with torch.cuda.device(device):
        st = lib.gft_raymarch_grid_transform_multi_grad_weights(shape, _p(Mh), nm, _p(Vh), _p(Ph), _p(Fh), nv,
                                                                _lib.i32(sum(shapes, [])), boundary, _p(ws),
                                                                ws.numel(), _stream(device))
    _lib.check(st, 'RaymarchGridTransformMulti weights')
    return ws


def _raymarch_multi_fwd(x, M, V, P, F, shapes, interp, boundary, blend):
    lib = _lib.load()
    Mh, nm = _mats(M)
    Vh, nv = _mats(V)
    Ph, npj = _mats(P)
    Fh, nf = _frustum(F)
    if not (nv == npj == nf):
        raise _lib.GftInvalidArgument('camera batch size mismatch')
    N, C = x.shape[0], x.shape[4]
    npix = sum(h * w for _, h, w in shapes)
    out = torch.empty((N, npix, C), dtype=torch.float32, device=x.device)
    with torch.cuda.device(x.device):
        st = lib.gft_raymarch_grid_transform_multi(_p(x), _dtype_code(x), _lib.i64(x.shape), _p(Mh), nm, _p(Vh),
                                                   _p(Ph), _p(Fh), nv, _lib.i32(sum(shapes, [])), interp, boundary,
                                                   blend, _p(out), _stream(x.device))
    _lib.check(st, 'RaymarchGridTransformMulti')
    return out


def _raymarch_multi_bwd(x, y, dy, M, V, P, F, shapes, interp, boundary, blend, gmode, weights=None):
    lib = _lib.load()
    Mh, nm = _mats(M)
    Vh, nv = _mats(V)
    Ph, _ = _mats(P)
    Fh, _ = _frustum(F)
    shape = _lib.i64(x.shape)
    grad = torch.empty(x.shape, dtype=torch.float32, device=x.device)
    if weights is not None and gmode == GRAD['REFERENCE']:
        ws = weights
        gmode = gmode | WEIGHTS_READY
    else:
        ws = _workspace(lib.gft_raymarch_grid_transform_multi_grad_workspace_size(shape, nv, gmode), x.device)
    with torch.cuda.device(x.device):
        st = lib.gft_raymarch_grid_transform_multi_grad(_p(x), _dtype_code(x), shape, _p(y), _p(dy), _p(Mh), nm,
                                                        _p(Vh), _p(Ph), _p(Fh), nv, _lib.i32(sum(shapes, [])),
                                                        interp, boundary, blend, gmode, _p(grad), _p(ws),
                                                        ws.numel(), _stream(x.device))
    _lib.check(st, 'RaymarchGridTransformMultiGrad')
    return grad


class _RaymarchMulti(torch.autograd.Function):
    @staticmethod
    def forward(ctx, x, M, V, P, F, shapes, interp, boundary, blend, storage_dtype):
        xs = _storage(x, storage_dtype)
        ctx.weights = None
        if (ctx.needs_input_grad[0] and _state['side_weights'] and get_grad_mode() == 'REFERENCE'
                and interp == FILTER['LINEAR'] and not _state['deterministic']):
            cur = torch.cuda.current_stream(xs.device)
            side = _side_stream(xs.device)
            side.wait_stream(cur)
            with torch.cuda.stream(side):
                ws = _raymarch_multi_weights(tuple(xs.shape), xs.device, M, V, P, F, shapes, boundary)
                ev = torch.cuda.Event()
                ev.record(side)
            ctx.weights = (ws, ev)
        y = _raymarch_multi_fwd(xs, M, V, P, F, shapes, interp, boundary, blend)
        ctx.save_for_backward(xs, y)
        ctx.args = (M, V, P, F, shapes, interp, boundary, blend)
        ctx.in_dtype = x.dtype
        return y

    @staticmethod
    def backward(ctx, dy):
        xs, y = ctx.saved_tensors
        M, V, P, F, shapes, interp, boundary, blend = ctx.args
        ws = None
        if ctx.weights is not None:
            ws, ev = ctx.weights
            torch.cuda.current_stream(xs.device).wait_event(ev)
        g = _raymarch_multi_bwd(xs, y, _cuda(dy, 'output_grad'), M, V, P, F, shapes, interp, boundary, blend,
                                _scatter_gmode(), weights=ws)
        ctx.weights = None
        return (g.to(ctx.in_dtype),) + (None,) * 9


def raymarch_grid_transform_multi(input, matrix_m, matrix_v, matrix_p, frustum_params, output_shapes,
                                  interpolation='LINEAR', boundary='BORDER', blending_mode='BEER_LAMBERT',
                                  storage_dtype=None):
    """RaymarchGridTransform for cameras of different image sizes in one launch
    (global sampling): camera c renders output_shapes[c] = (depth samples,
    height, width).  Returns one [N, H_c, W_c, C] image per camera, views of one
    [N, sum_c H_c W_c, C] buffer; each equals
    raymarch_grid_transform(input, ..., camera c alone, output_shapes[c])[:, 0]."""
    x = _cuda(input, 'input', (torch.float32, torch.bfloat16))
    if x.dim() != 5 or x.shape[4] > 4:
        raise _lib.GftInvalidArgument('Invalid input shape (NDHWC): %s' % (tuple(x.shape),))
    nv = _mats(matrix_v)[1]
    shapes = _shapes3(output_shapes, nv)
    y = _RaymarchMulti.apply(x, matrix_m, matrix_v, matrix_p, frustum_params, shapes,
                             _enum(FILTER, interpolation, 'interpolation'), _enum(BOUNDARY, boundary, 'boundary'),
                             _enum(BLEND, blending_mode, 'blending_mode'), storage_dtype)
    sizes = [h * w for _, h, w in shapes]
    return [part.view(x.shape[0], h, w, x.shape[4]) for part, (_, h, w) in zip(torch.split(y, sizes, dim=1), shapes)]


# ------------------------------------------------------------------ views bound to batch slices
def _views_args(M, V, P, F, camera_batch, shapes):
    Mh, nm = _mats(M)
    Vh, nv = _mats(V)
    Ph, npj = _mats(P)
    Fh, nf = _frustum(F)
    if not (nv == npj == nf == len(camera_batch) == len(shapes)):
        raise _lib.GftInvalidArgument('camera batch size mismatch')
    return Mh, nm, Vh, Ph, Fh, nv, _lib.i32(camera_batch), _lib.i32(sum(shapes, []))


def _raymarch_views_weights(x_shape, device, M, V, P, F, camera_batch, shapes, boundary):
    lib = _lib.load()
    Mh, nm, Vh, Ph, Fh, nv, cb, sh = _views_args(M, V, P, F, camera_batch, shapes)
    shape = _lib.i64(x_shape)
    ws = _workspace(lib.gft_raymarch_grid_transform_views_grad_workspace_size(shape, nv, GRAD['REFERENCE']), device)
    with torch.cuda.device(device):
        st = lib.gft_raymarch_grid_transform_views_grad_weights(shape, _p(Mh), nm, _p(Vh), _p(Ph), _p(Fh), nv, cb, sh,
                                                                boundary, _p(ws), ws.numel(), _stream(device))
    _lib.check(st, 'RaymarchGridTransformViews weights')
    return ws


def _raymarch_views_fwd(x, M, V, P, F, camera_batch, shapes, interp, boundary, blend):
    lib = _lib.load()
    Mh, nm, Vh, Ph, Fh, nv, cb, sh = _views_args(M, V, P, F, camera_batch, shapes)
    npix = sum(h * w for _, h, w in shapes)
    out = torch.empty((npix, x.shape[4]), dtype=torch.float32, device=x.device)
    with torch.cuda.device(x.device):
        st = lib.gft_raymarch_grid_transform_views(_p(x), _dtype_code(x), _lib.i64(x.shape), _p(Mh), nm, _p(Vh),
                                                   _p(Ph), _p(Fh), nv, cb, sh, interp, boundary, blend, _p(out),
                                                   _stream(x.device))
    _lib.check(st, 'RaymarchGridTransformViews')
    return out


def _raymarch_views_bwd(x, y, dy, M, V, P, F, camera_batch, shapes, interp, boundary, blend, gmode, weights=None):
    lib = _lib.load()
    Mh, nm, Vh, Ph, Fh, nv, cb, sh = _views_args(M, V, P, F, camera_batch, shapes)
    shape = _lib.i64(x.shape)
    grad = torch.empty(x.shape, dtype=torch.float32, device=x.device)
    if weights is not None and gmode == GRAD['REFERENCE']:
        ws = weights
        gmode = gmode | WEIGHTS_READY
    else:
        ws = _workspace(lib.gft_raymarch_grid_transform_views_grad_workspace_size(shape, nv, gmode), x.device)
    with torch.cuda.device(x.device):
        st = lib.gft_raymarch_grid_transform_views_grad(_p(x), _dtype_code(x), shape, _p(y), _p(dy), _p(Mh), nm,
                                                        _p(Vh), _p(Ph), _p(Fh), nv, cb, sh, interp, boundary, blend,
                                                        gmode, _p(grad), _p(ws), ws.numel(), _stream(x.device))
    _lib.check(st, 'RaymarchGridTransformViewsGrad')
    return grad


class _RaymarchViews(torch.autograd.Function):
    @staticmethod
    def forward(ctx, x, M, V, P, F, camera_batch, shapes, interp, boundary, blend, storage_dtype):
        xs = _storage(x, storage_dtype)
        ctx.weights = None
        if (ctx.needs_input_grad[0] and _state['side_weights'] and get_grad_mode() == 'REFERENCE'
                and interp == FILTER['LINEAR'] and not _state['deterministic']):
            cur = torch.cuda.current_stream(xs.device)
            side = _side_stream(xs.device)
            side.wait_stream(cur)
            with torch.cuda.stream(side):
                ws = _raymarch_views_weights(tuple(xs.shape), xs.device, M, V, P, F, camera_batch, shapes, boundary)
                ev = torch.cuda.Event()
                ev.record(side)
            ctx.weights = (ws, ev)
        y = _raymarch_views_fwd(xs, M, V, P, F, camera_batch, shapes, interp, boundary, blend)
        ctx.save_for_backward(xs, y)
        ctx.args = (M, V, P, F, camera_batch, shapes, interp, boundary, blend)
        ctx.in_dtype = x.dtype
        return y

    @staticmethod
    def backward(ctx, dy):
        xs, y = ctx.saved_tensors
        M, V, P, F, camera_batch, shapes, interp, boundary, blend = ctx.args
        ws = None
        if ctx.weights is not None:
            ws, ev = ctx.weights
            torch.cuda.current_stream(xs.device).wait_event(ev)
        g = _raymarch_views_bwd(xs, y, _cuda(dy, 'output_grad'), M, V, P, F, camera_batch, shapes, interp, boundary,
                                blend, _scatter_gmode(), weights=ws)
        ctx.weights = None
        return (g.to(ctx.in_dtype),) + (None,) * 10


def raymarch_grid_transform_views(input, camera_batch, matrix_m, matrix_v, matrix_p, frustum_params, output_shapes,
                                  interpolation='LINEAR', boundary='BORDER', blending_mode='BEER_LAMBERT',
                                  storage_dtype=None):
    """RaymarchGridTransform of views bound to batch slices, in one launch per
    16 views: camera c renders only batch slice camera_batch[c] into an image of
    output_shapes[c] = (depth samples, height, width).  Returns the images as
    one [sum_c H_c W_c, C] buffer, the cameras one after another (split it with
    views_split); camera c's image equals
    raymarch_grid_transform(input[b:b+1], M[b], camera c alone, output_shapes[c])
    with b = camera_batch[c]."""
    x = _cuda(input, 'input', (torch.float32, torch.bfloat16))
    if x.dim() != 5 or x.shape[4] > 4:
        raise _lib.GftInvalidArgument('Invalid input shape (NDHWC): %s' % (tuple(x.shape),))
    nv = _mats(matrix_v)[1]
    shapes = _shapes3(output_shapes, nv)
    cb = [int(b) for b in camera_batch]
    return _RaymarchViews.apply(x, matrix_m, matrix_v, matrix_p, frustum_params, cb, shapes,
                                _enum(FILTER, interpolation, 'interpolation'), _enum(BOUNDARY, boundary, 'boundary'),
                                _enum(BLEND, blending_mode, 'blending_mode'), storage_dtype)


def views_split(y, output_shapes):
    """The per-camera [H_c, W_c, C] images of a raymarch_grid_transform_views output."""
    sizes = [int(h) * int(w) for _, h, w in output_shapes]
    return [part.view(int(h), int(w), y.shape[-1]) for part, (_, h, w) in zip(torch.split(y, sizes, dim=0),
                                                                             output_shapes)]


# ------------------------------------------------------------------ SampleGridTransform
def _sample_transform_fwd(x, M, V, P, F, out_shape, interp, boundary, mip, num_mips, bias, coord, cco, separate):
    lib = _lib.load()
    Do, Ho, Wo = out_shape
    Mh, nm = _mats(M)
    Vh, nv = _mats(V)
    Ph, npj = _mats(P)
    Fh, nf = _frustum(F)
    if not (nv == npj == nf):
        raise _lib.GftInvalidArgument('camera batch size mismatch')
    N, C = x.shape[0], x.shape[4]
    shape = _lib.i64(x.shape)
    out = torch.empty((N, nv if separate else 1, Do, Ho, Wo, C), dtype=torch.float32, device=x.device)
    ws = _workspace(lib.gft_sample_grid_transform_workspace_size(shape, mip, num_mips), x.device)
    with torch.cuda.device(x.device):
        st = lib.gft_sample_grid_transform(_p(x), _dtype_code(x), shape, _p(Mh), nm, _p(Vh), _p(Ph), _p(Fh), nv,
                                           _lib.i32(out_shape), interp, boundary, mip, int(num_mips), float(bias),
                                           coord, float(cco), int(separate), _p(out), _p(ws), ws.numel(),
                                           _stream(x.device))
    _lib.check(st, 'SampleGridTransform')
    return out


def _sample_transform_bwd(in_shape, dy, M, V, P, F, interp, boundary, coord, cco, separate, gmode, device):
    lib = _lib.load()
    Mh, nm = _mats(M)
    Vh, nv = _mats(V)
    Ph, _ = _mats(P)
    Fh, _ = _frustum(F)
    shape = _lib.i64(in_shape)
    grad = torch.empty(tuple(in_shape), dtype=torch.float32, device=device)
    ws = _workspace(lib.gft_sample_grid_transform_grad_workspace_size(shape), device)
    with torch.cuda.device(device):
        st = lib.gft_sample_grid_transform_grad(shape, _p(dy), _lib.i64(dy.shape), _p(Mh), nm, _p(Vh), _p(Ph),
                                                _p(Fh), nv, interp, boundary, coord, float(cco), int(separate),
                                                gmode, _p(grad), _p(ws), ws.numel(), _stream(device))
    _lib.check(st, 'SampleGridTransformGrad')
    return grad


SAMPLE_DENSE = 0x100  # GFT_SAMPLE_DENSE


class _SampleTransform(torch.autograd.Function):
    @staticmethod
    def forward(ctx, x, M, V, P, F, out_shape, interp, boundary, mip, num_mips, bias, coord, cco, separate,
                storage_dtype, dense):
        xs = _storage(x, storage_dtype)
        y = _sample_transform_fwd(xs, M, V, P, F, out_shape, interp | (SAMPLE_DENSE if dense else 0), boundary, mip,
                                  num_mips, bias, coord, cco, separate)
        ctx.args = (tuple(x.shape), M, V, P, F, interp, boundary, mip, coord, cco, separate)
        ctx.in_dtype = x.dtype
        return y

    @staticmethod
    def backward(ctx, dy):
        in_shape, M, V, P, F, interp, boundary, mip, coord, cco, separate = ctx.args
        if mip != MIP['NONE']:
            # the registered gradient op only accepts mipmapping NONE (resample_grid.cc:73)
            raise _lib.GftInvalidArgument('SampleGridTransformGrad: mipmapping must be NONE')
        g = _sample_transform_bwd(in_shape, _cuda(dy, 'output_grad'), M, V, P, F, interp, boundary, coord, cco,
                                  separate, GRAD[get_grad_mode()], dy.device)
        return (g.to(ctx.in_dtype),) + (None,) * 15


def sample_grid_transform(input, matrix_m, matrix_v, matrix_p, frustum_params, output_shape,
                          interpolation='LINEAR', boundary='BORDER', mipmapping='NONE', num_mipmaps=0, mip_bias=0.0,
                          coordinate_mode='TRANSFORM_LINDEPTH', cell_center_offset=0.5, separate_camera_batch=True,
                          storage_dtype=None, dense_input=False):
    """SampleGridTransform: [N,D,H,W,C] -> [N, V (or 1), Do, Ho, Wo, C].
    dense_input: the input is known to be dense (e.g. a gradient), so no
    occupancy map is built for it (gft.h GFT_SAMPLE_DENSE); same result."""
    x = _cuda(input, 'input', (torch.float32, torch.bfloat16))
    if x.dim() != 5 or x.shape[4] > 4:
        raise _lib.GftInvalidArgument('Invalid input shape (NDHWC): %s' % (tuple(x.shape),))
    return _SampleTransform.apply(x, matrix_m, matrix_v, matrix_p, frustum_params, _shape3(output_shape),
                                  _enum(FILTER, interpolation, 'interpolation'), _enum(BOUNDARY, boundary, 'boundary'),
                                  _enum(MIP, mipmapping, 'mipmapping'), int(num_mipmaps), float(mip_bias),
                                  _enum(COORD, coordinate_mode, 'coordinate_mode'), float(cell_center_offset),
                                  bool(separate_camera_batch), storage_dtype, bool(dense_input))


def sample_grid_transform_grad(input, output_grad, matrix_m, matrix_v, matrix_p, frustum_params,
                               interpolation='LINEAR', boundary='BORDER', mipmapping='NONE', num_mipmaps=0,
                               mip_bias=0.0, coordinate_mode='TRANSFORM_LINDEPTH', cell_center_offset=0.5,
                               separate_camera_batch=True):
    """SampleGridTransformGrad (resample_grid.cc:64-84): trilinear scatter adjoint."""
    if _enum(MIP, mipmapping, 'mipmapping') != MIP['NONE']:
        raise _lib.GftInvalidArgument('SampleGridTransformGrad: mipmapping must be NONE')
    dy = _cuda(output_grad, 'output_grad')
    if dy.dim() != 6:
        raise _lib.GftInvalidArgument('Invalid output_grads shape (NVDHWC)')
    return _sample_transform_bwd(tuple(input.shape), dy, matrix_m, matrix_v, matrix_p, frustum_params,
                                 _enum(FILTER, interpolation, 'interpolation'), _enum(BOUNDARY, boundary, 'boundary'),
                                 _enum(COORD, coordinate_mode, 'coordinate_mode'), float(cell_center_offset),
                                 bool(separate_camera_batch), GRAD[get_grad_mode()], dy.device)


# ------------------------------------------------------------------ SampleGridLut
def _lut_fwd(x, lut, interp, boundary, mip, num_mips, bias, cco, separate, relative, normalized):
    lib = _lib.load()
    N, C = x.shape[0], x.shape[4]
    V = lut.shape[0]
    shape = _lib.i64(x.shape)
    out = torch.empty((N, V if separate else 1) + tuple(lut.shape[1:4]) + (C,), dtype=torch.float32,
                      device=x.device)
    ws = _workspace(lib.gft_sample_grid_lut_workspace_size(shape, mip, num_mips), x.device)
    with torch.cuda.device(x.device):
        st = lib.gft_sample_grid_lut(_p(x), _dtype_code(x), shape, _p(lut), _lib.i64(lut.shape), interp, boundary,
                                     mip, int(num_mips), float(bias), float(cco), int(separate), int(relative),
                                     int(normalized), _p(out), _p(ws), ws.numel(), _stream(x.device))
    _lib.check(st, 'SampleGridLut')
    return out


def _lut_bwd(x, lut, dy, interp, boundary, cco, separate, relative, normalized, gmode):
    lib = _lib.load()
    shape = _lib.i64(x.shape)
    gx = torch.empty(x.shape, dtype=torch.float32, device=x.device)
    glut = torch.empty(lut.shape, dtype=torch.float32, device=x.device)
    ws = _workspace(lib.gft_sample_grid_lut_grad_workspace_size(shape), x.device)
    with torch.cuda.device(x.device):
        st = lib.gft_sample_grid_lut_grad(_p(x), shape, _p(dy), _p(lut), _lib.i64(lut.shape), interp, boundary,
                                          float(cco), int(separate), int(relative), int(normalized), gmode, _p(gx),
                                          _p(glut), _p(ws), ws.numel(), _stream(x.device))
    _lib.check(st, 'SampleGridLutGrad')
    return gx, glut


class _SampleLut(torch.autograd.Function):
    @staticmethod
    def forward(ctx, x, lut, interp, boundary, mip, num_mips, bias, cco, separate, relative, normalized,
                storage_dtype):
        xs = _storage(x, storage_dtype)
        y = _lut_fwd(xs, lut, interp, boundary, mip, num_mips, bias, cco, separate, relative, normalized)
        ctx.save_for_backward(x, lut)
        ctx.args = (interp, boundary, mip, cco, separate, relative, normalized)
        return y

    @staticmethod
    def backward(ctx, dy):
        x, lut = ctx.saved_tensors
        interp, boundary, mip, cco, separate, relative, normalized = ctx.args
        if mip != MIP['NONE']:
            raise _lib.GftInvalidArgument('SampleGridLutGrad: mipmapping must be NONE')
        gx, glut = _lut_bwd(x.float(), lut, _cuda(dy, 'output_grad'), interp, boundary, cco, separate, relative,
                            normalized, GRAD[get_grad_mode()])
        return (gx.to(x.dtype), glut) + (None,) * 10


def sample_grid_lut(input, lookup, interpolation='LINEAR', boundary='BORDER', mipmapping='NONE', num_mipmaps=0,
                    mip_bias=0.0, coordinate_mode='LOOKUP', cell_center_offset=0.0, separate_camera_batch=True,
                    relative_coords=True, normalized_coords=False, storage_dtype=None):
    """SampleGridLut: input [N,D,H,W,C], lookup [V,Do,Ho,Wo,4] -> [N, V (or 1), Do, Ho, Wo, C]."""
    if str(coordinate_mode).upper() != 'LOOKUP':
        raise _lib.GftInvalidArgument('Invalid coorindate_mode')
    x = _cuda(input, 'input', (torch.float32, torch.bfloat16))
    lut = _cuda(lookup, 'lookup')
    if x.dim() != 5 or lut.dim() != 5 or lut.shape[4] != 4:
        raise _lib.GftInvalidArgument('Invalid lut shape (NDHWC) with C=4')
    return _SampleLut.apply(x, lut, _enum(FILTER, interpolation, 'interpolation'),
                            _enum(BOUNDARY, boundary, 'boundary'), _enum(MIP, mipmapping, 'mipmapping'),
                            int(num_mipmaps), float(mip_bias), float(cell_center_offset),
                            bool(separate_camera_batch), bool(relative_coords), bool(normalized_coords), storage_dtype)


def sample_grid_lut_grad(input, output_grad, lookup, interpolation='LINEAR', boundary='BORDER', mipmapping='NONE',
                         num_mipmaps=0, mip_bias=0.0, coordinate_mode='LOOKUP', cell_center_offset=0.0,
                         separate_camera_batch=True, relative_coords=True, normalized_coords=False):
    """SampleGridLutGrad: returns (input_grad, lookup_grad)."""
    if _enum(MIP, mipmapping, 'mipmapping') != MIP['NONE']:
        raise _lib.GftInvalidArgument('SampleGridLutGrad: mipmapping must be NONE')
    x = _cuda(input, 'input')
    return _lut_bwd(x, _cuda(lookup, 'lookup'), _cuda(output_grad, 'output_grad'),
                    _enum(FILTER, interpolation, 'interpolation'), _enum(BOUNDARY, boundary, 'boundary'),
                    float(cell_center_offset), bool(separate_camera_batch), bool(relative_coords),
                    bool(normalized_coords), GRAD[get_grad_mode()])


def lod_transform(input_shape, matrix_mv, matrix_p, frustum_params, output_shape, inverse_transform=False,
                  device=None):
    """LodTransform: [V, Do, Ho, Wo, 4] of sampling positions and LOD."""
    lib = _lib.load()
    dev = torch.device(device) if device is not None else torch.device('cuda', torch.cuda.current_device())
    MVh, n = _mats(matrix_mv)
    Ph, npj = _mats(matrix_p)
    Fh, nf = _frustum(frustum_params)
    if not (n == npj == nf):
        raise _lib.GftInvalidArgument('camera batch size mismatch')
    ins, outs = _shape3(input_shape), _shape3(output_shape)
    out = torch.empty((n,) + tuple(outs) + (4,), dtype=torch.float32, device=dev)
    with torch.cuda.device(dev):
        st = lib.gft_lod_transform(_lib.i32(ins), _p(MVh), _p(Ph), _p(Fh), n, _lib.i32(outs), int(inverse_transform),
                                   _p(out), _stream(dev))
    _lib.check(st, 'LodTransform')
    return out


# ------------------------------------------------------------------ ReduceGridBlend
def _blend_fwd(x, mode, keep):
    lib = _lib.load()
    N, D, H, W, C = x.shape
    out = torch.empty((N, D, H, W, C) if keep else (N, H, W, C), dtype=torch.float32, device=x.device)
    with torch.cuda.device(x.device):
        st = lib.gft_reduce_grid_blend(_p(x), _lib.i64(x.shape), mode, int(keep), _p(out), _stream(x.device))
    _lib.check(st, 'ReduceGridBlend')
    return out


def _blend_bwd(dy, y, x, mode, keep, gmode):
    lib = _lib.load()
    gx = torch.empty(x.shape, dtype=torch.float32, device=x.device)
    with torch.cuda.device(x.device):
        st = lib.gft_reduce_grid_blend_grad(_p(dy), _p(y), _p(x), _lib.i64(x.shape), mode, int(keep), gmode, _p(gx),
                                            _stream(x.device))
    _lib.check(st, 'ReduceGridBlendGrad')
    return gx


class _Blend(torch.autograd.Function):
    @staticmethod
    def forward(ctx, x, mode, keep):
        y = _blend_fwd(x, mode, keep)
        ctx.save_for_backward(x, y)
        ctx.args = (mode, keep)
        return y

    @staticmethod
    def backward(ctx, dy):
        x, y = ctx.saved_tensors
        mode, keep = ctx.args
        return _blend_bwd(_cuda(dy, 'output_grad'), y, x, mode, keep, GRAD[get_grad_mode()]), None, None


def reduce_grid_blend(input, blending_mode='BEER_LAMBERT', keep_dims=False):
    """ReduceGridBlend: [N,D,H,W,C] -> [N,H,W,C] or [N,D,H,W,C] (keep_dims)."""
    x = _cuda(input, 'input')
    if x.dim() != 5 or x.shape[4] > 4:
        raise _lib.GftInvalidArgument('Invalid input shape')
    return _Blend.apply(x, _enum(BLEND, blending_mode, 'blending_mode'), bool(keep_dims))


def reduce_grid_blend_grad(output_grad, output, input, blending_mode='BEER_LAMBERT', keep_dims=False):
    """ReduceGridBlendGrad (reduce_blend.cc:37-48)."""
    dy = _cuda(output_grad, 'output_grad')
    y = _cuda(output, 'output')
    if tuple(dy.shape) != tuple(y.shape):
        raise _lib.GftInvalidArgument('Mismatch between output gradients and output shape')
    return _blend_bwd(dy, y, _cuda(input, 'input'), _enum(BLEND, blending_mode, 'blending_mode'), bool(keep_dims),
                      GRAD[get_grad_mode()])


# ------------------------------------------------------------------ advection
FORWARD_READY = 0x200  # GFT_GRAD_FORWARD_READY


def _advect_fwd(d, vx, vy, vz, dt, order, clamp, boundary, ws=None):
    lib = _lib.load()
    shape = _lib.i64(d.shape)
    out = torch.empty(d.shape, dtype=torch.float32, device=d.device)
    if ws is None:
        ws = _workspace(lib.gft_advect_workspace_size(shape, order), d.device)
    with torch.cuda.device(d.device):
        st = lib.gft_advect(_p(d), _dtype_code(d), shape, _p(vx), _p(vy), _p(vz), float(dt), order, clamp, boundary,
                            _p(out), _p(ws), ws.numel(), _stream(d.device))
    _lib.check(st, 'advect')
    return out


def _advect_grad_bytes(shape, order, gmode):
    return int(_lib.load().gft_advect_grad_workspace_size_mode(_lib.i64(shape), order, gmode))


def _advect_grad_workspace(shape, order, device, gmode=0):
    return _workspace(_advect_grad_bytes(shape, order, gmode), device)


def _advect_bwd(d, vx, vy, vz, dy, dt, order, clamp, boundary, gmode, ws=None):
    """ws: the workspace the forward ran in (gmode then carries FORWARD_READY),
    else a new one."""
    lib = _lib.load()
    shape = _lib.i64(d.shape)
    gd = torch.empty(d.shape, dtype=torch.float32, device=d.device)
    gvx, gvy, gvz = (torch.empty(v.shape, dtype=torch.float32, device=d.device) for v in (vx, vy, vz))
    if ws is None:
        ws = _advect_grad_workspace(d.shape, order, d.device, gmode)
    with torch.cuda.device(d.device):
        st = lib.gft_advect_grad(_p(d), shape, _p(vx), _p(vy), _p(vz), float(dt), order, clamp, boundary, gmode,
                                 _p(dy), _p(gd), _p(gvx), _p(gvy), _p(gvz), _p(ws), ws.numel(), _stream(d.device))
    _lib.check(st, 'advect gradient')
    return gd, gvx, gvy, gvz


def _vel_component(v, name, expect):
    v = _cuda(v, name)
    if v.numel() != int(np.prod(expect)):
        raise _lib.GftInvalidArgument('Invalid shape of velocity %s component: %s, expected %s'
                                      % (name, tuple(v.shape), expect))
    return v


class _Advect(torch.autograd.Function):
    @staticmethod
    def forward(ctx, d, vx, vy, vz, dt, order, clamp, boundary, storage_dtype):
        ds = _storage(d, storage_dtype)
        # MacCormack on one fp32 slice: run the forward in the gradient's
        # workspace and keep it, so that the backward reads the intermediate
        # semi-Lagrangian grid instead of recomputing it
        ws = None
        if any(ctx.needs_input_grad[:4]) and order == 2 and ds.shape[0] == 1 and ds is d and d.dtype == torch.float32:
            ws = _advect_grad_workspace(d.shape, order, d.device, _scatter_gmode())
        y = _advect_fwd(ds, vx, vy, vz, dt, order, clamp, boundary, ws=ws)
        # the workspace is a saved tensor, so that checkpointing drops and recomputes it
        ctx.save_for_backward(d, vx, vy, vz, ws)
        ctx.args = (dt, order, clamp, boundary)
        return y

    @staticmethod
    def backward(ctx, dy):
        d, vx, vy, vz, ws = ctx.saved_tensors
        dt, order, clamp, boundary = ctx.args
        gmode = _scatter_gmode()
        if ws is not None and ws.numel() < _advect_grad_bytes(d.shape, order, gmode):
            ws = None  # the deterministic mode was switched on after the forward: recompute the intermediate
        gd, gvx, gvy, gvz = _advect_bwd(d.float().contiguous(), vx, vy, vz, _cuda(dy, 'output_grad'), dt, order,
                                        clamp, boundary, gmode | (FORWARD_READY if ws is not None else 0), ws=ws)
        return gd.to(d.dtype), gvx.view_as(vx), gvy.view_as(vy), gvz.view_as(vz), None, None, None, None, None


def advect(density, vel_x, vel_y, vel_z, dt=1.0, order=1, clamp='NONE', boundary='CLAMP', storage_dtype=None):
    """VelocityGrid.warp fused: density [N,D,H,W,C] advected by the staggered
    velocity x [..,D,H,W+1,1], y [..,D,H+1,W,1], z [..,D+1,H,W,1] (leading batch
    dims of the components must be 1).  order 1 semi-Lagrangian, 2 MacCormack;
    clamp NONE / MC_SMOOTH / NEGATIVE."""
    d = _cuda(density, 'density', (torch.float32, torch.bfloat16))
    if d.dim() != 5:
        raise _lib.GftInvalidArgument('density must be 5D (NDHWC)')
    _, D, H, W, _ = d.shape
    vx = _vel_component(vel_x, 'x', (D, H, W + 1))
    vy = _vel_component(vel_y, 'y', (D, H + 1, W))
    vz = _vel_component(vel_z, 'z', (D + 1, H, W))
    c = str(clamp).upper()
    if c == 'MC':
        raise NotImplementedError('MIM and MAX warp sampling have wrong gradients.')
    return _Advect.apply(d, vx, vy, vz, float(dt), int(order), _enum(CLAMP, c, 'clamp'),
                         _enum(BOUNDARY, boundary, 'boundary'), storage_dtype)


def raymarch_check(input, matrix_m, matrix_v, matrix_p, frustum_params, output_shape, output, ray_stride=1,
                   grid_shape=None, out=None):
    """FP64 recomputation of the density (last) channel of a BEER_LAMBERT /
    LINEAR / BORDER raymarch_grid_transform (separate camera batches) for
    every ray_stride-th pixel: a device float64 tensor [max |fp32 - fp64|,
    max |fp64|] of ``output`` [N, V, H, W, C] (written into ``out`` when
    given; the ratio is the max-norm relative error).  ``grid_shape``: the input is in the brick layout
    (raymarch_grid_transform_bricked)."""
    x = _cuda(input, 'input', (torch.float32, torch.bfloat16))
    y = _cuda(output, 'output')
    lib = _lib.load()
    Mh, nm = _mats(matrix_m)
    Vh, nv = _mats(matrix_v)
    Ph, _ = _mats(matrix_p)
    Fh, _ = _frustum(frustum_params)
    shape5, code = _grid5(x, tuple(grid_shape) if grid_shape is not None else None)
    res = out if out is not None else torch.empty(2, dtype=torch.float64, device=x.device)
    with torch.cuda.device(x.device):
        st = lib.gft_raymarch_check(_p(x), code, _lib.i64(shape5), _p(Mh), nm, _p(Vh), _p(Ph), _p(Fh), nv,
                                    _lib.i32(_shape3(output_shape)), _p(y), int(ray_stride), _p(res),
                                    _stream(x.device))
    _lib.check(st, 'RaymarchCheck')
    return res
