"""Fused raymarch op (RaymarchGridTransform and its gradient), float64.

Forward: kRaymarchGridTransformLindepth (raymarch_grid.cu.cc:107-143) driven by
RaymarchGridKernelLauncher (:222-294).  Per pixel (x, y) of an H x W image with
D depth samples: the ray runs from IDXtoOS(x+.5, y+.5, 0.5) to
IDXtoOS(x+.5, y+.5, zMax+.5), zMax = max(D-1, 1), in D uniform object-space
steps (non-linear NDC depth at the end points), each sample is fetched with
sample3D (sampling_v2.hpp:358-372) and blended front to back.

Gradient: kRaymarchGridTransformLindepthGrad (:343-372) walks back to front,
re-samples, applies blendGradients and scatters with trilinear weights; the
launcher (:451-574) normalises per camera by the per-voxel sum of weights
(NORMALIZE_GRADIENT_BY_WEIGHT, raymarch_grid.hpp:22-42) before summing the
cameras.  ``exact=True`` omits that normalisation and scatters only where the
forward samples (the true adjoint).

Test infrastructure only; see the package docstring.
"""
import numpy as np

from . import sampling as S
from . import transforms as T
from . import blend as B


def ray_endpoints(cam, H, W, D):
    """Near/far object-space positions of all pixels and the step, (H, W, 3)."""
    dims_out = np.array([W, H, D], dtype=np.float64)
    zmax = float(max(D - 1, 1))
    ys, xs = np.meshgrid(np.arange(H, dtype=np.float64), np.arange(W, dtype=np.float64), indexing='ij')
    near_idx = np.stack([xs + 0.5, ys + 0.5, np.full_like(xs, 0.5)], axis=-1)
    far_idx = np.stack([xs + 0.5, ys + 0.5, np.full_like(xs, zmax + 0.5)], axis=-1)
    near = T.idx_to_os(cam, near_idx, dims_out)
    far = T.idx_to_os(cam, far_idx, dims_out)
    return near, far, (far - near) / zmax


def _sample(grid, pos, filter_mode, boundary):
    return S.fetch(grid, pos - 0.5, filter_mode, boundary, raymarch_extrema=True)


def _cams(M, V, P, F, n, b, separate_camera_batch):
    nc = len(V)
    cams = range(nc) if separate_camera_batch else [b]
    return [(c, T.CameraXform(M[b], V[c], P[c], F[c])) for c in cams]


def _window(rows, cols, c):
    """Image window of camera index c: ``rows``/``cols`` are slices or, per
    camera, lists of slices."""
    r = rows[c] if isinstance(rows, (list, tuple)) else rows
    k = cols[c] if isinstance(cols, (list, tuple)) else cols
    return (slice(None) if r is None else r, slice(None) if k is None else k)


def raymarch_fwd(x, M, V, P, F, out_shape, filter_mode=S.LINEAR, boundary=S.BORDER,
                 blend_mode=B.BEER_LAMBERT, separate_camera_batch=True, rows=None, cols=None):
    """x [N,D,H,W,C]; M [N,16]; V,P [V,16]; F [V,6]; out_shape (D,H,W) of the frustum.
    Returns [N, V (or 1), H, W, C].  ``rows`` / ``cols`` optionally restrict the
    work to a window of image rows and columns (slices, or one slice per
    camera); the rest stay 0.  Used for bounded CPU timing and for checking
    the rays that reach a sub-block of a large grid."""
    x = np.asarray(x, dtype=np.float64)
    N, C = x.shape[0], x.shape[4]
    D, H, W = out_shape
    nv = len(V) if separate_camera_batch else 1
    out = np.zeros((N, nv, H, W, C))
    for b in range(N):
        for vi, (c, cam) in enumerate(_cams(M, V, P, F, N, b, separate_camera_batch)):
            rsel = _window(rows, cols, c)
            near, far, step = ray_endpoints(cam, H, W, D)
            near, step = near[rsel], step[rsel]
            acc = np.zeros(near.shape[:-1] + (C,))
            for i in range(D):
                pos = near + i * step
                acc = B.blend(blend_mode, acc, _sample(x[b], pos, filter_mode, boundary))
            out[b, vi if separate_camera_batch else 0][rsel] = acc
    return out


def raymarch_bwd(x, y, dy, M, V, P, F, out_shape, boundary=S.BORDER,
                 blend_mode=B.BEER_LAMBERT, separate_camera_batch=True, exact=False, rows=None, cols=None):
    """Gradient w.r.t. x of raymarch_fwd with LINEAR filtering (the only filter the
    gradient op accepts, raymarch_grid.cc:65).  y is the forward output, dy its
    gradient.  Returns [N,D,H,W,C].  With a window (``rows`` / ``cols``) only
    its rays contribute: exact at every voxel that no ray outside it reaches."""
    x = np.asarray(x, dtype=np.float64)
    y = np.asarray(y, dtype=np.float64)
    dy = np.asarray(dy, dtype=np.float64)
    N, C = x.shape[0], x.shape[4]
    D, H, W = out_shape
    gx = np.zeros_like(x)
    for b in range(N):
        for vi, (c, cam) in enumerate(_cams(M, V, P, F, N, b, separate_camera_batch)):
            ov = vi if separate_camera_batch else 0
            buf, cnt = camera_scatter(x[b], y[b, ov], dy[b, ov], cam, out_shape, _window(rows, cols, c), boundary,
                                      blend_mode, exact)
            if exact:
                gx[b] += buf
            else:
                nz = cnt > 0
                gx[b][nz] += buf[nz] / cnt[nz][:, None]
    return gx


def camera_scatter(xb, yv, dyv, cam, out_shape, window, boundary=S.BORDER, blend_mode=B.BEER_LAMBERT, exact=False):
    """The per-camera part of raymarch_bwd before normalisation: the trilinear
    scatter of the blend adjoint over the rays of ``window`` (rows, cols) of
    one camera, and the per-voxel sum of the trilinear weights.
    xb [D,H,W,C]; yv, dyv [H,W,C].  Returns (buf [D,H,W,C], weight_sum [D,H,W])."""
    D, H, W = out_shape
    near, far, step = ray_endpoints(cam, H, W, D)
    near, step = near[window], step[window]
    acc = np.asarray(yv, dtype=np.float64)[window].copy()
    g = np.asarray(dyv, dtype=np.float64)[window].copy()
    buf = np.zeros(xb.shape, dtype=np.float64)
    cnt = np.zeros(xb.shape[:3])
    for i in range(D - 1, -1, -1):
        pos = near + i * step
        smp = _sample(xb, pos, S.LINEAR, boundary)
        gcell, g, acc = B.blend_gradients(blend_mode, g, smp, acc, exact)
        S.scatter_linear(buf, pos - 0.5, gcell, boundary, cnt, count_weights=True, exact_window=exact)
    return buf, cnt
