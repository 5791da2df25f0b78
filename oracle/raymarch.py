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


def raymarch_fwd(x, M, V, P, F, out_shape, filter_mode=S.LINEAR, boundary=S.BORDER,
                 blend_mode=B.BEER_LAMBERT, separate_camera_batch=True, rows=None):
    """x [N,D,H,W,C]; M [N,16]; V,P [V,16]; F [V,6]; out_shape (D,H,W) of the frustum.
    Returns [N, V (or 1), H, W, C].  ``rows`` optionally restricts the work to a
    subset of image rows (the rest stay 0), used for bounded CPU timing."""
    x = np.asarray(x, dtype=np.float64)
    N, C = x.shape[0], x.shape[4]
    D, H, W = out_shape
    nv = len(V) if separate_camera_batch else 1
    out = np.zeros((N, nv, H, W, C))
    rsel = slice(None) if rows is None else rows
    for b in range(N):
        for vi, (c, cam) in enumerate(_cams(M, V, P, F, N, b, separate_camera_batch)):
            near, far, step = ray_endpoints(cam, H, W, D)
            near, step = near[rsel], step[rsel]
            acc = np.zeros(near.shape[:-1] + (C,))
            for i in range(D):
                pos = near + i * step
                acc = B.blend(blend_mode, acc, _sample(x[b], pos, filter_mode, boundary))
            out[b, vi if separate_camera_batch else 0][rsel] = acc
    return out


def raymarch_bwd(x, y, dy, M, V, P, F, out_shape, boundary=S.BORDER,
                 blend_mode=B.BEER_LAMBERT, separate_camera_batch=True, exact=False, rows=None):
    """Gradient w.r.t. x of raymarch_fwd with LINEAR filtering (the only filter the
    gradient op accepts, raymarch_grid.cc:65).  y is the forward output, dy its
    gradient.  Returns [N,D,H,W,C]."""
    x = np.asarray(x, dtype=np.float64)
    y = np.asarray(y, dtype=np.float64)
    dy = np.asarray(dy, dtype=np.float64)
    N, C = x.shape[0], x.shape[4]
    D, H, W = out_shape
    gx = np.zeros_like(x)
    rsel = slice(None) if rows is None else rows
    for b in range(N):
        for vi, (c, cam) in enumerate(_cams(M, V, P, F, N, b, separate_camera_batch)):
            near, far, step = ray_endpoints(cam, H, W, D)
            near, step = near[rsel], step[rsel]
            ov = vi if separate_camera_batch else 0
            acc = y[b, ov][rsel].copy()
            g = dy[b, ov][rsel].copy()
            buf = np.zeros_like(x[b])
            cnt = np.zeros(x.shape[1:4])
            for i in range(D - 1, -1, -1):
                pos = near + i * step
                smp = _sample(x[b], pos, S.LINEAR, boundary)
                gcell, g, acc = B.blend_gradients(blend_mode, g, smp, acc, exact)
                S.scatter_linear(buf, pos - 0.5, gcell, boundary, cnt, count_weights=True, exact_window=exact)
            if exact:
                gx[b] += buf
            else:
                nz = cnt > 0
                gx[b][nz] += buf[nz] / cnt[nz][:, None]
    return gx
