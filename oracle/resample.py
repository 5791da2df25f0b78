"""SampleGridTransform / SampleGridLut / LodTransform ops and their gradients, float64.

Test infrastructure only; see the package docstring.
"""
import numpy as np

from . import sampling as S
from . import transforms as T


def _out_coords(D, H, W):
    z, y, x = np.meshgrid(np.arange(D, dtype=np.float64), np.arange(H, dtype=np.float64),
                          np.arange(W, dtype=np.float64), indexing='ij')
    return np.stack([x, y, z], axis=-1)


def sample_grid_transform(x, M, V, P, F, out_shape, filter_mode=S.LINEAR, boundary=S.BORDER,
                          mip_mode=S.MIP_NONE, num_mips=0, mip_bias=0.0,
                          coord_mode=T.LINDEPTH, separate_camera_batch=True, out_box=None, mips=None):
    """SampleGridTransform (resample_grid.cc:23-61, :268-447; kSample3D
    resample_grid.cu.cc:240-252; launcher :289-438).
    x [N,D,H,W,C] -> [N, V (or 1), Do, Ho, Wo, C].  Only LINEAR/NEAREST filtering
    and BORDER/CLAMP boundaries reach a fetch in this op (Sampler2::_internal_fetch3D,
    sampling.hpp:567-585); other combinations give 0.  ``out_box`` = ((z0, z1),
    (y0, y1), (x0, x1)) computes only that box of output cells and returns
    [N, V (or 1), z1-z0, y1-y0, x1-x0, C].  ``mips``: the pyramid of a
    one-slice input as build_mips returns it, if already built."""
    x = np.asarray(x, dtype=np.float64)
    N, C = x.shape[0], x.shape[4]
    Do, Ho, Wo = out_shape
    dims_in = S.dims_xyz(x[0])
    dims_out = np.array([Wo, Ho, Do], dtype=np.int64)
    nv = len(V) if separate_camera_batch else 1
    use_mip = mip_mode != S.MIP_NONE
    L = S.usable_mip_levels(x.shape[1:4], num_mips) if use_mip else 0
    idx = _out_coords(Do, Ho, Wo) + 0.5
    if out_box is not None:
        (z0, z1), (y0, y1), (x0, x1) = out_box
        idx = idx[z0:z1, y0:y1, x0:x1]
    out = np.zeros((N, nv) + idx.shape[:3] + (C,))
    if filter_mode not in (S.LINEAR, S.NEAREST) or boundary not in (S.BORDER, S.CLAMP):
        return out
    for b in range(N):
        if mips is not None and N == 1:
            pyr = mips[:L + 1] if use_mip else mips[:1]
        else:
            pyr = S.build_mips(x[b], L) if use_mip else [x[b]]
        cams = range(len(V)) if separate_camera_batch else [b]
        for vi, c in enumerate(cams):
            cam = T.CameraXform(M[b], V[c], P[c], F[c])
            pos = T.sample_positions(cam, coord_mode, idx, dims_in, dims_out, use_mip)
            out[b, vi] = S.sample_mipmapped(pyr, pos, filter_mode, boundary,
                                            mip_mode if (use_mip and True) else S.MIP_NONE,
                                            mip_bias, 0.5, L)
    return out


def sample_grid_transform_grad(x, dy, M, V, P, F, boundary=S.BORDER,
                               coord_mode=T.LINDEPTH, separate_camera_batch=True, exact=False):
    """Scatter adjoint of SampleGridTransform without mips
    (SampleGridGradKernelLauncher, resample_grid.cu.cc:863-1018: kScatter3DGradients
    :841-861 then kNormalize3DGradients :814-832, dividing by the per-voxel count of
    reached corners once per batch).  The reference always scatters trilinearly.
    dy [N, V, Do, Ho, Wo, C] -> [N, D, H, W, C]."""
    x = np.asarray(x, dtype=np.float64)
    dy = np.asarray(dy, dtype=np.float64)
    N, C = x.shape[0], x.shape[4]
    Do, Ho, Wo = dy.shape[2:5]
    dims_in = S.dims_xyz(x[0])
    dims_out = np.array([Wo, Ho, Do], dtype=np.int64)
    idx = _out_coords(Do, Ho, Wo) + 0.5
    gx = np.zeros_like(x)
    for b in range(N):
        cnt = np.zeros(x.shape[1:4])
        cams = range(len(V)) if separate_camera_batch else [b]
        for vi, c in enumerate(cams):
            cam = T.CameraXform(M[b], V[c], P[c], F[c])
            pos = T.sample_positions(cam, coord_mode, idx, dims_in, dims_out, False)[..., :3]
            S.scatter_linear(gx[b], pos - 0.5, dy[b, vi], boundary, cnt, exact_window=exact)
        if not exact:
            nz = cnt > 0
            gx[b][nz] /= cnt[nz][:, None]
    return gx


def _lut_positions(lut, relative, normalized):
    """kSampleGrid3DLuT position set-up (resample_grid.cu.cc:468-478): the lookup
    xyz is scaled by the OUTPUT dims when normalized, then offset by the integer
    output index when relative; w (the LOD) is kept."""
    pos = np.asarray(lut, dtype=np.float64).copy()
    Do, Ho, Wo = pos.shape[:3]
    if normalized:
        pos[..., :3] *= np.array([Wo, Ho, Do], dtype=np.float64)
    if relative:
        pos[..., :3] += _out_coords(Do, Ho, Wo)
    return pos


def sample_grid_lut(x, lut, filter_mode=S.LINEAR, boundary=S.BORDER, mip_mode=S.MIP_NONE,
                    num_mips=0, mip_bias=0.0, cell_center_offset=0.0,
                    separate_camera_batch=True, relative=True, normalized=False):
    """SampleGridLut (resample_grid.cc:86-109, :650-802; kSampleGrid3DLuT
    resample_grid.cu.cc:465-484).  x [N,D,H,W,C], lut [V,Do,Ho,Wo,4] ->
    [N, V (or 1), Do, Ho, Wo, C]."""
    x = np.asarray(x, dtype=np.float64)
    lut = np.asarray(lut, dtype=np.float64)
    N, C = x.shape[0], x.shape[4]
    nv = lut.shape[0] if separate_camera_batch else 1
    out = np.zeros((N, nv) + lut.shape[1:4] + (C,))
    use_mip = mip_mode != S.MIP_NONE
    L = S.usable_mip_levels(x.shape[1:4], num_mips) if use_mip else 0
    for b in range(N):
        mips = S.build_mips(x[b], L) if use_mip else [x[b]]
        cams = range(lut.shape[0]) if separate_camera_batch else [b]
        for vi, c in enumerate(cams):
            pos = _lut_positions(lut[c], relative, normalized)
            if use_mip:
                out[b, vi] = S.sample_mipmapped(mips, pos, filter_mode, boundary, mip_mode,
                                                mip_bias, cell_center_offset, L)
            else:
                out[b, vi] = S.fetch(x[b], pos[..., :3] - cell_center_offset, filter_mode, boundary)
    return out


def sample_grid_lut_grad(x, dy, lut, filter_mode=S.LINEAR, boundary=S.BORDER,
                         cell_center_offset=0.0, separate_camera_batch=True, relative=True,
                         normalized=False, exact=False):
    """SampleGridLutGrad (resample_grid.cc:113-134, :828-979;
    kScatterLuT3DGradients resample_grid.cu.cc:1051-1081, launcher :1083-1251).
    Input gradient: trilinear scatter for every filter mode, divided by the
    per-voxel count of reached corners once per batch (reference mode).
    Lookup gradient (LINEAR only, else 0): (sum_c dy*d/dx, sum_c dy*d/dy,
    sum_c dy*d/dz, 0) at the sample position, WRITTEN per camera, so with N > 1
    the last batch wins (reference behaviour kept).  The lookup gradient is not
    scaled by the normalisation of ``normalized`` coordinates (as in the
    reference).  Returns (dx [N,D,H,W,C], dlut [V,Do,Ho,Wo,4])."""
    x = np.asarray(x, dtype=np.float64)
    dy = np.asarray(dy, dtype=np.float64)
    lut = np.asarray(lut, dtype=np.float64)
    N, C = x.shape[0], x.shape[4]
    gx = np.zeros_like(x)
    glut = np.zeros_like(lut)
    for b in range(N):
        cnt = np.zeros(x.shape[1:4])
        cams = range(lut.shape[0]) if separate_camera_batch else [b]
        for vi, c in enumerate(cams):
            pos = _lut_positions(lut[c], relative, normalized)[..., :3] - cell_center_offset
            g = dy[b, vi]
            if filter_mode == S.LINEAR:
                ddx, ddy, ddz = S.fetch_grad(x[b], pos, boundary)
                glut[c, ..., 0] = np.sum(g * ddx, axis=-1)
                glut[c, ..., 1] = np.sum(g * ddy, axis=-1)
                glut[c, ..., 2] = np.sum(g * ddz, axis=-1)
                glut[c, ..., 3] = 0.0
            S.scatter_linear(gx[b], pos, g, boundary, cnt, exact_window=exact)
        if not exact:
            nz = cnt > 0
            gx[b][nz] /= cnt[nz][:, None]
    return gx, glut


def lod_transform(in_shape, MV, P, F, out_shape, inverse=False):
    """LodTransform (resample_grid.cc:136-154, :986-1064; kComputeLoD3D
    resample_grid.cu.cc:1288-1300): per output cell, the sampling position
    (samplePos3D<CM,false>) with w = calcLoD(...).w, for CM = LINDEPTH or
    LINDEPTH_REVERSE.  MV [V,16] already holds the model-view matrix (M = I).
    Returns [V, Do, Ho, Wo, 4]."""
    Do, Ho, Wo = out_shape
    dims_in = np.array([in_shape[2], in_shape[1], in_shape[0]], dtype=np.int64)
    dims_out = np.array([Wo, Ho, Do], dtype=np.int64)
    cm = T.LINDEPTH_REVERSE if inverse else T.LINDEPTH
    idx = _out_coords(Do, Ho, Wo) + 0.5
    eye = np.eye(4).T.reshape(-1)
    out = np.zeros((len(MV), Do, Ho, Wo, 4))
    for v in range(len(MV)):
        cam = T.CameraXform(eye, MV[v], P[v], F[v])
        pos = T.sample_positions(cam, cm, idx, dims_in, dims_out, False)
        out[v, ..., :3] = pos[..., :3]
        out[v, ..., 3] = T.calc_lod(cam, cm, idx, dims_in, dims_out)[..., 3]
    return out
