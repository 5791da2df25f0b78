"""Grid fetches of the reference samplers, restated in float64 NumPy.

Conventions (reference ``kernel_setup.hpp:161-163``, ``vector_io.inl:12-20``):
grids are one NDHWC batch slice ``grid[D, H, W, C]``; positions are ``(..., 3)``
arrays in (x, y, z) = (W, H, D) order, already shifted so that cell centres are
at integer coordinates (the samplers subtract the cell-centre offset first).

Boundary modes (``sampling_settings_v2.hpp:9``): 0 BORDER, 1 CLAMP, 2 WRAP.
Filter modes: 0 NEAREST, 1 LINEAR, 2 MIN, 3 MAX.

Test infrastructure only; see the package docstring.
"""
import numpy as np

BORDER, CLAMP, WRAP = 0, 1, 2
NEAREST, LINEAR, MIN, MAX = 0, 1, 2, 3

# FLOAT_MAX of vectormath.hpp:13, stored as float32 by make_cudaFloat
FLOAT_MAX = float(np.float32(3.40282e38))


def dims_xyz(grid):
    """(W, H, D) of a [D, H, W, C] grid as an int64 array."""
    return np.array([grid.shape[2], grid.shape[1], grid.shape[0]], dtype=np.int64)


def _pmod(v, m):
    # vmath::positivemod (vectormath.hpp:262-266) is (v % m) + m*(v < 0) with C
    # truncating modulo; it yields m (out of range) for negative multiples of m.
    # The oracle uses the floor modulo, which agrees everywhere else.
    return np.mod(v, m)


def _flat(ix, iy, iz, dims):
    return (iz * dims[1] + iy) * dims[0] + ix


def _read(grid2, ix, iy, iz, dims, valid=None):
    """Gather grid2[flat] for integer corner indices; invalid corners read 0."""
    if valid is None:
        return grid2[_flat(ix, iy, iz, dims)]
    f = np.where(valid, _flat(np.clip(ix, 0, dims[0] - 1), np.clip(iy, 0, dims[1] - 1),
                              np.clip(iz, 0, dims[2] - 1), dims), 0)
    return np.where(valid[..., None], grid2[f], 0.0)


def _corners(pos, dims, boundary):
    """floor/ceil indices (after boundary remap), ceil weights and validity.

    Follows read3DInterpolated (sampling.hpp:175-255, sampling_v2.hpp:38-123):
    weights = fract(pos) = pos - floor(pos); ceil = ceilf(pos) (equal to floor
    for integral positions, where its weight is 0)."""
    pos = np.asarray(pos, dtype=np.float64)
    fl = np.floor(pos)
    ce = np.ceil(pos)
    w = pos - fl
    fl = fl.astype(np.int64)
    ce = ce.astype(np.int64)
    if boundary == BORDER:
        fv = (fl > -1) & (fl < dims)
        cv = (ce > -1) & (ce < dims)
    else:
        if boundary == CLAMP:
            fl = np.clip(fl, 0, dims - 1)
            ce = np.clip(ce, 0, dims - 1)
        elif boundary == WRAP:
            fl = _pmod(fl, dims)
            ce = _pmod(ce, dims)
        fv = np.ones(fl.shape, dtype=bool)
        cv = np.ones(ce.shape, dtype=bool)
    return fl, ce, w, fv, cv


def _border_inside(pos, dims):
    """BORDER early-out test: 0 <= pos + 0.5 < dims on every axis
    (sampling_v2.hpp:49-51, sampling.hpp:183-185)."""
    p = np.asarray(pos, dtype=np.float64) + 0.5
    return np.all((p >= 0) & (p < dims), axis=-1)


def _eight(grid, pos, boundary):
    """The 8 corner values (order fff, cff, fcf, ccf, ffc, cfc, fcc, ccc) with
    their validity, and the ceil weights."""
    dims = dims_xyz(grid)
    C = grid.shape[3]
    g2 = grid.reshape(-1, C)
    fl, ce, w, fv, cv = _corners(pos, dims, boundary)
    vals, valid = [], []
    for sz in (0, 1):
        for sy in (0, 1):
            for sx in (0, 1):
                ix = ce[..., 0] if sx else fl[..., 0]
                iy = ce[..., 1] if sy else fl[..., 1]
                iz = ce[..., 2] if sz else fl[..., 2]
                v = (cv[..., 0] if sx else fv[..., 0]) & (cv[..., 1] if sy else fv[..., 1]) & \
                    (cv[..., 2] if sz else fv[..., 2])
                vals.append(_read(g2, ix, iy, iz, dims, v))
                valid.append(v)
    return vals, valid, w


def _lerp(a, b, t):
    return a + t[..., None] * (b - a)


def fetch_linear(grid, pos, boundary):
    """Trilinear fetch (read3DInterpolated, sampling_v2.hpp:38-123)."""
    dims = dims_xyz(grid)
    vals, _, w = _eight(grid, pos, boundary)
    v00 = _lerp(vals[0], vals[1], w[..., 0])
    v01 = _lerp(vals[2], vals[3], w[..., 0])
    v0 = _lerp(v00, v01, w[..., 1])
    v10 = _lerp(vals[4], vals[5], w[..., 0])
    v11 = _lerp(vals[6], vals[7], w[..., 0])
    v1 = _lerp(v10, v11, w[..., 1])
    out = _lerp(v0, v1, w[..., 2])
    if boundary == BORDER:
        out = np.where(_border_inside(pos, dims)[..., None], out, 0.0)
    return out


def fetch_nearest(grid, pos, boundary):
    """Nearest fetch: idx = int(pos + 0.5), a truncation toward zero
    (read3DNearest, sampling_v2.hpp:124-139, sampling.hpp:354-371)."""
    dims = dims_xyz(grid)
    C = grid.shape[3]
    idx = np.trunc(np.asarray(pos, dtype=np.float64) + 0.5).astype(np.int64)
    if boundary == BORDER:
        inside = np.all((idx >= 0) & (idx < dims), axis=-1)
        return _read(grid.reshape(-1, C), idx[..., 0], idx[..., 1], idx[..., 2], dims, inside)
    if boundary == CLAMP:
        idx = np.clip(idx, 0, dims - 1)
    elif boundary == WRAP:
        idx = _pmod(idx, dims)
    return grid.reshape(-1, C)[_flat(idx[..., 0], idx[..., 1], idx[..., 2], dims)]


def fetch_extremum_lut(grid, pos, boundary, is_max):
    """MIN/MAX of the 8 corners as used by SampleGridLut / SampleGridTransform
    (read3DMin / read3DMax, sampling.hpp:372-491): under BORDER the result is 0
    outside the half-cell-extended domain, and starts at 0 (instead of +-FLOAT_MAX)
    when any corner is invalid."""
    dims = dims_xyz(grid)
    vals, valid, _ = _eight(grid, pos, boundary)
    shape = vals[0].shape
    if boundary == BORDER:
        allvalid = np.all(np.stack(valid, 0), axis=0)
        start = np.where(allvalid, -FLOAT_MAX if is_max else FLOAT_MAX, 0.0)
        acc = np.broadcast_to(start[..., None], shape).copy()
        for v, ok in zip(vals, valid):
            cand = np.maximum(acc, v) if is_max else np.minimum(acc, v)
            acc = np.where(ok[..., None], cand, acc)
        return np.where(_border_inside(pos, dims)[..., None], acc, 0.0)
    acc = np.full(shape, -FLOAT_MAX if is_max else FLOAT_MAX)
    for v in vals:
        acc = np.maximum(acc, v) if is_max else np.minimum(acc, v)
    return acc


def fetch_extremum_raymarch(grid, pos, boundary, is_max):
    """MIN/MAX as used by the fused raymarch (read3DInterpolatedWithExtrema,
    sampling_v2.hpp:158-256).  The running extremum starts at +-FLOAT_MAX and
    is updated per valid corner as m = m + t*(v - m), t = (v < m) resp. (m < v)
    (read3DWithExtrema, sampling_v2.hpp:149-156), in the corner order fff, cff,
    fcf, ccf, ffc, cfc, fcc, ccc (the argument evaluation order the reference
    build uses; pinned by the golden vectors).  The first update cancels
    against FLOAT_MAX to exactly 0, so the result is the extremum of 0 and the
    corners after the first valid one.  Under BORDER a position outside returns
    the start value."""
    dims = dims_xyz(grid)
    vals, valid, _ = _eight(grid, pos, boundary)
    shape = vals[0].shape
    acc = np.full(shape, -FLOAT_MAX if is_max else FLOAT_MAX)
    for v, ok in zip(vals, valid):
        t = (acc < v) if is_max else (v < acc)
        cand = acc + t * (v - acc)
        acc = np.where(ok[..., None], cand, acc)
    if boundary == BORDER:
        acc = np.where(_border_inside(pos, dims)[..., None], acc,
                       -FLOAT_MAX if is_max else FLOAT_MAX)
    return acc


def fetch(grid, pos, filter_mode, boundary, raymarch_extrema=False):
    if filter_mode == LINEAR:
        return fetch_linear(grid, pos, boundary)
    if filter_mode == NEAREST:
        return fetch_nearest(grid, pos, boundary)
    if filter_mode in (MIN, MAX):
        f = fetch_extremum_raymarch if raymarch_extrema else fetch_extremum_lut
        return f(grid, pos, boundary, filter_mode == MAX)
    raise ValueError(filter_mode)


def fetch_grad(grid, pos, boundary):
    """Spatial derivative of the trilinear fetch w.r.t. (x, y, z)
    (read3DGrad, sampling.hpp:257-352, sampling_v2.hpp:262-356)."""
    dims = dims_xyz(grid)
    v, _, w = _eight(grid, pos, boundary)
    fff, cff, fcf, ccf, ffc, cfc, fcc, ccc = v
    wx, wy, wz = w[..., 0], w[..., 1], w[..., 2]
    dx = _lerp(_lerp(cff - fff, ccf - fcf, wy), _lerp(cfc - ffc, ccc - fcc, wy), wz)
    dy = _lerp(_lerp(fcf - fff, ccf - cff, wx), _lerp(fcc - ffc, ccc - cfc, wx), wz)
    dz = _lerp(_lerp(ffc - fff, cfc - cff, wx), _lerp(fcc - fcf, ccc - ccf, wx), wy)
    if boundary == BORDER:
        inside = _border_inside(pos, dims)[..., None]
        dx, dy, dz = (np.where(inside, a, 0.0) for a in (dx, dy, dz))
    return dx, dy, dz


def scatter_linear(grad, pos, values, boundary, count=None, count_weights=False, exact_window=False):
    """Trilinear scatter adjoint with the reference's bounds handling.

    grad:   [D, H, W, C] accumulator (modified in place)
    values: (..., C) gradient to distribute to the 8 corners with trilinear weights
    count:  optional [D, H, W] accumulator; +1 per reached corner (the uint32
            counter of scatterGradInterpolated, resample_grid.cu.cc:760-812) or
            +w when ``count_weights`` (SingleSampleContribution<float>,
            sampling_v2.hpp:443-456).

    BORDER: the sample is dropped unless -1 < pos < dims on every axis, and each
    corner is dropped when outside [0, dims) (resample_grid.cu.cc:762, 776-805;
    sampling_v2.hpp:461, 445-447).  This window is wider than the forward's
    half-cell cut-off, so the reference adjoint is not exact there;
    ``exact_window`` applies the forward's cut-off instead (the true adjoint)."""
    dims = dims_xyz(grad)
    C = grad.shape[3]
    pos = np.asarray(pos, dtype=np.float64).reshape(-1, 3)
    values = np.asarray(values, dtype=np.float64).reshape(-1, C)
    g2 = grad.reshape(-1, C)
    c2 = count.reshape(-1) if count is not None else None
    if boundary == BORDER:
        if exact_window:
            keep = _border_inside(pos, dims)
        else:
            keep = np.all((pos > -1) & (pos < dims), axis=-1)
        pos, values = pos[keep], values[keep]
    fl, ce, w, fv, cv = _corners(pos, dims, boundary)
    for sz in (0, 1):
        for sy in (0, 1):
            for sx in (0, 1):
                ix = ce[:, 0] if sx else fl[:, 0]
                iy = ce[:, 1] if sy else fl[:, 1]
                iz = ce[:, 2] if sz else fl[:, 2]
                wt = (w[:, 0] if sx else 1 - w[:, 0]) * (w[:, 1] if sy else 1 - w[:, 1]) * \
                     (w[:, 2] if sz else 1 - w[:, 2])
                ok = (cv[:, 0] if sx else fv[:, 0]) & (cv[:, 1] if sy else fv[:, 1]) & \
                     (cv[:, 2] if sz else fv[:, 2])
                f = _flat(ix[ok], iy[ok], iz[ok], dims)
                np.add.at(g2, f, values[ok] * wt[ok, None])
                if c2 is not None:
                    np.add.at(c2, f, wt[ok] if count_weights else 1.0)


# --- mip pyramid -------------------------------------------------------------

def build_mips(grid, levels):
    """Box-filter pyramid: level m+1 is the 2x2x2 mean of level m, dims >> 1
    (kGenerateMip3D, resample_grid.cu.cc:46-72; MipAtlas3D::generate, :169-197).
    Returns [level0 (the input), level1, ..., level_levels]."""
    out = [np.asarray(grid, dtype=np.float64)]
    for _ in range(levels):
        g = out[-1]
        D, H, W = g.shape[0] >> 1, g.shape[1] >> 1, g.shape[2] >> 1
        g = g[:2 * D, :2 * H, :2 * W]
        z = (g[0::2] + g[1::2]) * 0.5
        y = (z[:, 0::2] + z[:, 1::2]) * 0.5
        x = (y[:, :, 0::2] + y[:, :, 1::2]) * 0.5
        out.append(x)
    return out


def usable_mip_levels(shape_dhw, num_mips):
    """setupMipAtlas (resample_grid.cc:201-220): the level count shrinks to the
    last level whose grid is non-empty."""
    L = int(num_mips)
    for m in range(1, L + 1):
        if (shape_dhw[0] >> m) * (shape_dhw[1] >> m) * (shape_dhw[2] >> m) <= 0:
            return m - 1
    return L


MIP_NONE, MIP_NEAREST, MIP_LINEAR = 0, 1, 2


def sample_mipmapped(mips, pos4, filter_mode, boundary, mip_mode, mip_bias,
                     cell_center_offset, max_level):
    """Sampler2::sample3D / Sampling::sample3D with mips (sampling.hpp:551-620, 690-712).

    pos4: (..., 4) position in coordinates (cell centres at +cell_center_offset)
    with the LOD in w.  Level m is fetched at pos/2^m - cell_center_offset on a
    grid of dims >> m."""
    pos4 = np.asarray(pos4, dtype=np.float64)
    xyz = pos4[..., :3]
    if mip_mode == MIP_NONE:
        return fetch(mips[0], xyz - cell_center_offset, filter_mode, boundary)
    lod = np.clip(pos4[..., 3] + mip_bias, 0.0, float(max_level))
    if mip_mode == MIP_NEAREST:
        lf = np.minimum((lod + 0.5).astype(np.int64), max_level)
    else:
        lf = np.minimum(lod.astype(np.int64), max_level)
    C = mips[0].shape[3]
    out = np.zeros(xyz.shape[:-1] + (C,))
    for m in range(max_level + 1):
        sel = lf == m
        if np.any(sel):
            out[sel] = fetch(mips[m], xyz[sel] / float(1 << m) - cell_center_offset,
                             filter_mode, boundary)
    if mip_mode == MIP_LINEAR:
        lc = np.minimum(np.ceil(lod).astype(np.int64), max_level)
        t = lod - np.floor(lod)
        for m in range(max_level + 1):
            sel = (lc == m) & (lc > lf)
            if np.any(sel):
                hi = fetch(mips[m], xyz[sel] / float(1 << m) - cell_center_offset,
                           filter_mode, boundary)
                out[sel] = out[sel] + t[sel, None] * (hi - out[sel])
    return out
