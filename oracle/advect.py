"""Advection of a density grid by a staggered velocity grid, float64.

Follows VelocityGrid (data_structures.py:380-1072):
  component_shapes (:381-389): x [D,H,W+1], y [D,H+1,W], z [D+1,H,W]
  centered (:819-833): mean of the two faces per axis
  centered_lut_grid (:864-868): lut = -dt * centered
  warp (:870-905): SL = SampleGridLut(d, lut, relative, LINEAR, cell offset 0);
      MacCormack: corr = fwd + 0.5*(d - SampleGridLut(fwd, -lut));
      MC_SMOOTH: corr -> fwd where corr < min or corr > max, min/max being the
      MIN/MAX lookups of d at the forward backtrace; NEGATIVE: max(., 0).
The gradient is the adjoint of that composition as TF differentiates it: the
SampleGridLut gradient op for each lookup (count-normalised input gradient in
reference mode), ``where`` routing, and no gradient through min/max.

Test infrastructure only; see the package docstring.
"""
import numpy as np

from . import sampling as S
from . import resample as R


def centered(vx, vy, vz):
    """[D,H,W+1,1], [D,H+1,W,1], [D+1,H,W,1] -> [D,H,W,3] (x, y, z)."""
    cx = (vx[:, :, 1:, 0] + vx[:, :, :-1, 0]) * 0.5
    cy = (vy[:, 1:, :, 0] + vy[:, :-1, :, 0]) * 0.5
    cz = (vz[1:, :, :, 0] + vz[:-1, :, :, 0]) * 0.5
    return np.stack([cx, cy, cz], axis=-1)


def centered_adjoint(g):
    """Adjoint of ``centered``: [D,H,W,3] -> (gx, gy, gz) staggered."""
    D, H, W, _ = g.shape
    gx = np.zeros((D, H, W + 1, 1))
    gy = np.zeros((D, H + 1, W, 1))
    gz = np.zeros((D + 1, H, W, 1))
    gx[:, :, 1:, 0] += 0.5 * g[..., 0]
    gx[:, :, :-1, 0] += 0.5 * g[..., 0]
    gy[:, 1:, :, 0] += 0.5 * g[..., 1]
    gy[:, :-1, :, 0] += 0.5 * g[..., 1]
    gz[1:, :, :, 0] += 0.5 * g[..., 2]
    gz[:-1, :, :, 0] += 0.5 * g[..., 2]
    return gx, gy, gz


def _lut(vbar, dt):
    l = -dt * vbar
    return np.concatenate([l, np.zeros(l.shape[:-1] + (1,))], axis=-1)[None]


def _lookup(d, lut, filt, boundary):
    return R.sample_grid_lut(d[None], lut, filter_mode=filt, boundary=boundary,
                             separate_camera_batch=False, relative=True)[0, 0]


def warp(d, vx, vy, vz, dt=1.0, order=1, clamp='NONE', boundary=S.CLAMP, return_parts=False):
    """d [D,H,W,C]; returns the advected [D,H,W,C] (and intermediates)."""
    d = np.asarray(d, dtype=np.float64)
    lut = _lut(centered(vx, vy, vz), dt)
    fwd = _lookup(d, lut, S.LINEAR, boundary)
    parts = {'lut': lut, 'fwd': fwd}
    out = fwd
    clamp = clamp.upper()
    if order == 2:
        back = _lookup(fwd, -lut, S.LINEAR, boundary)
        corr = fwd + 0.5 * (d - back)
        oob = np.zeros(corr.shape, dtype=bool)
        if clamp in ('MC', 'MC_SMOOTH'):
            mn = _lookup(d, lut, S.MIN, boundary)
            mx = _lookup(d, lut, S.MAX, boundary)
            if clamp == 'MC':
                raise NotImplementedError('clamp MC is rejected by the reference (data_structures.py:890-892)')
            oob = (corr < mn) | (corr > mx)
            corr = np.where(oob, fwd, corr)
        parts.update(back=back, oob=oob)
        out = corr
    elif order != 1:
        raise ValueError(order)
    if clamp == 'NEGATIVE':
        parts['neg_mask'] = out >= 0
        out = np.maximum(out, 0.0)
    return (out, parts) if return_parts else out


def warp_grad(d, vx, vy, vz, g_out, dt=1.0, order=1, clamp='NONE', boundary=S.CLAMP, exact=False):
    """Gradient of ``warp`` w.r.t. d and the staggered components.
    Returns (gd [D,H,W,C], gvx, gvy, gvz)."""
    d = np.asarray(d, dtype=np.float64)
    g_out = np.asarray(g_out, dtype=np.float64)
    _, p = warp(d, vx, vy, vz, dt, order, clamp, boundary, return_parts=True)
    lut = p['lut']
    if clamp.upper() == 'NEGATIVE':
        g_out = np.where(p['neg_mask'], g_out, 0.0)

    def lut_grad(src, g, l):
        gs, gl = R.sample_grid_lut_grad(src[None], g[None, None], l, filter_mode=S.LINEAR,
                                        boundary=boundary, separate_camera_batch=False,
                                        relative=True, exact=exact)
        return gs[0], gl[0]

    gd = np.zeros_like(d)
    glut = np.zeros(lut.shape[1:])
    if order == 2:
        oob = p['oob']
        g_fwd = g_out.copy()
        g_corr = np.where(oob, 0.0, g_out)
        gd += 0.5 * g_corr
        g_back = -0.5 * g_corr
        gf2, gl2 = lut_grad(p['fwd'], g_back, -lut)
        g_fwd += gf2
        glut -= gl2
    else:
        g_fwd = g_out
    gd2, gl1 = lut_grad(d, g_fwd, lut)
    gd += gd2
    glut += gl1
    gvbar = -dt * glut[..., :3]
    gvx, gvy, gvz = centered_adjoint(gvbar)
    return gd, gvx, gvy, gvz
