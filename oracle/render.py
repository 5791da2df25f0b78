"""Render composition of the reference (renderer.py / lighting.py), float64.

Light grid (ambient + spot light with the light-frustum shadow pass and the
point-light falloff), the depth-step pre-multiplication, the fused raymarch
per camera and the background composite of Renderer.render_density.

Test infrastructure only; see the package docstring.
"""
import numpy as np

from . import blend as B
from . import raymarch as RM
from . import resample as R
from . import sampling as S
from . import transforms as T


def point_falloff(grid_size_dhw, cell_size_ws, grid_size_ws, light_pos_grid_os, range_scale):
    """1/(1+(|x - x_L| s)^2) on cell centres in world-scaled grid units
    (PointLight.grid_lighting, lighting.py:49-71).  Returns [D,H,W,1]."""
    D, H, W = grid_size_dhw
    cs = np.asarray(cell_size_ws, dtype=np.float64)
    gs = np.asarray(grid_size_ws, dtype=np.float64)
    lp = np.asarray(light_pos_grid_os, dtype=np.float64)[:3] * cs
    xs = np.linspace(0.5 * cs[0], gs[0] - 0.5 * cs[0], W)
    ys = np.linspace(0.5 * cs[1], gs[1] - 0.5 * cs[1], H)
    zs = np.linspace(0.5 * cs[2], gs[2] - 0.5 * cs[2], D)
    z, y, x = np.meshgrid(zs - lp[2], ys - lp[1], xs - lp[0], indexing='ij')
    r = np.sqrt(x * x + y * y + z * z)[..., None]
    return 1.0 / (1.0 + (r * range_scale) ** 2)


def shadow_transmission(d, M, Vs, Ps, Fs, shadow_res, shadow_step, filter_mode=S.LINEAR, boundary=S.BORDER,
                        mip_mode=S.MIP_LINEAR, num_mips=2, mip_bias=0.0, blend_mode='BEER_LAMBERT'):
    """SpotLight._render_shadow_map (lighting.py:106-141) with cast_shadows and
    no cone mask: light-frustum resample of d*step (LINDEPTH, mips), inclusive
    depth sum, one-cell shift, transmission, back-projection (LINDEPTH_REVERSE,
    mips).  d [1,D,H,W,1] -> [D,H,W,1]."""
    sh = R.sample_grid_transform(d * shadow_step, M, Vs, Ps, Fs, shadow_res, filter_mode, boundary, mip_mode,
                                 num_mips, mip_bias, T.LINDEPTH)[0]  # [1,Ds,Hs,Ws,1]
    sh = B.reduce_grid_blend(sh, B.BEER_LAMBERT if blend_mode == 'BEER_LAMBERT' else B.ALPHA, True)
    if boundary == S.BORDER:
        pad = np.zeros_like(sh[:, :1])
    elif boundary == S.CLAMP:
        pad = sh[:, :1]
    else:
        pad = sh[:, -1:]
    sh = np.concatenate([pad, sh[:, :-1]], axis=1)
    tr = np.exp(-sh) if blend_mode == 'BEER_LAMBERT' else 1 - np.clip(sh, 0, 1)
    D, H, W = d.shape[1:4]
    back = R.sample_grid_transform(tr, M, Vs, Ps, Fs, (D, H, W), filter_mode, boundary, mip_mode, num_mips,
                                   mip_bias, T.LINDEPTH_REVERSE)
    return back[0, 0]


def render_fused(data, M, V, P, F, res, depth_step, boundary=S.BORDER, blend_mode=B.BEER_LAMBERT, background=None,
                 cut_alpha=True):
    """Renderer._render_cameras (fused) + render_density's composite
    (renderer.py:555-568, :626-640): data [1,D,H,W,4] -> list of [1,H,W,3|4]."""
    img = RM.raymarch_fwd(data * depth_step, M, V, P, F, res, S.LINEAR, boundary, blend_mode)[0]  # [V,H,W,4]
    t = np.exp(-img[..., -1:])
    if cut_alpha:
        img = img[..., :-1]
    if background is not None:
        img = img + np.asarray(background, dtype=np.float64)[:, None, None, :] * t
    return [img[i:i + 1] for i in range(img.shape[0])]
