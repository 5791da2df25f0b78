"""One render + advect iteration (forward and backward) in float64.

TEST INFRASTRUCTURE ONLY (imported by tests/ and bench.py's CPU legs).

The iteration is the reconstruction step of the reference restated over this
oracle's ops:

    d      = warp(d_prev, v)                         data_structures.py:870-905
    sh     = SampleGridTransform(d * s_sh, LINDEPTH, mips)       lighting.py:106-118
    tr     = exp(-shift(ReduceGridBlend(sh, BEER_LAMBERT)))      lighting.py:119-131
    trv    = SampleGridTransform(tr, LINDEPTH_REVERSE, mips)     lighting.py:132-141
    light  = d * (trv * falloff * colour + ambient)              lighting.py:23-147
    data   = concat(light, d) * depth_step                       renderer.py:420-437
    img    = RaymarchGridTransform(data, cameras)                renderer.py:555-568
    loss   = mean((tone(img.rgb + bkg * exp(-img.a)) - target)^2) renderer.py:626-640

The backward follows how the reference differentiates it: the raymarch and
lookup gradient ops (reference-normalised unless ``exact``) and, for both
resamplings of the shadow pass, the custom "sample gradient" of the renderer
(renderer.py:246-272): the output gradient resampled through the inverse
transform with the same mips.  ``shadow_grad='adjoint'`` uses the scatter
adjoint of the resampling instead (without mips), which makes the whole
backward the true gradient in exact mode -- used to check this composition
against finite differences.

``scene`` is a dict of plain arrays: M [1,16]; V, P [V,16]; F [V,6]; res
(D, H, W) of the camera frusta; depth_step; Vs, Ps, Fs of the light; shadow_res;
shadow_step; mips; falloff_col [D,H,W,3]; ambient; bkg [3]; order; clamp;
boundary (of the advection lookups); optionally tonemap (one of
oracle/tonemap.py MODES; NONE by default).
"""
import numpy as np

from . import advect as OA
from . import blend as B
from . import raymarch as RM
from . import resample as R
from . import sampling as S
from . import tonemap as TM
from . import transforms as T


def _shadow_resample(x, sc, out_shape, cm):
    return R.sample_grid_transform(x[None], sc['M'], sc['Vs'], sc['Ps'], sc['Fs'], out_shape, S.LINEAR, S.BORDER,
                                   S.MIP_LINEAR if sc['mips'] > 0 else S.MIP_NONE, sc['mips'], 0.0, cm)[0, 0]


def forward(sc, d_prev, vx, vy, vz, target):
    """Returns (loss, parts): parts holds every intermediate the backward uses.
    d_prev [D,H,W,1]; vx [D,H,W+1,1], vy [D,H+1,W,1], vz [D+1,H,W,1];
    target [V,H,W,3]."""
    d = OA.warp(d_prev, vx, vy, vz, 1.0, sc['order'], sc['clamp'], sc['boundary'])
    sh = _shadow_resample(d * sc['shadow_step'], sc, sc['shadow_res'], T.LINDEPTH)      # [Ds,Hs,Ws,1]
    incl = np.cumsum(sh, axis=0)                                                         # C=1 Beer-Lambert = sum
    excl = np.concatenate([np.zeros_like(incl[:1]), incl[:-1]], axis=0)                  # BORDER shift
    tr = np.exp(-excl)
    trv = _shadow_resample(tr, sc, d.shape[:3], T.LINDEPTH_REVERSE)                      # [D,H,W,1]
    fc = np.asarray(sc['falloff_col'], np.float64)
    light = d * (trv * fc + sc['ambient'])
    data = np.concatenate([light, d], axis=-1) * sc['depth_step']
    img = RM.raymarch_fwd(data[None], sc['M'], sc['V'], sc['P'], sc['F'], sc['res'], S.LINEAR, S.BORDER,
                          B.BEER_LAMBERT)[0]                                             # [V,H,W,4]
    bkg = np.asarray(sc['bkg'], np.float64)
    ea = np.exp(-img[..., 3:])
    tm = sc.get('tonemap', 'NONE')
    if tm != 'NONE':  # the renderer's tonemapping before the loss (renderer.py:528-541, :639-640)
        loss, g_img = TM.image_loss(img, target, bkg, tm)
        parts = dict(d=d, sh=sh, tr=tr, trv=trv, light=light, data=data, img=img, g_img=g_img)
        return loss, parts
    r = img[..., :3] + bkg * ea - np.asarray(target, np.float64)
    loss = float(np.mean(r * r))
    parts = dict(d=d, sh=sh, tr=tr, trv=trv, light=light, data=data, img=img, ea=ea, r=r)
    return loss, parts


def backward(sc, d_prev, vx, vy, vz, parts, exact=False, shadow_grad='inverse', inter=None):
    """Gradients of the loss w.r.t. (d_prev, vx, vy, vz).  ``inter``: optional
    dict that receives the intermediate gradients (g_img, g_data, g_trv,
    g_tr, g_sh, g_d of the advected density)."""
    p = parts
    img = p['img']
    if 'g_img' in p:
        g_img = p['g_img']
    else:
        r, ea = p['r'], p['ea']
        n = r.size
        bkg = np.asarray(sc['bkg'], np.float64)
        g_img = np.zeros_like(img)
        g_img[..., :3] = 2.0 * r / n
        g_img[..., 3] = -np.sum(2.0 * r / n * bkg, axis=-1) * ea[..., 0]
    g_data = RM.raymarch_bwd(p['data'][None], img[None], g_img[None], sc['M'], sc['V'], sc['P'], sc['F'], sc['res'],
                             S.BORDER, B.BEER_LAMBERT, exact=exact)[0]                   # [D,H,W,4]
    g_data = g_data * sc['depth_step']
    fc = np.asarray(sc['falloff_col'], np.float64)
    d, trv = p['d'], p['trv']
    g_light = g_data[..., :3]
    g_d = g_data[..., 3:] + np.sum(g_light * (trv * fc + sc['ambient']), axis=-1, keepdims=True)
    g_trv = np.sum(g_light * d * fc, axis=-1, keepdims=True)
    # tr (frustum) -> trv (volume), then d*s_sh (volume) -> sh (frustum)
    if shadow_grad == 'inverse':
        g_tr = _shadow_resample(g_trv, sc, sc['shadow_res'], T.LINDEPTH)
    else:
        g_tr = R.sample_grid_transform_grad(p['tr'][None], g_trv[None, None], sc['M'], sc['Vs'], sc['Ps'], sc['Fs'],
                                            S.BORDER, T.LINDEPTH_REVERSE, exact=True)[0]
    g_excl = -p['tr'] * g_tr
    # excl_k = sum_{j<k} sh_j  ->  g_sh_j = sum_{k>j} g_excl_k
    rev = np.cumsum(g_excl[::-1], axis=0)[::-1]
    g_sh = np.concatenate([rev[1:], np.zeros_like(rev[:1])], axis=0)
    if shadow_grad == 'inverse':
        g_dsh = _shadow_resample(g_sh, sc, d.shape[:3], T.LINDEPTH_REVERSE)
    else:
        g_dsh = R.sample_grid_transform_grad((d * sc['shadow_step'])[None], g_sh[None, None], sc['M'], sc['Vs'],
                                             sc['Ps'], sc['Fs'], S.BORDER, T.LINDEPTH, exact=True)[0]
    g_d = g_d + g_dsh * sc['shadow_step']
    if inter is not None:
        inter.update(g_img=g_img, g_data=g_data, g_trv=g_trv, g_tr=g_tr, g_sh=g_sh, g_d=g_d)
    return OA.warp_grad(d_prev, vx, vy, vz, g_d, 1.0, sc['order'], sc['clamp'], sc['boundary'], exact=exact)


def step(sc, d_prev, vx, vy, vz, target, exact=False, shadow_grad='inverse'):
    """(loss, img [V,H,W,4], (g_d_prev, g_vx, g_vy, g_vz))."""
    loss, parts = forward(sc, d_prev, vx, vy, vz, target)
    return loss, parts['img'], backward(sc, d_prev, vx, vy, vz, parts, exact, shadow_grad)


def scene_of(step):
    """The scene dict of a render + advect step object that carries the
    step's plain arrays as attributes (gft.pipeline.RenderAdvectStep: M, V,
    P, F, res, depth_step, Vs, Ps, Fs, shadow_res, shadow_step, rs.num_mips,
    falloff_col, ambient, bkg_host, order, clamp, tonemap)."""
    fc = step.falloff_col.detach().cpu().numpy()[0].astype(np.float64)
    return dict(M=np.asarray(step.M), V=np.asarray(step.V), P=np.asarray(step.P), F=np.asarray(step.F),
                res=tuple(step.res), depth_step=step.depth_step, Vs=np.asarray(step.Vs), Ps=np.asarray(step.Ps),
                Fs=np.asarray(step.Fs), shadow_res=tuple(step.shadow_res), shadow_step=step.shadow_step,
                mips=int(step.rs.num_mips), falloff_col=fc, ambient=float(step.ambient),
                bkg=np.asarray(step.bkg_host, np.float64), order=int(step.order), clamp=step.clamp,
                boundary=S.CLAMP, tonemap=getattr(step, 'tonemap', 'NONE'))
