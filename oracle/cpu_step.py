"""CPU baseline: the FP64 oracle port of one render + advect step, timed on a
bounded sample of the workload and extrapolated to a full step.

TEST / CPU-BASELINE INFRASTRUCTURE ONLY (imported by bench.py's CPU legs).

The step is the one of gft.pipeline (cfg2): MacCormack advection fwd+bwd, the
spot-light shadow pass (light-frustum resample with mips, cumulative sum,
inverse resample; its gradient is the same two resamples in the other
direction, renderer.py:246-272), and the 5-view raymarch fwd+bwd.  Each part
is timed on a sample (image rows, grid slabs, frustum rows) and scaled by the
ratio of full to sampled work units; elementwise glue is not counted.  With
``workers`` > 1 the samples run in that many spawned processes at once and the
throughput of all of them is used.
"""
import multiprocessing as mp
import os
import sys
import time

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_ROOT = os.path.dirname(_HERE)
for _p in (_ROOT, os.path.join(_ROOT, 'global-flow-transport_gb300')):
    if _p not in sys.path:
        sys.path.insert(0, _p)

from oracle import advect as OA  # noqa: E402
from oracle import raymarch as RM  # noqa: E402
from oracle import resample as R  # noqa: E402
from oracle import sampling as S  # noqa: E402
from oracle import transforms as T  # noqa: E402


def _scene(config):
    from gft import synthetic as syn
    from gft.pipeline import CONFIGS
    from phitest.render.lighting import SpotLight
    from phitest.render.transform import Transform
    cfg = CONFIGS[config]
    D, H, W = cfg['grid']
    Hi, Wi = cfg['image']
    res = (cfg['samples'], Hi, Wi)
    gt = syn.grid_transform((D, H, W))
    cams = syn.arc_cameras(cfg['views'], res, radius=2.5, fov=30.0)
    M = syn.model_matrix(gt)
    V, P, F = syn.camera_params(cams)
    spot = SpotLight(Transform(translation=[0, 0, 2.0], parent=Transform(rotation_deg=[-40, 0, 0])), intensity=0.85,
                     cast_shadows=True, shadow_clip=[0.85, 3.15], range_scale=0.825, angle_deg=60.0,
                     shadow_resolution=list(cfg['shadow']), cone_mask=False)
    Vs, Ps, Fs = syn.camera_params([spot.shadow_cam])
    d = syn.plume_density((D, H, W), cfg['seed'])
    vx, vy, vz = syn.curl_velocity((D, H, W), cfg['seed'] + 500)
    return dict(cfg=cfg, shape=(D, H, W), res=res, M=M, V=V, P=P, F=F, Vs=Vs, Ps=Ps, Fs=Fs, d=d,
                v=(vx[0], vy[0], vz[0]), depth_step=float(cams[0].depth_step))


def _raymarch_rows(sc, rows):
    """fwd + bwd of one camera over ``rows`` image rows; returns rays done."""
    x = np.concatenate([sc['d'] * 0.5] * 3 + [sc['d']], axis=-1) * sc['depth_step']
    r = slice(0, rows)
    y = RM.raymarch_fwd(x, sc['M'], sc['V'][:1], sc['P'][:1], sc['F'][:1], sc['res'], rows=r)
    dy = np.ones_like(y) * 1e-3
    RM.raymarch_bwd(x, y, dy, sc['M'], sc['V'][:1], sc['P'][:1], sc['F'][:1], sc['res'], rows=r)
    return rows * sc['res'][2]


def _advect_slab(sc, height):
    d = sc['d'][0][:, :height]
    vx, vy, vz = sc['v']
    vx, vy, vz = vx[:, :height], vy[:, :height + 1], vz[:, :height]
    out = OA.warp(d, vx, vy, vz, 1.0, 2, 'MC_SMOOTH', S.CLAMP)
    OA.warp_grad(d, vx, vy, vz, np.ones_like(out), 1.0, 2, 'MC_SMOOTH', S.CLAMP)
    return d.shape[0] * d.shape[1] * d.shape[2]


def _shadow_rows(sc, rows):
    """Light-frustum resample (LINDEPTH, mips) of ``rows`` frustum rows and the
    inverse resample (LINDEPTH_REVERSE, mips) of the same fraction of the volume;
    returns the fraction of one full pass done."""
    Ds, Hs, Ws = sc['cfg']['shadow']
    mips = sc['cfg']['mips']
    R.sample_grid_transform(sc['d'], sc['M'], sc['Vs'], sc['Ps'], sc['Fs'], (Ds, rows, Ws), S.LINEAR, S.BORDER,
                            S.MIP_LINEAR, mips, 0.0, T.LINDEPTH)
    D, H, W = sc['shape']
    frac = rows / float(Hs)
    vrows = max(1, int(round(H * frac)))
    tr = np.ones((1, Ds, Hs, Ws, 1))
    R.sample_grid_transform(tr, sc['M'], sc['Vs'], sc['Ps'], sc['Fs'], (D, vrows, W), S.LINEAR, S.BORDER,
                            S.MIP_LINEAR, mips, 0.0, T.LINDEPTH_REVERSE)
    return frac


def _worker(args):
    config, part, size = args
    sc = _scene(config)
    t = time.perf_counter()
    if part == 'raymarch':
        units = _raymarch_rows(sc, size)
    elif part == 'advect':
        units = _advect_slab(sc, size)
    else:
        units = _shadow_rows(sc, size)
    return units, time.perf_counter() - t


def _run(config, part, size, workers):
    if workers <= 1:
        units, t = _worker((config, part, size))
        return units / t
    ctx = mp.get_context('spawn')
    with ctx.Pool(workers) as pool:
        t0 = time.perf_counter()
        res = pool.map(_worker, [(config, part, size)] * workers)
        wall = time.perf_counter() - t0
    # per-worker compute time excludes the scene set-up inside each worker
    return sum(u for u, _ in res) / max(t for _, t in res) if wall > 0 else 0.0


def time_step(step=None, inputs=None, budget_s=20.0, workers=1, config='cfg2'):
    """Returns the bench.py ``cpu_baseline`` object: full-step throughput in
    iters/s extrapolated from sampled rates of each part."""
    sc = _scene(config)
    V = sc['cfg']['views']
    D, Hi, Wi = sc['res']
    nvox = int(np.prod(sc['shape']))
    # sample sizes chosen so the whole measurement takes roughly budget_s
    scale = max(0.05, budget_s / 20.0)
    ray_rows = max(4, int(32 * scale))
    adv_h = max(4, int(16 * scale))
    sh_rows = max(2, int(8 * scale))
    ray_rate = _run(config, 'raymarch', ray_rows, workers)      # rays / s (fwd+bwd)
    adv_rate = _run(config, 'advect', adv_h, workers)           # voxels / s (fwd+bwd)
    sh_rate = _run(config, 'shadow', sh_rows, workers)          # shadow passes / s (one direction)
    t_ray = V * Hi * Wi / ray_rate
    t_adv = nvox / adv_rate
    t_sh = 2.0 / sh_rate  # forward pass and the inverse-resampling gradient
    total = t_ray + t_adv + t_sh
    return {'value': 1.0 / total, 'unit': 'iters/s', 'cores': int(workers), 'kind': 'port',
            'sample': ('FP64 NumPy port of the reference ops; sampled %d image rows of one view (x%d views), '
                       'a %d-row slab of the advection grid and %d of %d shadow-frustum rows per worker, '
                       'extrapolated by work units: raymarch %.1f s, advect %.1f s, shadow %.1f s per step'
                       % (ray_rows, V, adv_h, sh_rows, sc['cfg']['shadow'][1], t_ray, t_adv, t_sh)),
            'seconds_per_step': total}
