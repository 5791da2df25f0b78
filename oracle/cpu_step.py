"""CPU baseline: the FP64 oracle port of one render + advect iteration.

TEST / CPU-BASELINE INFRASTRUCTURE ONLY (imported by bench.py's CPU legs).

The iteration is the one of gft.pipeline: MacCormack advection (MC_SMOOTH,
CLAMP), the spot-light shadow pass (volume -> light frustum resample with mips,
depth sum, transmittance, frustum -> volume resample; gradients by inverse
resampling, renderer.py:246-272), light composition, the multi-view raymarch
with reference-normalised gradients (raymarch_grid.cu.cc:319-574) and the L2
image loss with background -- forward and backward (oracle/step.py).

Two ways to time it:

* ``FullStep`` runs whole iterations over every voxel, ray and frustum cell,
  split over a pool of spawned worker processes that share their arrays
  through shared memory: advection on z-slabs with a 12-voxel halo (wider than
  the reach of the two MacCormack lookups, so each slab's result equals the
  full grid's), the resamplings on boxes of their output grids, the raymarch
  on (camera, image-row band) windows, its reference normalisation by summing
  every band's (scatter, weight-sum) partials of a camera before dividing.
  This is bench.py's reference arm.
* ``time_step`` times a bounded, evenly spaced sample of the same work (image
  rows across each view, slabs of the grid, bands of the frustum) on one core
  and scales it by work units: bench.py's ``cpu_baseline`` beside the GPU arm.
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
from oracle import blend as B  # noqa: E402
from oracle import raymarch as RM  # noqa: E402
from oracle import resample as R  # noqa: E402
from oracle import sampling as S  # noqa: E402
from oracle import transforms as T  # noqa: E402

HALO = 12


# ------------------------------------------------------------------- scene
def scene_arrays(config):
    """Plain-array scene and seeded inputs of a gft.pipeline configuration
    (the step's geometry, light, falloff and the frame-0 inputs)."""
    import torch
    from gft import synthetic as syn
    from gft.pipeline import RenderAdvectStep
    st = RenderAdvectStep(config, 'cpu')
    sc = dict(M=np.asarray(st.M), V=np.asarray(st.V), P=np.asarray(st.P), F=np.asarray(st.F), res=tuple(st.res),
              depth_step=st.depth_step, Vs=np.asarray(st.Vs), Ps=np.asarray(st.Ps), Fs=np.asarray(st.Fs),
              shadow_res=tuple(st.shadow_res), shadow_step=st.shadow_step, mips=int(st.rs.num_mips),
              ambient=float(st.ambient), bkg=np.asarray(st.bkg_host, np.float64), order=int(st.order),
              clamp=st.clamp, boundary=S.CLAMP, shape=tuple(st.shape))
    with torch.no_grad():
        fc = st.falloff_col[0].numpy().astype(np.float64)
    seed = st.cfg['seed']
    d = syn.plume_density(st.shape, seed)[0].astype(np.float64)
    vel = [v[0].astype(np.float64) for v in syn.curl_velocity(st.shape, seed + 500)]
    V, (_, H, W) = len(sc['V']), sc['res']
    target = np.random.default_rng(seed + 7).random((V, H, W, 3)) * 0.3
    return sc, fc, d, vel, target


# ------------------------------------------------------------ shared memory
_OPEN = {}


class _Spec:
    def __init__(self, name, shape, dtype='f8'):
        self.name, self.shape, self.dtype = name, tuple(shape), dtype


def _view(spec):
    from multiprocessing import shared_memory
    shm = _OPEN.get(spec.name)
    if shm is None:
        shm = shared_memory.SharedMemory(name=spec.name)
        _OPEN[spec.name] = shm
    return np.ndarray(spec.shape, dtype=spec.dtype, buffer=shm.buf)


_W = {}  # worker state: scene + array specs


def _init_worker(sc, specs):
    os.environ.setdefault('OMP_NUM_THREADS', '1')
    _W['sc'] = sc
    _W['specs'] = specs


def _a(name):
    return _view(_W['specs'][name])


def _bands(n, k):
    edges = np.linspace(0, n, k + 1).round().astype(int)
    return [(int(a), int(b)) for a, b in zip(edges[:-1], edges[1:]) if b > a]


def _crop(z0, z1, D):
    return max(0, z0 - HALO), min(D, z1 + HALO)


# ------------------------------------------------------------------ tasks
def _t_advect_fwd(z0, z1):
    sc = _W['sc']
    D = sc['shape'][0]
    c0, c1 = _crop(z0, z1, D)
    d, vx, vy, vz = _a('d_prev'), _a('vx'), _a('vy'), _a('vz')
    out = OA.warp(d[c0:c1], vx[c0:c1], vy[c0:c1], vz[c0:c1 + 1], 1.0, sc['order'], sc['clamp'], sc['boundary'])
    _a('d')[z0:z1] = out[z0 - c0:z1 - c0]


def _shadow(x, out_shape, cm, box):
    sc = _W['sc']
    return R.sample_grid_transform(x[None], sc['M'], sc['Vs'], sc['Ps'], sc['Fs'], out_shape, S.LINEAR, S.BORDER,
                                   S.MIP_LINEAR if sc['mips'] > 0 else S.MIP_NONE, sc['mips'], 0.0, cm,
                                   out_box=box)[0, 0]


def _t_resample(src, dst, to_frustum, z0, z1, scale=1.0, add=False):
    """dst[z0:z1] (+)= scale * resample(src) on that slab of the output."""
    sc = _W['sc']
    out_shape = sc['shadow_res'] if to_frustum else sc['shape']
    _, Ho, Wo = out_shape
    r = _shadow(_a(src), out_shape, T.LINDEPTH if to_frustum else T.LINDEPTH_REVERSE,
                ((z0, z1), (0, Ho), (0, Wo))) * scale
    if add:
        _a(dst)[z0:z1] += r
    else:
        _a(dst)[z0:z1] = r


def _t_compose(z0, z1):
    sc = _W['sc']
    d, trv, fc = _a('d')[z0:z1], _a('trv')[z0:z1], _a('falloff')[z0:z1]
    light = d * (trv * fc + sc['ambient'])
    _a('data')[z0:z1] = np.concatenate([light, d], axis=-1) * sc['depth_step']


def _cam(c):
    sc = _W['sc']
    return T.CameraXform(sc['M'][0], sc['V'][c], sc['P'][c], sc['F'][c])


def _t_ray_fwd(c, r0, r1):
    sc = _W['sc']
    img = RM.raymarch_fwd(_a('data')[None], sc['M'], sc['V'][c:c + 1], sc['P'][c:c + 1], sc['F'][c:c + 1], sc['res'],
                          rows=slice(r0, r1))
    _a('img')[c, r0:r1] = img[0, 0, r0:r1]


def _t_ray_bwd(c, r0, r1, slot):
    sc = _W['sc']
    buf, cnt = RM.camera_scatter(_a('data'), _a('img')[c], _a('g_img')[c], _cam(c), sc['res'],
                                 (slice(r0, r1), slice(None)), S.BORDER, B.BEER_LAMBERT, False)
    _a('p_buf')[slot] = buf
    _a('p_cnt')[slot] = cnt


def _t_ray_reduce(z0, z1, nslots):
    buf = np.sum(_a('p_buf')[:nslots, z0:z1], axis=0)
    cnt = np.sum(_a('p_cnt')[:nslots, z0:z1], axis=0)
    nz = cnt > 0
    g = _a('g_data')[z0:z1]
    g[nz] += buf[nz] / cnt[nz][:, None]


def _t_compose_bwd(z0, z1):
    sc = _W['sc']
    g = _a('g_data')[z0:z1] * sc['depth_step']
    d, trv, fc = _a('d')[z0:z1], _a('trv')[z0:z1], _a('falloff')[z0:z1]
    gl = g[..., :3]
    _a('g_d')[z0:z1] = g[..., 3:] + np.sum(gl * (trv * fc + sc['ambient']), axis=-1, keepdims=True)
    _a('g_trv')[z0:z1] = np.sum(gl * d * fc, axis=-1, keepdims=True)


def _t_advect_bwd(z0, z1):
    sc = _W['sc']
    D = sc['shape'][0]
    c0, c1 = _crop(z0, z1, D)
    d, vx, vy, vz, gy = _a('d_prev'), _a('vx'), _a('vy'), _a('vz'), _a('g_d')
    gd, gx, gyy, gz = OA.warp_grad(d[c0:c1], vx[c0:c1], vy[c0:c1], vz[c0:c1 + 1], gy[c0:c1], 1.0, sc['order'],
                                   sc['clamp'], sc['boundary'], exact=False)
    a, b = z0 - c0, z1 - c0
    _a('g_dprev')[z0:z1] = gd[a:b]
    _a('g_vx')[z0:z1] = gx[a:b]
    _a('g_vy')[z0:z1] = gyy[a:b]
    zb = b + 1 if z1 == D else b  # the last slab also owns face D
    _a('g_vz')[z0:z0 + (zb - a)] = gz[a:zb]


def _run_task(args):
    fn, a = args
    t = time.perf_counter()
    globals()[fn](*a)
    return time.perf_counter() - t


# --------------------------------------------------------------- full step
class FullStep:
    """Whole render + advect iterations of a configuration in FP64 on
    ``workers`` processes (see the module docstring)."""

    def __init__(self, config='cfg5', workers=None):
        from multiprocessing import shared_memory
        self.config = config
        self.workers = int(workers or os.cpu_count() or 1)
        sc, fc, d, vel, target = scene_arrays(config)
        self.sc = sc
        D, H, W = sc['shape']
        V, (_, Hi, Wi) = len(sc['V']), sc['res']
        Ds, Hs, Ws = sc['shadow_res']
        self.nslots = self.workers
        shapes = {
            'd_prev': (D, H, W, 1), 'vx': (D, H, W + 1, 1), 'vy': (D, H + 1, W, 1), 'vz': (D + 1, H, W, 1),
            'falloff': (D, H, W, 3), 'target': (V, Hi, Wi, 3),
            'd': (D, H, W, 1), 'xsh': (D, H, W, 1), 'sh': (Ds, Hs, Ws, 1), 'tr': (Ds, Hs, Ws, 1),
            'trv': (D, H, W, 1), 'data': (D, H, W, 4), 'img': (V, Hi, Wi, 4), 'g_img': (V, Hi, Wi, 4),
            'p_buf': (self.nslots, D, H, W, 4), 'p_cnt': (self.nslots, D, H, W), 'g_data': (D, H, W, 4),
            'g_d': (D, H, W, 1), 'g_trv': (D, H, W, 1), 'g_tr': (Ds, Hs, Ws, 1), 'g_sh': (Ds, Hs, Ws, 1),
            'g_dprev': (D, H, W, 1), 'g_vx': (D, H, W + 1, 1), 'g_vy': (D, H + 1, W, 1), 'g_vz': (D + 1, H, W, 1),
        }
        self._shm = []
        self.specs = {}
        for k, shp in shapes.items():
            n = int(np.prod(shp)) * 8
            shm = shared_memory.SharedMemory(create=True, size=max(n, 8))
            self._shm.append(shm)
            self.specs[k] = _Spec(shm.name, shp)
            _OPEN[shm.name] = shm
        for k, v in (('d_prev', d), ('vx', vel[0]), ('vy', vel[1]), ('vz', vel[2]), ('falloff', fc),
                     ('target', target)):
            self.a(k)[...] = v
        ctx = mp.get_context('spawn')
        self.pool = ctx.Pool(self.workers, initializer=_init_worker, initargs=(sc, self.specs))
        self.stage_s = {}

    def a(self, name):
        return _view(self.specs[name])

    def _map(self, stage, tasks):
        t = time.perf_counter()
        self.pool.map(_run_task, tasks, chunksize=1)
        self.stage_s[stage] = self.stage_s.get(stage, 0.0) + time.perf_counter() - t

    def step(self):
        """One forward + backward; returns (loss, seconds)."""
        sc = self.sc
        D = sc['shape'][0]
        Ds = sc['shadow_res'][0]
        V, (_, Hi, _) = len(sc['V']), sc['res']
        slabs = _bands(D, self.workers)
        fslabs = _bands(Ds, self.workers)
        rbands = _bands(Hi, self.workers)
        t0 = time.perf_counter()
        self._map('advect', [('_t_advect_fwd', s) for s in slabs])
        self.a('xsh')[...] = self.a('d') * sc['shadow_step']
        self._map('shadow', [('_t_resample', ('xsh', 'sh', True) + s) for s in fslabs])
        sh = self.a('sh')
        incl = np.cumsum(sh, axis=0)
        self.a('tr')[...] = np.exp(-np.concatenate([np.zeros_like(incl[:1]), incl[:-1]], axis=0))
        self._map('shadow', [('_t_resample', ('tr', 'trv', False) + s) for s in slabs])
        self._map('compose', [('_t_compose', s) for s in slabs])
        self._map('raymarch', [('_t_ray_fwd', (c,) + r) for c in range(V) for r in rbands])
        img, ea = self.a('img'), None
        ea = np.exp(-img[..., 3:])
        r = img[..., :3] + sc['bkg'] * ea - self.a('target')
        loss = float(np.mean(r * r))
        n = r.size
        g_img = self.a('g_img')
        g_img[..., :3] = 2.0 * r / n
        g_img[..., 3] = -np.sum(2.0 * r / n * sc['bkg'], axis=-1) * ea[..., 0]
        self.a('g_data')[...] = 0.0
        for c in range(V):
            self._map('raymarch', [('_t_ray_bwd', (c,) + rb + (k,)) for k, rb in enumerate(rbands)])
            self._map('raymarch', [('_t_ray_reduce', s + (len(rbands),)) for s in slabs])
        self._map('compose', [('_t_compose_bwd', s) for s in slabs])
        self._map('shadow', [('_t_resample', ('g_trv', 'g_tr', True) + s) for s in fslabs])
        g_excl = -self.a('tr') * self.a('g_tr')
        rev = np.cumsum(g_excl[::-1], axis=0)[::-1]
        self.a('g_sh')[...] = np.concatenate([rev[1:], np.zeros_like(rev[:1])], axis=0)
        self._map('shadow', [('_t_resample', ('g_sh', 'g_d', False) + s + (sc['shadow_step'], True))
                             for s in slabs])
        self._map('advect', [('_t_advect_bwd', s) for s in slabs])
        return loss, time.perf_counter() - t0

    def gradients(self):
        return tuple(self.a(k).copy() for k in ('g_dprev', 'g_vx', 'g_vy', 'g_vz'))

    def close(self):
        self.pool.close()
        self.pool.join()
        for shm in self._shm:
            _OPEN.pop(shm.name, None)
            shm.close()
            shm.unlink()
        self._shm = []

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()


def time_full_steps(config='cfg5', workers=None, budget_s=240.0, max_steps=20):
    """Runs whole iterations until ``budget_s`` of step time is spent (at least
    one); returns the per-step seconds and the stage breakdown."""
    with FullStep(config, workers) as fs:
        times, losses = [], []
        while len(times) < max_steps:
            loss, t = fs.step()
            times.append(t)
            losses.append(loss)
            if sum(times) + t > budget_s:
                break
        stages = {k: v / len(times) for k, v in fs.stage_s.items()}
        return {'seconds_per_step': times, 'loss': losses, 'stages_s': stages, 'workers': fs.workers}


# ------------------------------------------------------ sampled (1 core)
def _scene(config):
    sc, fc, d, vel, target = scene_arrays(config)
    return dict(sc=sc, fc=fc, d=d, vel=vel, target=target)


def time_step(step=None, inputs=None, budget_s=20.0, workers=1, config='cfg2'):
    """bench.py's ``cpu_baseline`` beside the GPU arm: one core, a bounded
    sample of the iteration -- evenly spaced image rows of every view (raymarch
    forward + backward), a z-slab of the grid (advection forward + backward)
    and a band of the light frustum plus the matching slab of the volume (the
    two shadow resamplings, each run twice for the forward and its inverse-
    resampling gradient) -- scaled to a full iteration by work units."""
    S_ = _scene(config)
    sc = S_['sc']
    D, H, W = sc['shape']
    V, (Dc, Hi, Wi) = len(sc['V']), sc['res']
    scale = max(0.05, budget_s / 20.0)
    nrows = max(1, int(2 * scale))
    rows = np.linspace(0, Hi - 1, nrows + 2).round().astype(int)[1:-1]
    d = S_['d']
    data = np.concatenate([d * 0.5] * 3 + [d], axis=-1)[None] * sc['depth_step']
    t = time.perf_counter()
    for c in range(V):
        for r in rows:
            y = RM.raymarch_fwd(data, sc['M'], sc['V'][c:c + 1], sc['P'][c:c + 1], sc['F'][c:c + 1], sc['res'],
                                rows=slice(r, r + 1))
            RM.raymarch_bwd(data, y, np.ones_like(y) * 1e-3, sc['M'], sc['V'][c:c + 1], sc['P'][c:c + 1],
                            sc['F'][c:c + 1], sc['res'], rows=slice(r, r + 1))
    t_ray = (time.perf_counter() - t) * Hi / len(rows)
    hz = max(1, int(4 * scale))
    z0 = D // 2
    c0, c1 = max(0, z0 - HALO), min(D, z0 + hz + HALO)
    vx, vy, vz = S_['vel']
    t = time.perf_counter()
    out = OA.warp(d[c0:c1], vx[c0:c1], vy[c0:c1], vz[c0:c1 + 1], 1.0, sc['order'], sc['clamp'], S.CLAMP)
    OA.warp_grad(d[c0:c1], vx[c0:c1], vy[c0:c1], vz[c0:c1 + 1], np.ones_like(out), 1.0, sc['order'], sc['clamp'],
                 S.CLAMP)
    t_adv = (time.perf_counter() - t) * D / (c1 - c0)
    Ds, Hs, Ws = sc['shadow_res']
    fz = max(1, int(4 * scale))
    vz_ = max(1, int(round(fz * D / Ds)))
    mode = S.MIP_LINEAR if sc['mips'] > 0 else S.MIP_NONE
    t = time.perf_counter()
    R.sample_grid_transform(d[None] * sc['shadow_step'], sc['M'], sc['Vs'], sc['Ps'], sc['Fs'], sc['shadow_res'],
                            S.LINEAR, S.BORDER, mode, sc['mips'], 0.0, T.LINDEPTH,
                            out_box=((Ds // 2, Ds // 2 + fz), (0, Hs), (0, Ws)))
    R.sample_grid_transform(np.ones((1, Ds, Hs, Ws, 1)), sc['M'], sc['Vs'], sc['Ps'], sc['Fs'], sc['shape'],
                            S.LINEAR, S.BORDER, mode, sc['mips'], 0.0, T.LINDEPTH_REVERSE,
                            out_box=((D // 2, D // 2 + vz_), (0, H), (0, W)))
    t_sh = (time.perf_counter() - t) * 2.0 * Ds / fz  # forward + inverse-resampling gradient
    total = t_ray + t_adv + t_sh
    return {'value': 1.0 / total, 'unit': 'iters/s', 'cores': int(workers), 'kind': 'port',
            'sample': ('FP64 NumPy port of the reference ops on one core: %d evenly spaced image rows of each of '
                       'the %d views (raymarch fwd+bwd), a %d-slice z-slab of the grid with its halo (MacCormack '
                       'fwd+bwd) and a %d-slice band of the %dx%dx%d light frustum (both shadow resamplings), '
                       'scaled by work units to a full iteration: raymarch %.0f s, advect %.0f s, shadow %.0f s'
                       % (len(rows), V, hz, fz, Ds, Hs, Ws, t_ray, t_adv, t_sh)),
            'seconds_per_step': total}
