"""Deterministic gradient mode (GFT_GRAD_DETERMINISTIC, gft.ops.deterministic):
the raymarch and advection adjoints accumulate fixed-point int64 sums, so
repeated backward passes give bit-identical gradients, which agree with the
FP64 oracle as closely as the float path does.  The captured render + advect
step (whose other gradients are gathers and scans) is then bit-reproducible
from replay to replay."""
import numpy as np
import pytest
import torch

from scene_utils import rel_l2, scene, small_grid

pytestmark = pytest.mark.gpu

GRAD_TOL = 1e-4   # vs the FP64 oracle, as for the float path
FLOAT_TOL = 1e-5  # vs the float path: summation order and the fixed-point rounding
RUNS = 3
BOUNDS = ['BORDER', 'CLAMP', 'WRAP']


@pytest.fixture(scope='module')
def ops():
    if not torch.cuda.is_available():
        pytest.skip('no CUDA device')
    from gft import ops as _ops
    return _ops


def cuda(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def np_(t):
    return t.detach().cpu().numpy().astype(np.float64)


def _runs(fn, det=True):
    from gft import ops
    out = []
    for _ in range(RUNS):
        with ops.deterministic(det):
            out.append([g.detach().clone() for g in fn()])
    return out


def _all_equal(runs):
    return all(torch.equal(a, b) for r in runs[1:] for a, b in zip(runs[0], r))


# ------------------------------------------------------------------ raymarch
@pytest.mark.parametrize('boundary', ['BORDER', 'CLAMP'])
def test_raymarch_deterministic_weights_ahead(ops, boundary):
    """The deterministic adjoint's integer weight sums computed ahead on the
    side stream during the forward (gft_raymarch_grid_transform_grad_weights_mode
    + GFT_GRAD_WEIGHTS_READY) give the very gradient, bit for bit, of the
    gradient call that sums them itself."""
    _, _, M, V, P, F = scene((10, 14, 12), 3, (13, 9, 11))
    x = small_grid((10, 14, 12), 4, 61) * 0.4
    dy = cuda(np.random.default_rng(62).standard_normal((1, 3, 9, 11, 4)).astype(np.float32))
    ops.set_raymarch_sample_store(False)  # both re-sample: the same samples
    try:
        with ops.deterministic(True), ops.grad_mode('REFERENCE'):
            xt = cuda(x).requires_grad_(True)
            y = ops.raymarch_grid_transform(xt, M, V, P, F, (13, 9, 11), 'LINEAR', boundary)
            y.backward(dy)
            g_inline = ops.raymarch_grid_transform_grad(cuda(x), y.detach(), dy, M, V, P, F, (13, 9, 11),
                                                        'LINEAR', boundary)
    finally:
        ops.set_raymarch_sample_store(True)
    assert np.abs(np_(g_inline)).max() > 0
    assert torch.equal(xt.grad, g_inline)


@pytest.mark.parametrize('C', [1, 4])
@pytest.mark.parametrize('blend', ['BEER_LAMBERT', 'ADDITIVE'])
@pytest.mark.parametrize('boundary', ['BORDER', 'CLAMP'])
@pytest.mark.parametrize('mode', ['REFERENCE', 'EXACT'])
@pytest.mark.parametrize('store', [False, True])
def test_raymarch_deterministic(ops, C, blend, boundary, mode, store):
    from oracle import blend as OB
    from oracle import raymarch as RM
    _, _, M, V, P, F = scene((10, 14, 12), 3, (13, 9, 11))
    x = small_grid((10, 14, 12), C, 113) * 0.4
    dy = cuda(np.random.default_rng(114).standard_normal((1, 3, 9, 11, C)).astype(np.float32))

    def grad():
        xt = cuda(x).requires_grad_(True)
        with ops.grad_mode(mode):
            y = ops.raymarch_grid_transform(xt, M, V, P, F, (13, 9, 11), 'LINEAR', boundary, blend)
            y.backward(dy)
        grad.y = y
        return [xt.grad]

    ops.set_raymarch_sample_store(store)
    try:
        det = _runs(grad)
        flt = _runs(grad, det=False)
    finally:
        ops.set_raymarch_sample_store(True)
    assert _all_equal(det)
    ref = RM.raymarch_bwd(x, np_(grad.y), np_(dy), M, V, P, F, (13, 9, 11), BOUNDS.index(boundary),
                          getattr(OB, blend), exact=(mode == 'EXACT'))
    assert rel_l2(np_(det[0][0]), ref) <= GRAD_TOL
    assert rel_l2(np_(det[0][0]), np_(flt[0][0])) <= FLOAT_TOL


@pytest.mark.parametrize('C', [1, 2])
@pytest.mark.parametrize('blend', ['ALPHA', 'ALPHA_ADDITIVE'])
def test_raymarch_deterministic_single_channel_any_blend(ops, C, blend):
    """Any blending with one channel; the front-to-back modes with several
    channels are refused (their adjoint carries no bound of the kind the
    fixed-point scale needs)."""
    from gft import _lib
    from oracle import blend as OB
    from oracle import raymarch as RM
    _, _, M, V, P, F = scene((10, 14, 12), 2, (13, 9, 11))
    x = small_grid((10, 14, 12), C, 115) * 0.4
    dy = cuda(np.random.default_rng(116).standard_normal((1, 2, 9, 11, C)).astype(np.float32))

    def grad():
        xt = cuda(x).requires_grad_(True)
        y = ops.raymarch_grid_transform(xt, M, V, P, F, (13, 9, 11), 'LINEAR', 'BORDER', blend)
        y.backward(dy)
        grad.y = y
        return [xt.grad]

    if C > 1:
        with pytest.raises(_lib.GftUnimplemented):
            _runs(grad)
        return
    det = _runs(grad)
    assert _all_equal(det)
    ref = RM.raymarch_bwd(x, np_(grad.y), np_(dy), M, V, P, F, (13, 9, 11), 0, getattr(OB, blend))
    assert rel_l2(np_(det[0][0]), ref) <= GRAD_TOL


@pytest.mark.parametrize('mode', ['REFERENCE', 'EXACT'])
def test_raymarch_bricked_and_views_deterministic(ops, mode):
    """The brick-layout op and the views op (batch slices with their own
    cameras, two launch tables)."""
    from test_gpu_parity import _views_scene
    _, _, M, V, P, F = scene((9, 13, 11), 3, (13, 9, 11))
    x = small_grid((9, 13, 11), 4, 117) * 0.4
    dy = cuda(np.random.default_rng(118).standard_normal((1, 3, 9, 11, 4)).astype(np.float32))

    def bricked():
        xb = ops.to_bricks(cuda(x)).requires_grad_(True)
        with ops.grad_mode(mode):
            ops.raymarch_grid_transform_bricked(xb, (9, 13, 11), M, V, P, F, (13, 9, 11), 'BORDER').backward(dy)
        return [xb.grad]

    det = _runs(bricked)
    assert _all_equal(det)
    assert rel_l2(np_(det[0][0]), np_(_runs(bricked, det=False)[0][0])) <= FLOAT_TOL

    xv, Mv, Vv, Pv, Fv, cb, shapes = _views_scene(4, 119)
    rng = np.random.default_rng(120)
    w = torch.cat([cuda(rng.standard_normal((h * wd, 4)).astype(np.float32)) for _, h, wd in shapes])

    def views():
        xt = cuda(xv).requires_grad_(True)
        with ops.grad_mode(mode):
            (ops.raymarch_grid_transform_views(xt, cb, Mv, Vv, Pv, Fv, shapes) * w).sum().backward()
        return [xt.grad]

    det = _runs(views)
    assert _all_equal(det)
    assert rel_l2(np_(det[0][0]), np_(_runs(views, det=False)[0][0])) <= FLOAT_TOL


def test_raymarch_deterministic_large_sums(ops):
    """Many rays per voxel (a 128 x 128 image of a 16^3 grid, 96 samples) and a
    wide range of output gradients: the bound-derived fixed-point scale keeps
    the small gradients as accurate as the float path."""
    from gft import synthetic as syn
    from oracle import raymarch as RM
    shape, res = (16, 16, 16), (96, 128, 128)
    _, _, M, V, P, F = scene(shape, 2, res)
    x = syn.plume_density(shape, 121)
    rng = np.random.default_rng(122)
    dy = (rng.standard_normal((1, 2, 128, 128, 1)) * np.exp(rng.uniform(-8, 8, (1, 2, 128, 128, 1)))).astype(
        np.float32)

    def grad():
        xt = cuda(x).requires_grad_(True)
        y = ops.raymarch_grid_transform(xt, M, V, P, F, res)
        y.backward(cuda(dy))
        grad.y = y
        return [xt.grad]

    det = _runs(grad)
    assert _all_equal(det)
    ref = RM.raymarch_bwd(x, np_(grad.y), dy, M, V, P, F, res)
    e_det = rel_l2(np_(det[0][0]), ref)
    e_flt = rel_l2(np_(_runs(grad, det=False)[0][0]), ref)
    assert e_det <= max(2.0 * e_flt, 1e-6)


def test_raymarch_deterministic_nonfinite_gives_nan(ops):
    _, _, M, V, P, F = scene((10, 14, 12), 2, (13, 9, 11))
    x = small_grid((10, 14, 12), 1, 123) * 0.4
    dy = np.random.default_rng(124).standard_normal((1, 2, 9, 11, 1)).astype(np.float32)
    dy[0, 1, 4, 5, 0] = np.inf
    xt = cuda(x).requires_grad_(True)
    with ops.deterministic():
        ops.raymarch_grid_transform(xt, M, V, P, F, (13, 9, 11)).backward(cuda(dy))
    assert torch.isnan(xt.grad).any()


# ------------------------------------------------------------------ advection
@pytest.mark.parametrize('order,clamp', [(1, 'NONE'), (1, 'NEGATIVE'), (2, 'NONE'), (2, 'MC_SMOOTH')])
@pytest.mark.parametrize('boundary', BOUNDS)
@pytest.mark.parametrize('mode', ['REFERENCE', 'EXACT'])
@pytest.mark.parametrize('C', [1, 4])
def test_advect_deterministic(ops, order, clamp, boundary, mode, C):
    """Two density slices sharing the velocity (rows of 45 voxels across
    warps, a partial last block)."""
    from oracle import advect as OA
    D, H, W = 5, 6, 45
    rng = np.random.default_rng(130 + C)
    pos = clamp != 'NEGATIVE'
    d = np.stack([small_grid((D, H, W), C, 131, positive=pos)[0], small_grid((D, H, W), C, 132, positive=pos)[0]])
    vx = (rng.standard_normal((1, D, H, W + 1, 1)) * 0.8).astype(np.float32)
    vy = (rng.standard_normal((1, D, H + 1, W, 1)) * 0.8).astype(np.float32)
    vz = (rng.standard_normal((1, D + 1, H, W, 1)) * 0.8).astype(np.float32)
    go = rng.standard_normal(d.shape).astype(np.float32)
    bi = BOUNDS.index(boundary)

    def grad():
        dtn = cuda(d).requires_grad_(True)
        vs = [cuda(v).requires_grad_(True) for v in (vx, vy, vz)]
        with ops.grad_mode(mode):
            ops.advect(dtn, *vs, dt=1.3, order=order, clamp=clamp, boundary=boundary).backward(cuda(go))
        return [dtn.grad] + [v.grad for v in vs]

    det = _runs(grad)
    assert _all_equal(det)
    flt = _runs(grad, det=False)[0]
    for a, b in zip(det[0], flt):
        assert rel_l2(np_(a), np_(b)) <= FLOAT_TOL
    gv_want = [np.zeros(v.shape[1:]) for v in (vx, vy, vz)]
    for n in range(2):
        gd, *gv = OA.warp_grad(d[n], vx[0], vy[0], vz[0], go[n], 1.3, order, clamp, bi, exact=(mode == 'EXACT'))
        assert rel_l2(np_(det[0][0])[n], gd) <= GRAD_TOL
        for acc, g in zip(gv_want, gv):
            acc += g
    for got, want in zip(det[0][1:], gv_want):
        assert rel_l2(np_(got)[0], want) <= GRAD_TOL


def test_advect_deterministic_reuses_forward_intermediate(ops):
    """The deterministic MacCormack adjoint reading the forward's
    semi-Lagrangian grid from a deterministic-size workspace
    (GFT_GRAD_FORWARD_READY) equals the one recomputing it, bit for bit, as
    does the autograd op (which reads it, or recomputes it when the mode is
    switched on between forward and backward)."""
    from gft import synthetic as syn
    shape = (10, 12, 9)
    d = cuda(syn.plume_density(shape, 133))
    vx, vy, vz = (cuda(v) for v in syn.curl_velocity(shape, 134))
    dy = cuda(np.random.default_rng(135).standard_normal((1,) + shape + (1,)).astype(np.float32))
    ref = ops._advect_bwd(d, vx, vy, vz, dy, 1.0, 2, ops.CLAMP['MC_SMOOTH'], ops.BOUNDARY['CLAMP'],
                          ops.GRAD['REFERENCE'] | ops.DETERMINISTIC)
    gm = ops.GRAD['REFERENCE'] | ops.DETERMINISTIC
    ws = ops._advect_grad_workspace(d.shape, 2, d.device, gm)
    ops._advect_fwd(d, vx, vy, vz, 1.0, 2, ops.CLAMP['MC_SMOOTH'], ops.BOUNDARY['CLAMP'], ws=ws)
    ready = ops._advect_bwd(d, vx, vy, vz, dy, 1.0, 2, ops.CLAMP['MC_SMOOTH'], ops.BOUNDARY['CLAMP'],
                            gm | ops.FORWARD_READY, ws=ws)
    for a, b in zip(ready, ref):
        assert torch.equal(a, b)
    for switch_late in (False, True):
        ts = [t.clone().requires_grad_(True) for t in (d, vx, vy, vz)]
        with ops.deterministic(not switch_late):
            y = ops.advect(*ts, dt=1.0, order=2, clamp='MC_SMOOTH', boundary='CLAMP')
        with ops.deterministic():
            y.backward(dy)
        for t, r in zip(ts, ref):
            assert torch.equal(t.grad.reshape(-1), r.reshape(-1))


def test_advect_deterministic_large_grid(ops):
    """A 96^3 plume: bit-identical runs, agreement with the float path."""
    from gft import synthetic as syn
    shape = (96, 96, 96)
    d = syn.plume_density_device(shape, 136, torch.device('cuda'))
    vx, vy, vz = syn.curl_velocity_device(shape, 137, torch.device('cuda'))
    dy = torch.randn((1,) + shape + (1,), device='cuda', generator=torch.Generator('cuda').manual_seed(138))

    def grad():
        ts = [t.clone().requires_grad_(True) for t in (d, vx, vy, vz)]
        ops.advect(*ts, dt=1.0, order=2, clamp='MC_SMOOTH', boundary='CLAMP').backward(dy)
        return [t.grad for t in ts]

    det = _runs(grad)
    assert _all_equal(det)
    for a, b in zip(det[0], _runs(grad, det=False)[0]):
        assert rel_l2(np_(a), np_(b)) <= FLOAT_TOL


# ------------------------------------------------------------------ the captured step
@pytest.mark.parametrize('storage', [torch.float32, torch.bfloat16])
def test_captured_step_bit_reproducible(ops, storage):
    from gft.pipeline import RenderAdvectStep
    with ops.deterministic():
        s = RenderAdvectStep('tiny', torch.device('cuda', 0), storage_dtype=storage)
        s.setup_static(s.make_inputs())
        s.capture(warmup=3)
        runs = []
        for _ in range(RUNS):
            loss, grads = s.replay()
            torch.cuda.synchronize()
            runs.append([loss.clone()] + [g.clone() for g in grads])
        # the same step run eagerly (outside the graph) gives the same bits
        loss_e, grads_e = s.step(s.s_d, s.s_vx, s.s_vy, s.s_vz, s.s_t)
        torch.cuda.synchronize()
    assert _all_equal(runs)
    assert torch.equal(runs[0][0], loss_e.detach())
    for a, b in zip(runs[0][1:], grads_e):
        assert torch.equal(a, b)
