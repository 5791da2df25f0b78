"""CPU checks of the FP64 oracle itself: exact adjoints against central finite
differences, reference-mode gradient structure, and small known answers."""
import numpy as np
import pytest

from scene_utils import scene, small_grid

from oracle import advect as OA
from oracle import blend as OB
from oracle import raymarch as RM
from oracle import resample as R
from oracle import sampling as S
from oracle import transforms as T

EPS = 1e-6


def _fd(f, x, d):
    return (f(x + EPS * d) - f(x - EPS * d)) / (2 * EPS)


@pytest.mark.parametrize('boundary', [S.BORDER, S.CLAMP, S.WRAP])
@pytest.mark.parametrize('blend', [OB.BEER_LAMBERT, OB.ALPHA, OB.ALPHA_ADDITIVE, OB.ADDITIVE])
def test_raymarch_exact_adjoint_fd(boundary, blend):
    _, _, M, V, P, F = scene((8, 10, 9), 2, (9, 6, 7))
    rng = np.random.default_rng(1)
    x = small_grid((8, 10, 9), 4, 2) * 0.3
    y = RM.raymarch_fwd(x, M, V, P, F, (9, 6, 7), boundary=boundary, blend_mode=blend)
    dy = rng.standard_normal(y.shape)
    g = RM.raymarch_bwd(x, y, dy, M, V, P, F, (9, 6, 7), boundary=boundary, blend_mode=blend, exact=True)
    d = rng.standard_normal(x.shape)
    fd = _fd(lambda z: np.sum(RM.raymarch_fwd(z, M, V, P, F, (9, 6, 7), boundary=boundary, blend_mode=blend) * dy), x, d)
    assert abs(fd - np.sum(g * d)) <= 1e-6 * max(1.0, abs(fd))


def test_raymarch_reference_normalisation_is_per_camera_weight_mean():
    """With a constant cell gradient the reference-mode result per voxel is the
    per-camera weighted mean, so for ADDITIVE blending and dy = 1 every reached
    voxel gets exactly (number of cameras reaching it)."""
    _, _, M, V, P, F = scene((8, 10, 9), 2, (9, 6, 7))
    x = small_grid((8, 10, 9), 1, 3)
    y = RM.raymarch_fwd(x, M, V, P, F, (9, 6, 7), boundary=S.CLAMP, blend_mode=OB.ADDITIVE)
    g = RM.raymarch_bwd(x, y, np.ones_like(y), M, V, P, F, (9, 6, 7), boundary=S.CLAMP, blend_mode=OB.ADDITIVE)
    vals = np.unique(np.round(g, 9))
    assert set(vals.tolist()) <= {0.0, 1.0, 2.0}


@pytest.mark.parametrize('boundary', [S.BORDER, S.CLAMP, S.WRAP])
def test_lut_exact_adjoint_fd(boundary):
    rng = np.random.default_rng(4)
    x = small_grid((7, 8, 6), 2, 5)
    lut = np.concatenate([rng.standard_normal((1, 7, 8, 6, 3)) * 1.4, np.zeros((1, 7, 8, 6, 1))], -1)
    dy = rng.standard_normal((1, 1, 7, 8, 6, 2))
    gx, gl = R.sample_grid_lut_grad(x, dy, lut, boundary=boundary, exact=True)
    f = lambda xx, ll: np.sum(R.sample_grid_lut(xx, ll, boundary=boundary) * dy)
    d = rng.standard_normal(x.shape)
    assert np.isclose(_fd(lambda z: f(z, lut), x, d), np.sum(gx * d), rtol=1e-6, atol=1e-8)
    dl = rng.standard_normal(lut.shape)
    dl[..., 3] = 0
    assert np.isclose(_fd(lambda z: f(x, z), lut, dl), np.sum(gl * dl), rtol=1e-5, atol=1e-7)


@pytest.mark.parametrize('order,clamp', [(1, 'NONE'), (2, 'NONE'), (2, 'MC_SMOOTH'), (1, 'NEGATIVE')])
def test_advect_exact_adjoint_fd(order, clamp):
    rng = np.random.default_rng(6)
    D, H, W = 7, 8, 6
    d = small_grid((D, H, W), 1, 7)[0]
    vx = rng.standard_normal((D, H, W + 1, 1)) * 0.7
    vy = rng.standard_normal((D, H + 1, W, 1)) * 0.7
    vz = rng.standard_normal((D + 1, H, W, 1)) * 0.7
    go = rng.standard_normal(d.shape)
    gd, gx, gy, gz = OA.warp_grad(d, vx, vy, vz, go, 1.1, order, clamp, S.CLAMP, exact=True)
    f = lambda dd, a, b, c: np.sum(OA.warp(dd, a, b, c, 1.1, order, clamp, S.CLAMP) * go)
    dd = rng.standard_normal(d.shape)
    assert np.isclose(_fd(lambda z: f(z, vx, vy, vz), d, dd), np.sum(gd * dd), rtol=1e-6, atol=1e-8)
    ex = rng.standard_normal(vx.shape)
    assert np.isclose(_fd(lambda z: f(d, z, vy, vz), vx, ex), np.sum(gx * ex), rtol=1e-5, atol=1e-7)


@pytest.mark.parametrize('blend', [OB.BEER_LAMBERT, OB.ALPHA, OB.ADDITIVE])
@pytest.mark.parametrize('keep', [False, True])
def test_blend_exact_adjoint_fd(blend, keep):
    rng = np.random.default_rng(8)
    x = rng.random((1, 9, 4, 3, 4)) * 0.3
    y = OB.reduce_grid_blend(x, blend, keep)
    dy = rng.standard_normal(y.shape)
    g = OB.reduce_grid_blend_grad(dy, y, x, blend, keep, exact=True)
    d = rng.standard_normal(x.shape)
    fd = _fd(lambda z: np.sum(OB.reduce_grid_blend(z, blend, keep) * dy), x, d)
    assert np.isclose(fd, np.sum(g * d), rtol=1e-6, atol=1e-9)


def test_beer_lambert_matches_closed_form():
    """renderer._blend_grid's closed form: L = sum l_i exp(-cumsum(s)_i), d = sum s."""
    rng = np.random.default_rng(9)
    x = rng.random((1, 12, 3, 2, 4)) * 0.2
    y = OB.reduce_grid_blend(x, OB.BEER_LAMBERT, False)
    cs = np.cumsum(x[..., 3:], axis=1)
    L = np.sum(x[..., :3] * np.exp(-cs), axis=1)
    assert np.allclose(y[..., :3], L) and np.allclose(y[..., 3:], cs[:, -1])


def test_sampling_known_answers():
    g = np.arange(2 * 3 * 4, dtype=np.float64).reshape(2, 3, 4, 1)  # value = 12 z + 4 y + x
    p = np.array([[1.25, 0.5, 0.75]])
    assert np.isclose(S.fetch_linear(g, p, S.CLAMP)[0, 0], 12 * 0.75 + 4 * 0.5 + 1.25)
    # BORDER: half a cell outside -> 0, inside the half cell -> interpolated with a zero corner
    assert S.fetch_linear(g, np.array([[-0.6, 0.0, 0.0]]), S.BORDER)[0, 0] == 0.0
    assert np.isclose(S.fetch_linear(g, np.array([[-0.25, 0.0, 0.0]]), S.BORDER)[0, 0], 0.0)
    assert np.isclose(S.fetch_linear(g, np.array([[3.25, 0.0, 0.0]]), S.BORDER)[0, 0], 3 * 0.75)
    # NEAREST truncates pos + 0.5 toward zero
    assert S.fetch_nearest(g, np.array([[-0.7, 0.0, 0.0]]), S.BORDER)[0, 0] == 0.0
    assert S.fetch_nearest(g, np.array([[1.49, 1.6, 0.2]]), S.CLAMP)[0, 0] == 4 * 2 + 1
    # WRAP
    assert np.isclose(S.fetch_linear(g, np.array([[-1.0, 0.0, 0.0]]), S.WRAP)[0, 0], 3.0)
    # mips: 2x2x2 means
    m = S.build_mips(np.ones((4, 6, 8, 1)), 3)
    assert [l.shape for l in m] == [(4, 6, 8, 1), (2, 3, 4, 1), (1, 1, 2, 1), (0, 0, 1, 1)]
    assert S.usable_mip_levels((4, 6, 8), 3) == 2


def test_lindepth_round_trip():
    _, cams, M, V, P, F = scene((10, 12, 8), 1, (16, 9, 11))
    cam = T.CameraXform(M[0], V[0], P[0], F[0])
    rng = np.random.default_rng(10)
    idx = rng.random((50, 3)) * [11, 9, 16]
    os_ = T.idx_to_os_lindepth(cam, idx, np.array([11, 9, 16.0]))
    back = T.os_to_idx_lindepth(cam, os_, np.array([11, 9, 16.0]))
    assert np.allclose(back, idx, atol=1e-9)
    back2 = T.os_to_idx(cam, T.idx_to_os(cam, idx, np.array([11, 9, 16.0])), np.array([11, 9, 16.0]))
    assert np.allclose(back2, idx, atol=1e-9)


@pytest.mark.parametrize('order', [1, 2])
def test_step_oracle_gradient_fd(order):
    """The FP64 step oracle (oracle/step.py) with exact op adjoints and the
    scatter adjoint for the shadow resamplings (no mips) is the true gradient
    of its forward: directional derivatives against central differences for
    the previous density and all three velocity components.  The density is
    positive everywhere and noisy, so no Beer-Lambert max(., 0) kink sits at
    the evaluation point; MacCormack runs without the MC_SMOOTH clamp, whose
    selection ties (lookups clamped to one edge cell) make central differences
    jump -- its adjoint is checked on random data by
    test_advect_exact_adjoint_fd."""
    from gft import synthetic as syn
    from gft.pipeline import RenderAdvectStep
    from oracle import step as OS
    from scene_utils import step_scene
    st = RenderAdvectStep('tiny', 'cpu', order=order)
    sc = step_scene(st)
    sc['mips'] = 0
    sc['clamp'] = 'NONE'
    rng = np.random.default_rng(11 + order)
    d = syn.plume_density(st.shape, 7)[0].astype(np.float64) * 8 + 0.05 + 0.01 * rng.random(st.shape + (1,))
    vel = [v[0].astype(np.float64) for v in syn.curl_velocity(st.shape, 8)]
    tgt = rng.random((len(st.cams), st.res[1], st.res[2], 3)) * 0.3
    _, _, grads = OS.step(sc, d, *vel, tgt, exact=True, shadow_grad='adjoint')
    xs = [d] + vel
    for k in range(4):
        u = rng.standard_normal(xs[k].shape)

        def loss(e):
            a = [x.copy() for x in xs]
            a[k] = a[k] + e * u
            return OS.forward(sc, *a, tgt)[0]
        fd = (loss(EPS) - loss(-EPS)) / (2 * EPS)
        assert abs(fd - np.sum(grads[k] * u)) <= 1e-4 * abs(fd), (k, fd, np.sum(grads[k] * u))


def test_step_oracle_forward_is_the_render_composition():
    """The step oracle's image equals the oracle render composition
    (shadow_transmission + render_fused) applied to the advected density."""
    from gft import synthetic as syn
    from gft.pipeline import RenderAdvectStep
    from oracle import render as ORd
    from oracle import step as OS
    from scene_utils import step_scene
    st = RenderAdvectStep('tiny', 'cpu')
    sc = step_scene(st)
    d = syn.plume_density(st.shape, 3)[0].astype(np.float64) * 8
    vel = [v[0].astype(np.float64) for v in syn.curl_velocity(st.shape, 4)]
    tgt = np.zeros((len(st.cams), st.res[1], st.res[2], 3))
    _, parts = OS.forward(sc, d, *vel, tgt)
    da = OA.warp(d, *vel, 1.0, 2, 'MC_SMOOTH', S.CLAMP)
    trv = ORd.shadow_transmission(da[None], sc['M'], sc['Vs'], sc['Ps'], sc['Fs'], sc['shadow_res'],
                                  sc['shadow_step'], num_mips=sc['mips'])
    light = da * (trv * sc['falloff_col'] + sc['ambient'])
    imgs = ORd.render_fused(np.concatenate([light, da], -1)[None], sc['M'], sc['V'], sc['P'], sc['F'], sc['res'],
                            sc['depth_step'], cut_alpha=False)
    ref = np.concatenate(imgs, 0)
    assert np.max(np.abs(parts['img'] - ref)) <= 1e-12 * max(1.0, np.max(np.abs(ref)))


@pytest.mark.parametrize('mode', ['NONE', 'CLIP_NEGATIVE', 'SATURATE', 'NORMALIZE'])
@pytest.mark.parametrize('shift', [0.0, -0.8])
def test_tonemapped_image_loss_fd(mode, shift):
    """The image loss through the renderer's tonemapping: gradient against
    central differences (random values, no ties or kinks within EPS)."""
    from oracle import tonemap as TM
    rng = np.random.default_rng(71)
    img = rng.random((3, 5, 7, 4)) * 1.6 - 0.3
    img[..., :3] += shift
    tgt = rng.random((3, 5, 7, 3))
    bkg = np.array([0.0, 0.5, 1.0])
    d = rng.standard_normal(img.shape)
    _, g = TM.image_loss(img, tgt, bkg, mode)
    fd = _fd(lambda x: TM.image_loss(x, tgt, bkg, mode)[0], img, d)
    assert abs(np.sum(g * d) - fd) <= 1e-6 * max(abs(fd), 1e-12)


@pytest.mark.parametrize('mode', ['CLIP_NEGATIVE', 'SATURATE', 'NORMALIZE'])
def test_tonemap_ties_and_kinks_follow_tensor_autograd(mode):
    """At ties of the min / max and at the clip points the oracle's gradient
    is the one tensor autograd gives (even split among tied extrema; the
    clip passes at its end points), in float64."""
    import torch
    from gft.pipeline import tonemap_tensor
    from oracle import tonemap as TM
    rng = np.random.default_rng(72)
    c = rng.random((4, 6, 3)) * 2.0 - 0.5
    c[0, 0, 0] = c[1, 2, 1] = c.max() + 0.25    # two maxima
    c[2, 3, 2] = c[3, 1, 0] = c.min() - 0.25    # two minima
    c[1, 1, :] = [0.0, 1.0, 0.5]                # the clip points
    g = rng.standard_normal(c.shape)
    t = torch.tensor(c, dtype=torch.float64, requires_grad=True)
    y = tonemap_tensor(t, mode)
    y.backward(torch.tensor(g))
    assert np.allclose(y.detach().numpy(), TM.tonemap(c, mode), rtol=0, atol=1e-15)
    assert np.allclose(t.grad.numpy(), TM.tonemap_grad(c, g, mode), rtol=1e-12, atol=1e-15)


@pytest.mark.parametrize('mode', ['SATURATE', 'NORMALIZE'])
def test_step_oracle_tonemapped_loss_fd(mode):
    """The step oracle with the tonemapped loss is the true gradient of its
    forward (set-up of test_step_oracle_gradient_fd, MacCormack without the
    clamp)."""
    from gft import synthetic as syn
    from gft.pipeline import RenderAdvectStep
    from oracle import step as OS
    from scene_utils import step_scene
    st = RenderAdvectStep('tiny', 'cpu', order=2, tonemap=mode)
    sc = step_scene(st)
    assert sc['tonemap'] == mode
    sc['mips'] = 0
    sc['clamp'] = 'NONE'
    rng = np.random.default_rng(74)
    d = syn.plume_density(st.shape, 7)[0].astype(np.float64) * 8 + 0.05 + 0.01 * rng.random(st.shape + (1,))
    vel = [v[0].astype(np.float64) for v in syn.curl_velocity(st.shape, 8)]
    tgt = rng.random((len(st.cams), st.res[1], st.res[2], 3)) * 0.3
    _, _, grads = OS.step(sc, d, *vel, tgt, exact=True, shadow_grad='adjoint')
    xs = [d] + vel
    for k in range(4):
        u = rng.standard_normal(xs[k].shape)

        def loss(e):
            a = [x.copy() for x in xs]
            a[k] = a[k] + e * u
            return OS.forward(sc, *a, tgt)[0]
        fd = (loss(EPS) - loss(-EPS)) / (2 * EPS)
        assert abs(fd - np.sum(grads[k] * u)) <= 1e-4 * abs(fd), (k, fd, np.sum(grads[k] * u))
