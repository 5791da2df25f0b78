"""The Python composition on the hot path (phitest.render.{renderer, lighting,
data_structures} mirrors) against the oracle's restatement of the reference
composition, on the GPU."""
import numpy as np
import pytest
import torch

from scene_utils import rel_l2, scene, small_grid

pytestmark = pytest.mark.gpu

FWD_TOL = 1e-5
GRAD_TOL = 1e-4


@pytest.fixture(scope='module')
def mods():
    if not torch.cuda.is_available():
        pytest.skip('no CUDA device')
    from gft import ops
    from phitest.render import data_structures as ds
    from phitest.render import lighting, renderer
    return ops, renderer, lighting, ds


def cuda(a):
    return torch.from_numpy(np.ascontiguousarray(a, dtype=np.float32)).cuda()


def np_(t):
    return t.detach().cpu().numpy().astype(np.float64)


def _spot(lighting, res=(12, 10, 10)):
    from phitest.render.transform import Transform
    return lighting.SpotLight(Transform(translation=[0, 0, 2.0], parent=Transform(rotation_deg=[-35, 20, 0])),
                              intensity=0.9, cast_shadows=True, shadow_clip=[1.0, 3.0], range_scale=0.8,
                              angle_deg=50.0, shadow_resolution=list(res), cone_mask=False)


@pytest.mark.parametrize('fused', [True, False])
def test_render_density_with_shadowed_spot_light(mods, fused):
    ops, renderer, lighting, _ = mods
    from oracle import render as ORr
    from oracle import raymarch as RM
    from oracle import resample as R
    from oracle import sampling as S
    from oracle import transforms as OT
    from oracle import blend as OB
    from gft import synthetic as syn
    shape, res = (10, 14, 12), (13, 9, 11)
    gt, cams, M, V, P, F = scene(shape, 2, res)
    d = small_grid(shape, 1, 70) * 0.5
    gt.set_data(cuda(d))
    spot = _spot(lighting)
    amb = lighting.Light(intensity=0.6)
    r = renderer.Renderer(filter_mode='LINEAR', boundary_mode='BORDER', mipmapping='LINEAR', num_mips=2,
                          blend_mode='BEER_LAMBERT', sample_gradients=True, fused=fused)
    bkg = [np.array([0.0, 0.5, 1.0], dtype=np.float32)] * 2
    imgs = r.render_density(gt, [spot, amb], cams, background=bkg)
    # oracle composition
    Vs, Ps, Fs = syn.camera_params([spot.shadow_cam])
    T = ORr.shadow_transmission(d.astype(np.float64), M, Vs, Ps, Fs, tuple(spot.shadow_resolution),
                                spot.shadow_cam.depth_step, S.LINEAR, S.BORDER, S.MIP_LINEAR, 2)
    pos_os = (gt.get_inverse_transform() @ spot.t.position_global())[:3]
    fall = ORr.point_falloff(shape, gt.cell_size_world(), gt.grid_size_world(), pos_os, spot.s)
    col = spot.c * spot.i
    light = d[0] * (T * fall * col) + d[0] * (amb.c * amb.i)
    data = np.concatenate([light, d[0]], -1)[None]
    step = cams[0].depth_step
    if fused:
        ref = ORr.render_fused(data, M, V, P, F, res, step, background=np.stack(bkg))
    else:
        fr = R.sample_grid_transform(data * step, M, V, P, F, res, S.LINEAR, S.BORDER, S.MIP_LINEAR, 2, 0.0,
                                     OT.LINDEPTH)[0]  # [V,D,H,W,4]
        img = OB.reduce_grid_blend(fr, OB.BEER_LAMBERT, False)
        t = np.exp(-img[..., -1:])
        img = img[..., :-1] + np.stack(bkg)[:, None, None, :] * t
        ref = [img[i:i + 1] for i in range(2)]
    for got, want in zip(imgs, ref):
        assert rel_l2(np_(got), want) <= FWD_TOL


def test_shadow_sample_gradient_is_inverse_resampling(mods):
    """sample_gradients=True: the gradient of a frustum resample is dy resampled
    back with the inverse coordinate mode, summed over views (renderer.py:246-272)."""
    ops, renderer, lighting, _ = mods
    from oracle import resample as R
    from oracle import sampling as S
    from oracle import transforms as OT
    shape, res = (10, 14, 12), (13, 9, 11)
    gt, cams, M, V, P, F = scene(shape, 2, res)
    d = small_grid(shape, 2, 71)
    r = renderer.Renderer(mipmapping='LINEAR', num_mips=2, sample_gradients=True, fast_gradient_mip_bias_add=0.5)
    x = cuda(d).requires_grad_(True)
    y = r.sample_camera(x, gt, cams)
    dy = np.random.default_rng(72).standard_normal(tuple(y.shape)).astype(np.float32)
    y.backward(cuda(dy))
    ref = sum(R.sample_grid_transform(dy[v:v + 1], M, V[v:v + 1], P[v:v + 1], F[v:v + 1], shape, S.LINEAR, S.BORDER,
                                      S.MIP_LINEAR, 2, 0.5, OT.LINDEPTH_REVERSE)[0, 0] for v in range(2))
    assert rel_l2(np_(x.grad)[0], ref) <= FWD_TOL


def _velocity(ds, renderer, shape, seed):
    rng = np.random.default_rng(seed)
    D, H, W = shape
    vx = cuda(rng.standard_normal((1, D, H, W + 1, 1)) * 0.8)
    vy = cuda(rng.standard_normal((1, D, H + 1, W, 1)) * 0.8)
    vz = cuda(rng.standard_normal((1, D + 1, H, W, 1)) * 0.8)
    warp_r = renderer.Renderer(filter_mode='LINEAR', boundary_mode='CLAMP', mipmapping='NONE', blend_mode='ADDITIVE')
    scale_r = renderer.Renderer(filter_mode='LINEAR', boundary_mode='CLAMP', mipmapping='NONE', blend_mode='ADDITIVE')
    return ds.VelocityGrid(list(shape), x=vx, y=vy, z=vz, warp_renderer=warp_r, scale_renderer=scale_r)


@pytest.mark.parametrize('order,clamp', [(1, 'NONE'), (2, 'MC_SMOOTH'), (2, 'NEGATIVE')])
@pytest.mark.parametrize('mode', ['REFERENCE', 'EXACT'])
def test_fused_warp_equals_reference_composition(mods, order, clamp, mode):
    """VelocityGrid.warp (one fused CUDA pass per stage) against the reference's
    composition of SampleGridLut calls, values and both gradient modes."""
    ops, renderer, _, ds = mods
    shape = (9, 10, 8)
    vel = _velocity(ds, renderer, shape, 80)
    d0 = small_grid(shape, 1, 81, positive=(clamp != 'NEGATIVE'))
    go = cuda(np.random.default_rng(82).standard_normal(d0.shape))
    outs, grads = [], []
    with ops.grad_mode(mode):
        for fn in (vel.warp, vel.warp_composed):
            d = cuda(d0).requires_grad_(True)
            for c in (vel._x, vel._y, vel._z):
                c.requires_grad_(True)
                c.grad = None
            y = fn(d, order=order, dt=1.2, clamp=clamp)
            y.backward(go)
            outs.append(np_(y))
            grads.append([np_(d.grad), np_(vel._x.grad), np_(vel._y.grad), np_(vel._z.grad)])
    assert rel_l2(outs[0], outs[1]) <= FWD_TOL
    for a, b in zip(grads[0], grads[1]):
        assert rel_l2(a, b) <= GRAD_TOL


def test_velocity_self_advection_vs_oracle(mods):
    ops, renderer, _, ds = mods
    from oracle import resample as R
    from oracle import sampling as S
    shape = (7, 8, 6)
    vel = _velocity(ds, renderer, shape, 90)
    x, y, z = vel.warped(order=2, dt=1.0, clamp='MC_SMOOTH')
    comps = [np_(vel.x)[0], np_(vel.y)[0], np_(vel.z)[0]]
    shapes = vel.x_shape, vel.y_shape, vel.z_shape
    f, t = 0.5, -0.5
    offs = {('X', 'Y'): [f, t, 0.0], ('X', 'Z'): [f, 0.0, t], ('Y', 'X'): [t, f, 0.0], ('Y', 'Z'): [0.0, f, t],
            ('Z', 'X'): [t, 0.0, f], ('Z', 'Y'): [0.0, t, f]}

    def shifted(src_i, target, tshape):
        src = 'XYZ'[src_i]
        if src == target:
            return comps[src_i]
        lut = np.zeros((1,) + tuple(tshape) + (4,))
        lut[..., :3] = offs[(src, target)]
        return R.sample_grid_lut(comps[src_i][None], lut, S.LINEAR, S.CLAMP)[0, 0]

    def look(data, lut, filt):
        l4 = np.concatenate([lut, np.zeros(lut.shape[:-1] + (1,))], -1)[None]
        return R.sample_grid_lut(data[None], l4, filt, S.CLAMP, separate_camera_batch=False)[0, 0]

    for ci, (comp, tshape, got) in enumerate(zip('XYZ', shapes, (x, y, z))):
        lut = -np.concatenate([shifted(i, comp, tshape) for i in range(3)], -1)
        data = comps[ci]
        fwd = look(data, lut, S.LINEAR)
        back = look(fwd, -lut, S.LINEAR)
        corr = fwd + 0.5 * (data - back)
        mn, mx = look(data, lut, S.MIN), look(data, lut, S.MAX)
        want = np.where((corr < mn) | (corr > mx), fwd, corr)
        assert rel_l2(np_(got)[0], want) <= FWD_TOL


def test_sequence_density_chain(mods):
    ops, renderer, _, ds = mods
    from oracle import advect as OA
    from oracle import sampling as S
    shape = (8, 9, 7)
    vels = [_velocity(ds, renderer, shape, 100 + i) for i in range(3)]
    d0 = small_grid(shape, 1, 110)
    seq = ds.Sequence([ds.State(ds.DensityGrid(list(shape), d=cuda(d0) if i == 0 else None), vels[i], frame=i)
                       for i in range(3)])
    seq.densities_advect_fwd(dt=1.0, order=2, clamp='MC_SMOOTH')
    ref = d0[0].astype(np.float64)
    for i in range(1, 3):
        v = vels[i - 1]
        ref = OA.warp(ref, np_(v.x)[0], np_(v.y)[0], np_(v.z)[0], 1.0, 2, 'MC_SMOOTH', S.CLAMP)
        assert rel_l2(np_(seq[i].density.d)[0], ref) <= 1e-5 * (i + 1)


def test_resample_grid3D_aligned(mods):
    ops, renderer, _, _ = mods
    from oracle import resample as R
    from oracle import sampling as S
    from oracle import transforms as OT
    from phitest.render.transform import GridTransform
    r = renderer.Renderer(filter_mode='LINEAR', boundary_mode='CLAMP', mipmapping='NONE')
    d = small_grid((6, 7, 5), 2, 120)
    y = r.resample_grid3D_aligned(cuda(d), [9, 11, 8], 'BORDER', 'CENTER', 'STAGGER_OUTPUT')
    in_t = GridTransform([6, 7, 5], scale=[2. / 5, 2. / 11 * 10. / 6., 2. / 7], center=True)
    tgt = GridTransform([9, 11, 8])
    Mm = in_t.get_transform_matrix().T[None]
    Vv = tgt.get_inverse_transform().T[None]
    Pp = np.eye(4, dtype=np.float32)[None]
    Ff = np.array([[-1, 1, -1, 1, 1, -1]], dtype=np.float32)
    ref = R.sample_grid_transform(d, Mm, Vv, Pp, Ff, (9, 11, 8), S.LINEAR, S.CLAMP, S.MIP_NONE, 0, 0.0,
                                  OT.TRANSFORM)[:, 0]
    assert rel_l2(np_(y), ref) <= FWD_TOL
