"""Parity at the benchmark configurations, against the FP64 oracle.

* cfg1 at full size (density 64^3, one 128x128 view, 64 depth samples, spot
  light with a 64^3 shadow frustum and 3 mips, one advection step): the whole
  render + advect iteration -- image, loss and the gradients to the previous
  density and the three staggered velocity components -- against the FP64
  step oracle, for semi-Lagrangian and MacCormack advection, reference and
  exact gradients, FP32 and BF16 storage.
* cfg2 (128x227x128, 5 views of 480x270, 192 samples, 3 mips) and cfg5
  (256x455x256, 5 views of 960x540, 256 samples, 4 mips): the ops of the
  iteration on the full grids, compared with the oracle on a 32^3 sub-block.
  Raymarch: the oracle marches every ray that can reach the block (the
  block's projection into each image, widened by two pixels) and the density
  gradient is compared inside the block.  Advection: the oracle advects a
  crop of the block plus a 12-voxel halo, wider than the reach of the two
  MacCormack lookups, so the block's forward values and gradients are those
  of the full grid.  Shadow resampling: a 32^3 box of the light frustum
  (volume -> frustum, mips) and of the volume (frustum -> volume).

Tolerances (rel-L2 against FP64): FP32 storage 1e-5 forward and 1e-4 for
gradients; BF16 storage 1e-2 for both.  The inputs are seeded synthetic plumes
with the configurations' shapes.

Advection gradients are compared outside the few voxels (well under 1 % of
the grid, bounded by MASK_FRACTION) where the reference's adjoint is
discontinuous in the lookup positions -- its sample-count normalisation, the
one-sided spatial derivative at cell boundaries and the MC_SMOOTH selection
(tests/tie_masks.py) -- so that FP32 and FP64 rounding legitimately pick
different sides there.
"""
import numpy as np
import pytest
import torch

from scene_utils import rel_l2, step_scene

pytestmark = pytest.mark.gpu

FWD_F32, GRAD_F32, BF16 = 1e-5, 1e-4, 1e-2
BLOCK = 32
MASK_FRACTION = 0.02


def _masked_rel_l2(a, b, mask=None):
    if mask is not None:
        m = np.broadcast_to(mask.reshape(mask.shape + (1,) * (np.ndim(b) - mask.ndim)), np.shape(b))
        a = np.where(m, 0.0, a)
        b = np.where(m, 0.0, b)
    return rel_l2(a, b)


@pytest.fixture(scope='module')
def gpu():
    if not torch.cuda.is_available():
        pytest.skip('no CUDA device')
    from gft import ops
    ops.set_grad_mode('REFERENCE')
    return torch.device('cuda', 0)


def _np(t):
    return t.detach().float().cpu().numpy().astype(np.float64)


def _tol(storage, fwd):
    if storage == 'bf16':
        return BF16
    return FWD_F32 if fwd else GRAD_F32


def _dtype(storage):
    return torch.bfloat16 if storage == 'bf16' else None


# ----------------------------------------------------------------- cfg1 step
_cfg1_oracle = {}
_cfg1_inputs = {}


def _cfg1_step_inputs(order, gpu):
    """Seeded inputs of cfg1 (target images rendered by the FP32 step), shared
    by the FP32 and BF16 storage cases."""
    if order not in _cfg1_inputs:
        from gft.pipeline import RenderAdvectStep
        _cfg1_inputs[order] = RenderAdvectStep('cfg1', gpu, order=order).make_inputs()
    return _cfg1_inputs[order]


def _cfg1_reference(step, inputs, exact):
    from oracle import step as OS
    key = (step.order, exact)
    if key not in _cfg1_oracle:
        sc = step_scene(step)
        d = inputs['d_prev'][0].astype(np.float64)
        vel = [inputs[k].astype(np.float64) for k in ('vx', 'vy', 'vz')]
        _cfg1_oracle[key] = OS.step(sc, d, *vel, inputs['target'], exact=exact)
    return _cfg1_oracle[key]


@pytest.mark.parametrize('storage', ['f32', 'bf16'])
@pytest.mark.parametrize('mode', ['REFERENCE', 'EXACT'])
@pytest.mark.parametrize('order', [1, 2])
def test_cfg1_step_vs_fp64_oracle(gpu, order, mode, storage):
    from gft import ops
    from gft.pipeline import RenderAdvectStep
    st = RenderAdvectStep('cfg1', gpu, storage_dtype=_dtype(storage), order=order)
    inputs = _cfg1_step_inputs(order, gpu)
    st.setup_static(inputs)
    with ops.grad_mode(mode):
        loss, grads = st.run_static()
        with torch.no_grad():
            img = st.render(st.advect(st.s_d, st.s_vx, st.s_vy, st.s_vz))
    torch.cuda.synchronize()
    ref_loss, ref_img, ref_grads = _cfg1_reference(st, inputs, mode == 'EXACT')
    assert rel_l2(_np(img), ref_img) <= _tol(storage, True)
    assert abs(float(loss.detach()) - ref_loss) <= _tol(storage, True) * abs(ref_loss)
    import tie_masks as TM
    d0 = inputs['d_prev'][0].astype(np.float64)
    vel = [inputs[k].astype(np.float64) for k in ('vx', 'vy', 'vz')]
    dmask, vmask = TM.advect_masks(d0, *vel, order=order, clamp=st.clamp, reference=mode == 'REFERENCE')
    assert dmask.mean() <= MASK_FRACTION and vmask.mean() <= MASK_FRACTION
    masks = (dmask,) + TM.face_masks(vmask)
    for name, g, r, m in zip(('density', 'vel_x', 'vel_y', 'vel_z'), grads, ref_grads, masks):
        e = _masked_rel_l2(_np(g).reshape(r.shape), r, m)
        assert e <= _tol(storage, False), '%s gradient rel-L2 %.3g' % (name, e)


# --------------------------------------------------------- full-size scenes
_scenes = {}


def _scene(cfg, gpu):
    """Host scene of a configuration: cameras, light, seeded plume density and
    staggered velocity at full size."""
    if cfg not in _scenes:
        from gft import synthetic as syn
        from gft.pipeline import RenderAdvectStep
        st = RenderAdvectStep(cfg, gpu)
        d = syn.plume_density(st.shape, st.cfg['seed'])
        vel = syn.curl_velocity(st.shape, st.cfg['seed'] + 500)
        _scenes[cfg] = (step_scene(st), st.shape, d, vel)
    return _scenes[cfg]


def _blocks(shape):
    """A 32^3 block inside the plume (on its axis, in its lower half) and one
    at the grid's corner (x = 0, y = 0), where the BORDER cut-off lies."""
    D, H, W = shape
    z0, x0 = D // 2 - BLOCK // 2, W // 2 - BLOCK // 2
    y0 = max(0, int(0.2 * H) - BLOCK // 2)
    return {'plume': (z0, y0, x0), 'corner': (z0, 0, 0)}


def _box(b):
    z0, y0, x0 = b
    return (slice(z0, z0 + BLOCK), slice(y0, y0 + BLOCK), slice(x0, x0 + BLOCK))


def _raymarch_input(sc, d):
    return (np.concatenate([d * 0.7, d * 0.5, d * 0.3, d], axis=-1) * sc['depth_step']).astype(np.float32)


_rm_gpu = {}


def _raymarch_gpu(cfg, gpu, storage, mode, adjoint):
    key = (cfg, storage, mode, adjoint)
    if key not in _rm_gpu:
        from gft import ops
        sc, shape, d, _ = _scene(cfg, gpu)
        x = torch.from_numpy(_raymarch_input(sc, d)).to(gpu).requires_grad_(True)
        with ops.grad_mode(mode):
            y = ops.raymarch_grid_transform(x, sc['M'], sc['V'], sc['P'], sc['F'], sc['res'],
                                            storage_dtype=_dtype(storage))
            if adjoint == 'image':
                dy = (y.detach() * 1e-2).contiguous()    # the gradient of 0.005 |img|^2
            else:
                g = torch.Generator(device=gpu).manual_seed(17)
                dy = torch.randn(y.shape, generator=g, device=gpu) * 1e-3
            (gx,) = torch.autograd.grad(y, x, dy)
        torch.cuda.synchronize()
        _rm_gpu.clear()  # keep one full-size result at a time
        _rm_gpu[key] = (_np(y), _np(dy), gx.detach().cpu().numpy())
    return _rm_gpu[key]


def _raymarch_oracle(sc, x, dy_full, b, exact):
    from oracle import subblock as SB
    return SB.raymarch_block(x, sc['M'], sc['V'], sc['P'], sc['F'], sc['res'], dy_full, b, BLOCK, exact)


@pytest.mark.parametrize('storage', ['f32', 'bf16'])
@pytest.mark.parametrize('mode', ['REFERENCE', 'EXACT'])
@pytest.mark.parametrize('cfg', ['cfg2', 'cfg5'])
def test_raymarch_subblock_vs_fp64(gpu, cfg, mode, storage):
    sc, shape, d, _ = _scene(cfg, gpu)
    b = _blocks(shape)['plume']
    y_gpu, dy, gx = _raymarch_gpu(cfg, gpu, storage, mode, 'image')
    x = _raymarch_input(sc, d)
    y_ref, g_ref, rows, cols = _raymarch_oracle(sc, x, dy, b, mode == 'EXACT')
    for c in range(len(sc['V'])):
        w = (0, c, rows[c], cols[c])
        assert rel_l2(y_gpu[w], y_ref[w]) <= _tol(storage, True), 'camera %d image window' % c
    box = (0,) + _box(b)
    assert np.abs(g_ref[box]).max() > 0
    e = rel_l2(gx[box], g_ref[box])
    assert e <= _tol(storage, False), '%s %s sub-block gradient rel-L2 %.3g' % (cfg, mode, e)


# Noise adjoint: an i.i.d. Gaussian output gradient weights every sample
# equally, including those on the BORDER cut-off half a cell outside the grid,
# where a sample is in or out depending on the last bit of its position.  The
# positions here come from fp64-folded camera matrices rounded to fp32, the
# oracle's from fp64 end to end, so a few samples on the cut-off differ.  The
# stated bound covers that; inside the plume the image adjoint above holds
# the gradient to 1e-4.
NOISE_BOUND = 1e-3


@pytest.mark.parametrize('where', ['plume', 'corner'])
def test_raymarch_noise_adjoint_bound_cfg2(gpu, where):
    sc, shape, d, _ = _scene('cfg2', gpu)
    b = _blocks(shape)[where]
    _, dy, gx = _raymarch_gpu('cfg2', gpu, 'f32', 'REFERENCE', 'noise')
    x = _raymarch_input(sc, d)
    _, g_ref, _, _ = _raymarch_oracle(sc, x, dy, b, False)
    box = (0,) + _box(b)
    e = rel_l2(gx[box], g_ref[box])
    assert e <= NOISE_BOUND, '%s block: noise-adjoint gradient rel-L2 %.3g' % (where, e)


# ---------------------------------------------------------------- advection
HALO = 12


def _crop(shape, b, halo=HALO):
    D, H, W = shape
    z0, y0, x0 = b
    return tuple((max(0, o - halo), min(n, o + BLOCK + halo)) for o, n in ((z0, D), (y0, H), (x0, W)))


@pytest.mark.parametrize('storage', ['f32', 'bf16'])
@pytest.mark.parametrize('mode', ['REFERENCE', 'EXACT'])
@pytest.mark.parametrize('cfg', ['cfg2', 'cfg5'])
def test_advect_subblock_vs_fp64(gpu, cfg, mode, storage):
    from gft import ops
    from oracle import advect as OA
    from oracle import sampling as S
    sc, shape, d, (vx, vy, vz) = _scene(cfg, gpu)
    b = _blocks(shape)['plume']
    dt = torch.from_numpy(d).to(gpu).requires_grad_(True)
    vs = [torch.from_numpy(v).to(gpu).requires_grad_(True) for v in (vx, vy, vz)]
    g = torch.Generator(device=gpu).manual_seed(23)
    with ops.grad_mode(mode):
        out = ops.advect(dt, *vs, dt=1.0, order=2, clamp='MC_SMOOTH', boundary='CLAMP', storage_dtype=_dtype(storage))
        dy = torch.randn(out.shape, generator=g, device=gpu)
        grads = torch.autograd.grad(out, [dt] + vs, dy)
    torch.cuda.synchronize()
    (cz0, cz1), (cy0, cy1), (cx0, cx1) = _crop(shape, b)
    dc = d[0, cz0:cz1, cy0:cy1, cx0:cx1].astype(np.float64)
    vxc = vx[0, cz0:cz1, cy0:cy1, cx0:cx1 + 1].astype(np.float64)
    vyc = vy[0, cz0:cz1, cy0:cy1 + 1, cx0:cx1].astype(np.float64)
    vzc = vz[0, cz0:cz1 + 1, cy0:cy1, cx0:cx1].astype(np.float64)
    dyc = _np(dy)[0, cz0:cz1, cy0:cy1, cx0:cx1]
    ref = OA.warp(dc, vxc, vyc, vzc, 1.0, 2, 'MC_SMOOTH', S.CLAMP)
    rg = OA.warp_grad(dc, vxc, vyc, vzc, dyc, 1.0, 2, 'MC_SMOOTH', S.CLAMP, exact=mode == 'EXACT')
    import tie_masks as TM
    dmask, vmask = TM.advect_masks(dc, vxc, vyc, vzc, reference=mode == 'REFERENCE')
    mfx, mfy, mfz = TM.face_masks(vmask)
    z0, y0, x0 = b
    lb = (slice(z0 - cz0, z0 - cz0 + BLOCK), slice(y0 - cy0, y0 - cy0 + BLOCK), slice(x0 - cx0, x0 - cx0 + BLOCK))
    gb = _box(b)
    assert dmask[lb].mean() <= MASK_FRACTION and vmask[lb].mean() <= MASK_FRACTION
    assert rel_l2(_np(out)[0][gb], ref[lb]) <= _tol(storage, True)
    e = _masked_rel_l2(_np(grads[0])[0][gb], rg[0][lb], dmask[lb])
    assert e <= _tol(storage, False), 'density gradient rel-L2 %.3g' % e
    # staggered faces of the block's voxels (x faces x0..x0+BLOCK, ...)
    fx = (gb[0], gb[1], slice(x0, x0 + BLOCK + 1))
    lfx = (lb[0], lb[1], slice(lb[2].start, lb[2].stop + 1))
    fy = (gb[0], slice(y0, y0 + BLOCK + 1), gb[2])
    lfy = (lb[0], slice(lb[1].start, lb[1].stop + 1), lb[2])
    fz = (slice(z0, z0 + BLOCK + 1), gb[1], gb[2])
    lfz = (slice(lb[0].start, lb[0].stop + 1), lb[1], lb[2])
    for name, gg, r, f, lf, m in (('x', grads[1], rg[1], fx, lfx, mfx), ('y', grads[2], rg[2], fy, lfy, mfy),
                                  ('z', grads[3], rg[3], fz, lfz, mfz)):
        e = _masked_rel_l2(_np(gg)[0][f], r[lf], m[lf])
        assert e <= _tol(storage, False), 'velocity %s gradient rel-L2 %.3g' % (name, e)


# ------------------------------------------------------- shadow resampling
@pytest.mark.parametrize('cfg', ['cfg2', 'cfg5'])
def test_shadow_resampling_subblock_vs_fp64(gpu, cfg):
    """The two resamplings of the shadow pass with mips: volume -> light
    frustum (LINDEPTH) on a 32^3 box of the frustum, and frustum -> volume
    (LINDEPTH_REVERSE) on a 32^3 box of the volume."""
    from gft import ops
    from oracle import resample as R
    from oracle import sampling as S
    from oracle import transforms as T
    sc, shape, d, _ = _scene(cfg, gpu)
    x = (d * sc['shadow_step']).astype(np.float32)
    kw = dict(interpolation='LINEAR', boundary='BORDER', mipmapping='LINEAR', num_mipmaps=sc['mips'])
    sh = ops.sample_grid_transform(torch.from_numpy(x).to(gpu), sc['M'], sc['Vs'], sc['Ps'], sc['Fs'],
                                   sc['shadow_res'], coordinate_mode='TRANSFORM_LINDEPTH', **kw)
    sh = _np(sh)[0]                                                    # [1, Ds, Hs, Ws, 1]
    Ds, Hs, Ws = sc['shadow_res']
    # a 32^3 box of the frustum centred on the plume's light-facing side: the
    # cell of the largest sample
    cz, cy, cx = np.unravel_index(np.argmax(sh[0, ..., 0]), sh.shape[1:4])
    fbox = tuple((min(max(0, c - BLOCK // 2), n - BLOCK), min(max(0, c - BLOCK // 2), n - BLOCK) + BLOCK)
                 for c, n in ((cz, Ds), (cy, Hs), (cx, Ws)))
    ref = R.sample_grid_transform(x.astype(np.float64), sc['M'], sc['Vs'], sc['Ps'], sc['Fs'], sc['shadow_res'],
                                  S.LINEAR, S.BORDER, S.MIP_LINEAR, sc['mips'], 0.0, T.LINDEPTH, out_box=fbox)[0, 0]
    got = sh[0][tuple(slice(a, b) for a, b in fbox)]
    assert np.abs(ref).max() > 0
    assert rel_l2(got, ref) <= FWD_F32
    # frustum -> volume on a smooth frustum field (the transmittance of sh)
    tr = np.exp(-np.cumsum(sh[0], axis=0)).astype(np.float32)[None]
    back = ops.sample_grid_transform(torch.from_numpy(tr).to(gpu), sc['M'], sc['Vs'], sc['Ps'], sc['Fs'], shape,
                                     coordinate_mode='TRANSFORM_LINDEPTH_REVERSE', **kw)
    z0, y0, x0 = _blocks(shape)['plume']
    vbox = ((z0, z0 + BLOCK), (y0, y0 + BLOCK), (x0, x0 + BLOCK))
    ref = R.sample_grid_transform(tr.astype(np.float64), sc['M'], sc['Vs'], sc['Ps'], sc['Fs'], shape, S.LINEAR,
                                  S.BORDER, S.MIP_LINEAR, sc['mips'], 0.0, T.LINDEPTH_REVERSE, out_box=vbox)[0, 0]
    got = _np(back)[0, 0][tuple(slice(a, b) for a, b in vbox)]
    assert rel_l2(got, ref) <= FWD_F32
