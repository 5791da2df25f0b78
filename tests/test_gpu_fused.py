"""The fused pipeline kernels (gft.fused) against the tensor-op compositions
they replace: forward and gradients on seeded inputs."""
import numpy as np
import pytest
import torch

from scene_utils import rel_l2

pytestmark = pytest.mark.gpu


@pytest.fixture(scope='module')
def fused():
    if not torch.cuda.is_available():
        pytest.skip('no CUDA device')
    from gft import fused as _f
    return _f


def _np(t):
    return t.detach().cpu().numpy().astype(np.float64)


@pytest.mark.parametrize('shape', [(1, 7, 5, 9, 1), (2, 16, 12, 33, 1)])
def test_transmittance(fused, shape):
    from gft import ops
    g = torch.Generator().manual_seed(3)
    x = (torch.rand(shape, generator=g) * 0.3).cuda()
    gy = torch.randn(shape, generator=g).cuda()
    a = x.clone().requires_grad_(True)
    y = fused.transmittance(a)
    y.backward(gy)
    b = x.clone().requires_grad_(True)
    sh = ops.reduce_grid_blend(b, 'BEER_LAMBERT', keep_dims=True)
    ref = torch.exp(-torch.cat([torch.zeros_like(sh[:, :1]), sh[:, :-1]], dim=1))
    ref.backward(gy)
    assert rel_l2(_np(y), _np(ref)) <= 1e-7
    assert rel_l2(_np(a.grad), _np(b.grad)) <= 1e-6


@pytest.mark.parametrize('N', [1, 2])
def test_light_compose(fused, N):
    g = torch.Generator().manual_seed(4)
    D, H, W = 6, 10, 7
    d0 = torch.rand((N, D, H, W, 1), generator=g).cuda()
    t0 = torch.rand((N, D, H, W, 1), generator=g).cuda()
    col = torch.rand((1, D, H, W, 3), generator=g).cuda()
    gy = torch.randn((N, D, H, W, 4), generator=g).cuda()
    d1, t1 = d0.clone().requires_grad_(True), t0.clone().requires_grad_(True)
    y = fused.light_compose(d1, t1, col, 0.64, 0.37)
    y.backward(gy)
    d2, t2 = d0.clone().requires_grad_(True), t0.clone().requires_grad_(True)
    ref = torch.cat([d2 * (t2 * col + 0.64), d2], dim=-1) * 0.37
    ref.backward(gy)
    assert rel_l2(_np(y), _np(ref)) <= 1e-7
    assert rel_l2(_np(d1.grad), _np(d2.grad)) <= 1e-6
    assert rel_l2(_np(t1.grad), _np(t2.grad)) <= 1e-6


def test_image_loss(fused):
    g = torch.Generator().manual_seed(5)
    img0 = torch.rand((5, 27, 48, 4), generator=g).cuda()
    tgt = torch.rand((5, 27, 48, 3), generator=g).cuda()
    bkg = torch.tensor([0.0, 0.5, 1.0]).cuda()
    a = img0.clone().requires_grad_(True)
    loss = fused.image_loss(a, tgt, bkg)
    (loss * 3.0).backward()
    b = img0.clone().requires_grad_(True)
    ref = torch.mean((b[..., :3] + bkg * torch.exp(-b[..., 3:]) - tgt) ** 2)
    (ref * 3.0).backward()
    assert abs(float(loss) - float(ref)) <= 1e-6 * abs(float(ref))
    assert rel_l2(_np(a.grad), _np(b.grad)) <= 1e-6
    # repeated calls are deterministic (fixed-order reduction)
    assert float(fused.image_loss(a, tgt, bkg)) == float(loss)


@pytest.mark.parametrize('mode', ['NONE', 'CLIP_NEGATIVE', 'SATURATE', 'NORMALIZE'])
@pytest.mark.parametrize('ties', [False, True])
def test_image_loss_tonemap(fused, mode, ties):
    """The loss with the renderer's tonemapping folded in against the FP64
    oracle and against the tensor-op composition (pipeline.tonemap_tensor):
    values below 0 and above 1, and (ties) repeated extrema and pixels exactly
    at the clip points, where the gradient is shared / passed as autograd
    does."""
    from gft.pipeline import tonemap_tensor
    from oracle import tonemap as TM
    g = torch.Generator().manual_seed(8)
    img0 = torch.rand((5, 27, 48, 4), generator=g) * 1.6 - 0.5
    img0[..., 3] = img0[..., 3].abs()
    if ties:
        img0[0, 0, 0, :] = torch.tensor([3.0, -2.0, 0.0, 0.0])
        img0[3, 5, 7, :] = torch.tensor([3.0, -2.0, 0.0, 0.0])   # same composite: tied max (r), tied min (g)
        img0[1, 2, 3, :] = torch.tensor([0.0, 0.5, 0.0, 0.0])    # composite r = 0, g = 1: the clip points
    img0 = img0.cuda()
    tgt = torch.rand((5, 27, 48, 3), generator=g).cuda()
    bkg_host = np.array([0.0, 0.5, 1.0], np.float32)
    bkg = torch.from_numpy(bkg_host).cuda()
    a = img0.clone().requires_grad_(True)
    loss = fused.image_loss(a, tgt, bkg_host, tonemap=mode)
    (loss * 3.0).backward()
    b = img0.clone().requires_grad_(True)
    ref = torch.mean((tonemap_tensor(b[..., :3] + bkg * torch.exp(-b[..., 3:]), mode) - tgt) ** 2)
    (ref * 3.0).backward()
    l64, g64 = TM.image_loss(_np(img0), _np(tgt), bkg_host, mode)
    assert abs(float(loss) - l64) <= 1e-5 * abs(l64)
    assert abs(float(loss) - float(ref)) <= 1e-6 * abs(float(ref))
    assert rel_l2(_np(a.grad), 3.0 * g64) <= 1e-5
    assert rel_l2(_np(a.grad), _np(b.grad)) <= 1e-6
    assert float(fused.image_loss(a, tgt, bkg_host, tonemap=mode)) == float(loss)


@pytest.mark.parametrize('storage', [None, torch.bfloat16])
def test_render_bricked_equals_compose_then_raymarch(fused, storage):
    """The fused composition + bricked raymarch (the composition writing the
    raymarch input in its storage type) against light_compose(brick=True)
    followed by raymarch_grid_transform_bricked with the same storage type:
    identical input bits and images, gradients equal up to summation order."""
    from gft import ops
    from scene_utils import scene
    g = torch.Generator().manual_seed(9)
    D, H, W = 9, 13, 11
    _, _, M, V, P, F = scene((D, H, W), 3, (13, 9, 11))
    d0 = (torch.rand((1, D, H, W, 1), generator=g) * 0.3).cuda()
    t0 = torch.rand((1, D, H, W, 1), generator=g).cuda()
    col = torch.rand((1, D, H, W, 3), generator=g).cuda()
    dy = torch.randn((1, 3, 9, 11, 4), generator=g).cuda()
    d1, t1 = d0.clone().requires_grad_(True), t0.clone().requires_grad_(True)
    img, xs = fused.render_bricked(d1, t1, col, 0.64, 0.37, M, V, P, F, (13, 9, 11), storage_dtype=storage)
    img.backward(dy)
    d2, t2 = d0.clone().requires_grad_(True), t0.clone().requires_grad_(True)
    data = fused.light_compose(d2, t2, col, 0.64, 0.37, brick=True)
    ref = ops.raymarch_grid_transform_bricked(data, (D, H, W), M, V, P, F, (13, 9, 11), storage_dtype=storage)
    ref.backward(dy)
    want = data.detach() if storage is None else data.detach().to(storage)
    assert xs.dtype == want.dtype
    # the bricks of odd-sized grids carry padding cells that nothing writes
    assert torch.equal(ops.from_bricks(xs.float(), (D, H, W)), ops.from_bricks(want.float(), (D, H, W)))
    assert torch.equal(img, ref)
    assert rel_l2(_np(d1.grad), _np(d2.grad)) <= 1e-6
    assert rel_l2(_np(t1.grad), _np(t2.grad)) <= 1e-6


@pytest.mark.parametrize('storage', [None, torch.bfloat16])
@pytest.mark.parametrize('gmode', ['REFERENCE', 'REFERENCE_CAMERA_SUMS', 'EXACT', 'DETERMINISTIC'])
@pytest.mark.parametrize('store', [True, False])
def test_render_bricked_factored_light(fused, storage, gmode, store):
    """A factored light (falloff [D, H, W, 1] x rgb): the composition forms
    falloff * rgb by the same rounded product as a precomputed colour grid, so
    the raymarch input and images equal those of the colour grid bit for bit;
    the adjoint accumulates the two projections of the raymarch gradient that
    the composition's adjoint reads (REFERENCE: the weight pass ahead and a
    normalised scatter, or per-camera value and weight sums from one pass,
    divided per voxel; the deterministic adjoint: projected after its integer
    sums), and the density and transmittance gradients equal the colour
    grid's up to summation order."""
    from gft import ops
    from scene_utils import scene
    g = torch.Generator().manual_seed(19)
    D, H, W = 9, 13, 11
    _, _, M, V, P, F = scene((D, H, W), 3, (13, 9, 11))
    d0 = (torch.rand((1, D, H, W, 1), generator=g) * 0.3).cuda()
    t0 = torch.rand((1, D, H, W, 1), generator=g).cuda()
    fall = torch.rand((D, H, W, 1), generator=g).cuda()
    rgb = np.array([0.9, 0.7, 1.3], np.float32)
    col = (fall * torch.from_numpy(rgb).cuda())[None].contiguous()
    dy = torch.randn((1, 3, 9, 11, 4), generator=g).cuda()
    saved = ops.get_grad_mode(), ops._state['deterministic'], ops._state['sample_store'], ops._state['camera_sums']
    try:
        ops.set_grad_mode('EXACT' if gmode == 'EXACT' else 'REFERENCE')
        ops.set_deterministic(gmode == 'DETERMINISTIC')
        ops.set_raymarch_sample_store(store)
        ops.set_raymarch_camera_sums(gmode == 'REFERENCE_CAMERA_SUMS')
        res = []
        for light in ((fall, rgb), col):
            d1, t1 = d0.clone().requires_grad_(True), t0.clone().requires_grad_(True)
            img, xs = fused.render_bricked(d1, t1, light, 0.64, 0.37, M, V, P, F, (13, 9, 11),
                                           storage_dtype=storage)
            img.backward(dy)
            res.append((img.detach(), ops.from_bricks(xs.float(), (D, H, W)), d1.grad, t1.grad))
    finally:
        ops.set_grad_mode(saved[0])
        ops.set_deterministic(saved[1])
        ops.set_raymarch_sample_store(saved[2])
        ops.set_raymarch_camera_sums(saved[3])
    (i1, x1, gd1, gt1), (i2, x2, gd2, gt2) = res
    assert torch.equal(x1, x2)
    assert torch.equal(i1, i2)
    assert np.abs(_np(gd2)).max() > 0 and np.abs(_np(gt2)).max() > 0
    assert rel_l2(_np(gd1), _np(gd2)) <= 1e-6
    assert rel_l2(_np(gt1), _np(gt2)) <= 1e-6


@pytest.mark.parametrize('gmode', ['REFERENCE', 'EXACT'])
@pytest.mark.parametrize('det', [False, True])
def test_raymarch_grad_projected(fused, gmode, det):
    """gft_raymarch_grid_transform_grad_projected against the projection of the
    plain 4-channel gradient (bricked input, both grad modes; deterministic:
    two int64 sums per cell, bit-identical from run to run)."""
    from gft import ops
    from scene_utils import scene
    g = torch.Generator().manual_seed(21)
    D, H, W = 10, 14, 12
    _, _, M, V, P, F = scene((D, H, W), 2, (12, 10, 9))
    x = (torch.rand((1, D, H, W, 4), generator=g) * 0.3).cuda()
    xb = ops.to_bricks(x)
    y = ops.raymarch_grid_transform_bricked(xb, (D, H, W), M, V, P, F, (12, 10, 9)).detach().contiguous()
    dy = torch.randn(y.shape, generator=g).cuda()
    proj = np.array([0.3, -1.2, 0.7, 0.0, 0.5, 0.5, 0.5, 1.1], np.float32)
    gm = ops.GRAD[gmode]
    args = (xb, y, dy, M, V, P, F, (12, 10, 9), ops.FILTER['LINEAR'], ops.BOUNDARY['BORDER'],
            ops.BLEND['BEER_LAMBERT'], True)
    g4 = ops._raymarch_bwd(*args, gm, grid=(D, H, W))
    gp = gm | (ops.DETERMINISTIC if det else 0)
    g2 = ops._raymarch_bwd(*args, gp, grid=(D, H, W), projection=proj)
    if det:
        assert torch.equal(g2, ops._raymarch_bwd(*args, gp, grid=(D, H, W), projection=proj))
    assert tuple(g2.shape) == tuple(xb.shape[:-1]) + (2,)
    pm = torch.from_numpy(proj.reshape(2, 4)).cuda()
    ref = torch.stack([(g4 * pm[0]).sum(-1), (g4 * pm[1]).sum(-1)], -1)
    a, b = _np(ops.from_bricks(g2, (D, H, W))), _np(ops.from_bricks(ref, (D, H, W)))
    assert np.abs(b).max() > 0
    assert rel_l2(a, b) <= 1e-6


def test_fused_argument_errors(fused):
    from gft import _lib
    with pytest.raises(_lib.GftInvalidArgument):
        fused.transmittance(torch.zeros((1, 4, 4, 4, 2), device='cuda'))
    with pytest.raises(_lib.GftInvalidArgument):
        fused.light_compose(torch.zeros((1, 4, 4, 4, 1), device='cuda'), torch.zeros((1, 4, 4, 3, 1), device='cuda'),
                            torch.zeros((4, 4, 4, 3), device='cuda'), 0.5, 1.0)
    with pytest.raises(_lib.GftInvalidArgument):
        fused.image_loss(torch.zeros((2, 3, 4), device='cuda'), torch.zeros((2, 3, 4), device='cuda'), [0, 0, 0])
    with pytest.raises(_lib.GftInvalidArgument):
        fused.image_loss(torch.zeros((2, 3, 4), device='cuda'), torch.zeros((2, 3, 3), device='cuda'), [0, 0, 0],
                         tonemap='GAMMA')
