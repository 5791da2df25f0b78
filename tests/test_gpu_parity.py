"""CUDA path (libgft.so via gft.ops) vs the FP64 oracle on small seeded cases.

Tolerances: forward rel-L2 <= 1e-5 (fp32 storage) and <= 1e-2 (bf16 storage);
gradients rel-L2 <= 1e-4 (fp32 atomics change only the summation order).
"""
import numpy as np
import pytest
import torch

from scene_utils import rel_l2, scene, small_grid

pytestmark = pytest.mark.gpu

FWD_TOL = 1e-5
BF16_TOL = 1e-2
GRAD_TOL = 1e-4

BLENDS = ['BEER_LAMBERT', 'ALPHA', 'ALPHA_ADDITIVE', 'ADDITIVE']
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


# ------------------------------------------------------------------ raymarch
@pytest.mark.parametrize('C', [1, 2, 4])
@pytest.mark.parametrize('blend', BLENDS)
@pytest.mark.parametrize('boundary', BOUNDS)
def test_raymarch_forward(ops, C, blend, boundary):
    from oracle import raymarch as RM
    from oracle import blend as OB
    from oracle import sampling as OS
    _, _, M, V, P, F = scene((10, 14, 12), 3, (13, 9, 11))
    x = small_grid((10, 14, 12), C, 11) * 0.4
    y = ops.raymarch_grid_transform(cuda(x), M, V, P, F, (13, 9, 11), 'LINEAR', boundary, blend)
    ref = RM.raymarch_fwd(x, M, V, P, F, (13, 9, 11), OS.LINEAR, BOUNDS.index(boundary),
                          getattr(OB, blend))
    assert y.shape == ref.shape
    assert rel_l2(np_(y), ref) <= FWD_TOL


@pytest.mark.parametrize('filt', ['NEAREST', 'MIN', 'MAX'])
@pytest.mark.parametrize('boundary', ['CLAMP', 'WRAP'])
def test_raymarch_forward_filters(ops, filt, boundary):
    from oracle import raymarch as RM
    from oracle import blend as OB
    _, _, M, V, P, F = scene((10, 14, 12), 2, (13, 9, 11))
    x = small_grid((10, 14, 12), 4, 12) * 0.4
    y = ops.raymarch_grid_transform(cuda(x), M, V, P, F, (13, 9, 11), filt, boundary, 'ADDITIVE')
    ref = RM.raymarch_fwd(x, M, V, P, F, (13, 9, 11), ['NEAREST', 'LINEAR', 'MIN', 'MAX'].index(filt),
                          BOUNDS.index(boundary), OB.ADDITIVE)
    assert rel_l2(np_(y), ref) <= FWD_TOL


@pytest.mark.parametrize('C', [1, 4])
@pytest.mark.parametrize('blend', BLENDS)
@pytest.mark.parametrize('boundary', ['BORDER', 'CLAMP'])
@pytest.mark.parametrize('mode', ['REFERENCE', 'EXACT'])
def test_raymarch_backward(ops, C, blend, boundary, mode):
    from oracle import raymarch as RM
    from oracle import blend as OB
    _, _, M, V, P, F = scene((10, 14, 12), 3, (13, 9, 11))
    x = small_grid((10, 14, 12), C, 13) * 0.4
    rng = np.random.default_rng(14)
    dy = rng.standard_normal((1, 3, 9, 11, C)).astype(np.float32)
    xt = cuda(x).requires_grad_(True)
    with ops.grad_mode(mode):
        y = ops.raymarch_grid_transform(xt, M, V, P, F, (13, 9, 11), 'LINEAR', boundary, blend)
        y.backward(cuda(dy))
    ref = RM.raymarch_bwd(x, np_(y), dy, M, V, P, F, (13, 9, 11), BOUNDS.index(boundary),
                          getattr(OB, blend), exact=(mode == 'EXACT'))
    assert rel_l2(np_(xt.grad), ref) <= GRAD_TOL


@pytest.mark.parametrize('boundary', ['BORDER', 'CLAMP'])
def test_raymarch_backward_weights_on_side_stream(ops, boundary):
    """Autograd runs the reference-mode weight pass on a side stream during the
    forward; the gradient op called alone runs it inline: same gradient."""
    _, _, M, V, P, F = scene((10, 14, 12), 3, (13, 9, 11))
    x = small_grid((10, 14, 12), 4, 21) * 0.4
    dy = cuda(np.random.default_rng(22).standard_normal((1, 3, 9, 11, 4)).astype(np.float32))
    xt = cuda(x).requires_grad_(True)
    with ops.grad_mode('REFERENCE'):
        y = ops.raymarch_grid_transform(xt, M, V, P, F, (13, 9, 11), 'LINEAR', boundary)
        y.backward(dy)
        g_inline = ops.raymarch_grid_transform_grad(cuda(x), y.detach(), dy, M, V, P, F, (13, 9, 11), 'LINEAR',
                                                    boundary)
    assert rel_l2(np_(xt.grad), np_(g_inline)) <= 1e-6


def test_raymarch_backward_prefetched_weights(ops):
    """A weight pass prefetched for the same geometry is taken over by the next
    differentiable raymarch; a different geometry does not take it."""
    _, _, M, V, P, F = scene((10, 14, 12), 3, (13, 9, 11))
    x = small_grid((10, 14, 12), 4, 23) * 0.4
    dy = cuda(np.random.default_rng(24).standard_normal((1, 3, 9, 11, 4)).astype(np.float32))
    grads = []
    for prefetch in (False, True):
        xt = cuda(x).requires_grad_(True)
        with ops.grad_mode('REFERENCE'):
            if prefetch:
                ops.prefetch_raymarch_weights(x.shape, M, V, P, F, (13, 9, 11), device='cuda')
                assert len(ops._prefetched) == 1
            y = ops.raymarch_grid_transform(xt, M, V, P, F, (13, 9, 11))
            assert len(ops._prefetched) == 0
            y.backward(dy)
        grads.append(np_(xt.grad))
    assert rel_l2(grads[1], grads[0]) <= 1e-6
    ops.prefetch_raymarch_weights(x.shape, M, V, P, F, (13, 9, 12), device='cuda')
    with ops.grad_mode('REFERENCE'):
        ops.raymarch_grid_transform(cuda(x).requires_grad_(True), M, V, P, F, (13, 9, 11))
    assert len(ops._prefetched) == 1
    ops._prefetched.clear()


def test_raymarch_weight_cache_static_cameras(ops):
    """With the weight cache on, a repeated geometry reuses its weight sums (no
    new entry), changed cameras get their own entry, and every gradient matches
    the uncached one (float atomics: summation order only); a step captured in
    a CUDA graph after the entry exists replays to the same gradient."""
    _, _, M, V, P, F = scene((10, 14, 12), 3, (13, 9, 11))
    _, _, M2, V2, P2, F2 = scene((10, 14, 12), 3, (13, 9, 11), arc=120.0, tilt=20.0)
    x = small_grid((10, 14, 12), 4, 25) * 0.4
    dy = cuda(np.random.default_rng(26).standard_normal((1, 3, 9, 11, 4)).astype(np.float32))

    def grad(m, v, p, f):
        xt = cuda(x).requires_grad_(True)
        with ops.grad_mode('REFERENCE'):
            ops.raymarch_grid_transform(xt, m, v, p, f, (13, 9, 11)).backward(dy)
        return xt.grad.clone()

    base, base2 = grad(M, V, P, F), grad(M2, V2, P2, F2)
    ops.set_raymarch_weight_cache(True, max_entries=2)
    try:
        g1 = grad(M, V, P, F)
        assert len(ops._weight_cache['entries']) == 1
        g2 = grad(M, V, P, F)
        assert len(ops._weight_cache['entries']) == 1
        assert rel_l2(np_(g1), np_(base)) <= 1e-6 and rel_l2(np_(g2), np_(base)) <= 1e-6
        g3 = grad(M2, V2, P2, F2)
        assert len(ops._weight_cache['entries']) == 2 and rel_l2(np_(g3), np_(base2)) <= 1e-6
        xt = cuda(x).requires_grad_(True)
        s = torch.cuda.Stream()
        s.wait_stream(torch.cuda.current_stream())
        with torch.cuda.stream(s), ops.grad_mode('REFERENCE'):
            ops.raymarch_grid_transform(xt, M, V, P, F, (13, 9, 11)).backward(dy)
        torch.cuda.current_stream().wait_stream(s)
        xt.grad = None
        graph = torch.cuda.CUDAGraph()
        with torch.cuda.graph(graph), ops.grad_mode('REFERENCE'):
            ops.raymarch_grid_transform(xt, M, V, P, F, (13, 9, 11)).backward(dy)
        graph.replay()
        torch.cuda.synchronize()
        assert len(ops._weight_cache['entries']) == 2 and rel_l2(np_(xt.grad), np_(base)) <= 1e-6
    finally:
        ops.set_raymarch_weight_cache(False)
    assert len(ops._weight_cache['entries']) == 0


@pytest.mark.parametrize('C', [1, 4])
@pytest.mark.parametrize('blend', BLENDS)
@pytest.mark.parametrize('boundary', BOUNDS)
@pytest.mark.parametrize('mode', ['REFERENCE', 'EXACT'])
def test_raymarch_sample_store(ops, C, blend, boundary, mode):
    """The backward reading the samples the forward stored equals the backward
    re-sampling the grid, up to the rounding of the sample positions (forward
    front to back, adjoint back to front); the forward output is unchanged."""
    _, _, M, V, P, F = scene((10, 14, 12), 3, (13, 9, 11))
    x = small_grid((10, 14, 12), C, 27) * 0.4
    dy = cuda(np.random.default_rng(28).standard_normal((1, 3, 9, 11, C)).astype(np.float32))
    grads, outs = [], []
    for store in (False, True):
        ops.set_raymarch_sample_store(store)
        try:
            xt = cuda(x).requires_grad_(True)
            with ops.grad_mode(mode):
                y = ops.raymarch_grid_transform(xt, M, V, P, F, (13, 9, 11), 'LINEAR', boundary, blend)
                y.backward(dy)
        finally:
            ops.set_raymarch_sample_store(True)
        grads.append(np_(xt.grad))
        outs.append(np_(y))
    assert np.array_equal(outs[0], outs[1])
    assert rel_l2(grads[1], grads[0]) <= 1e-5


@pytest.mark.parametrize('boundary', BOUNDS)
@pytest.mark.parametrize('mode', ['REFERENCE', 'EXACT'])
def test_raymarch_sample_store_sparse_grid(ops, boundary, mode):
    """A grid that is zero outside a sub-box: the storing forward skips the
    samples of empty occupancy blocks (exactly zero), its output is identical
    to the plain forward's, it stores fewer samples than its rays take (none
    for an all-zero grid under BORDER and CLAMP, where the boundary samples are
    covered too), and the gradient equals the re-sampling one."""
    _, _, M, V, P, F = scene((12, 14, 13), 3, (13, 9, 11))
    x = small_grid((12, 14, 13), 4, 31) * 0.4
    x[:, :3] = 0.0
    x[:, 9:] = 0.0
    x[:, :, 10:] = 0.0
    x[:, :, :, :4] = 0.0
    dy = cuda(np.random.default_rng(32).standard_normal((1, 3, 9, 11, 4)).astype(np.float32))
    grads, outs = [], []
    for store in (False, True):
        ops.set_raymarch_sample_store(store)
        try:
            xt = cuda(x).requires_grad_(True)
            with ops.grad_mode(mode):
                y = ops.raymarch_grid_transform(xt, M, V, P, F, (13, 9, 11), 'LINEAR', boundary)
                y.backward(dy)
        finally:
            ops.set_raymarch_sample_store(True)
        grads.append(np_(xt.grad))
        outs.append(np_(y))
    assert np.array_equal(outs[0], outs[1])
    assert rel_l2(grads[1], grads[0]) <= 1e-5
    counts = []
    for grid in (x, np.zeros_like(x)):
        smp = ops._samples_buffer(grid.shape, 3, (13, 9, 11), True, 'cuda')
        ops._raymarch_fwd(cuda(grid), M, V, P, F, (13, 9, 11), 1, BOUNDS.index(boundary), 0, True, samples=smp)
        counts.append(ops.stored_sample_count(smp, grid.shape, 3, (13, 9, 11)))
    assert 0 < counts[0] < 3 * 9 * 11 * 13
    assert counts[1] == 0 if boundary != 'WRAP' else counts[1] < counts[0]


@pytest.mark.parametrize('C', [1, 4])
@pytest.mark.parametrize('blend', BLENDS)
@pytest.mark.parametrize('boundary', ['BORDER', 'CLAMP'])
@pytest.mark.parametrize('negative', [False, True])
def test_raymarch_empty_space_skipping(ops, C, blend, boundary, negative):
    """A 48x56x40 grid that is zero outside two small boxes, rays of 96
    samples: the storing forward steps over runs of samples its empty-space
    distance map proves zero (the positions come from the step index, so the
    samples it processes are the same); its images equal the plain forward's
    bit for bit, for every blend mode (also with negative values, where a zero
    sample still leaves the blend unchanged), and the gradient from the stored
    samples equals the re-sampling one."""
    shape, res = (48, 56, 40), (96, 40, 44)
    _, _, M, V, P, F = scene(shape, 3, res)
    x = np.zeros((1,) + shape + (C,), np.float32)
    x[:, 20:28, 24:33, 15:24] = small_grid((8, 9, 9), C, 41, positive=not negative)[0] * 0.4
    x[:, 40:44, 5:9, 30:35] = small_grid((4, 4, 5), C, 42, positive=not negative)[0] * 0.4
    dy = cuda(np.random.default_rng(43).standard_normal((1, 3) + res[1:] + (C,)).astype(np.float32))
    grads, outs = [], []
    for store in (False, True):
        ops.set_raymarch_sample_store(store)
        try:
            xt = cuda(x).requires_grad_(True)
            y = ops.raymarch_grid_transform(xt, M, V, P, F, res, 'LINEAR', boundary, blend)
            y.backward(dy)
        finally:
            ops.set_raymarch_sample_store(True)
        grads.append(np_(xt.grad))
        outs.append(np_(y))
    assert np.abs(outs[0]).max() > 0
    assert np.array_equal(outs[0], outs[1])
    assert rel_l2(grads[1], grads[0]) <= 1e-5
    smp = ops._samples_buffer(x.shape, 3, res, True, 'cuda')
    ops._raymarch_fwd(cuda(x), M, V, P, F, res, 1, BOUNDS.index(boundary), ops.BLEND[blend], True, samples=smp)
    n = ops.stored_sample_count(smp, x.shape, 3, res)
    assert 0 < n < 3 * 40 * 44 * 96 // 4


def test_raymarch_empty_space_distance_map(ops):
    """The distance map the storing forward builds next to the occupancy map
    (4^3-voxel blocks, one byte each, per input slice): the Chebyshev distance
    in blocks to the nearest occupied block, capped at 7, equal to a direct
    computation from the occupancy map the store holds."""
    shape, res = (52, 60, 44), (40, 30, 32)
    _, _, M, V, P, F = scene(shape, 2, res)
    x = np.zeros((2,) + shape + (4,), np.float32)
    x[0, 20:24, 30:35, 10:14] = 0.5
    x[0, 45:48, 2:5, 40:44] = 0.3
    x[1, 5:9, 50:55, 20:30] = 0.2
    M2 = np.stack([M[0], M[0]])
    smp = ops._samples_buffer(x.shape, 2, res, True, 'cuda')
    ops._raymarch_fwd(cuda(x), M2, V, P, F, res, 1, 0, 0, True, samples=smp)
    torch.cuda.synchronize()
    D, H, W = res
    cells = 2 * 2 * ((W + 7) // 8) * ((H + 15) // 16) * D * 128  # 2 slices x 2 views
    words = -(-4 * (cells // 32) // 256) * 256
    nb = tuple(-(-n // 4) for n in shape)
    nvox = int(np.prod(nb))
    part = -(-nvox * 2 // 256) * 256
    raw = smp.view(torch.uint8).cpu().numpy()
    occ = raw[256 + 2 * words:][:nvox * 2].reshape((2,) + nb)
    dist = raw[256 + 2 * words + part:][:nvox * 2].reshape((2,) + nb)
    assert occ.any() and not occ.all()
    for n in range(2):
        z, y, xx = np.nonzero(occ[n])
        grid = np.stack(np.meshgrid(*[np.arange(k) for k in nb], indexing='ij'), -1)
        pts = np.stack([z, y, xx], -1)
        cheb = np.abs(grid[..., None, :] - pts[None, None, None]).max(-1).min(-1)
        assert np.array_equal(dist[n], np.minimum(cheb, 7).astype(np.uint8))


@pytest.mark.parametrize('fraction', [0.0, 0.01, 1.0])
@pytest.mark.parametrize('mode', ['REFERENCE', 'EXACT'])
def test_raymarch_sample_store_pool_sizes(ops, fraction, mode):
    """A sample pool too small for the launch (none, about one chunk) or as
    large as every sample: the forward output is bit-identical, the samples
    that did not fit are re-sampled by the adjoint (gradient equal to the
    re-sampling one up to rounding), and the warps stop taking chunks at the
    pool's end."""
    _, _, M, V, P, F = scene((10, 14, 12), 3, (13, 9, 11))
    x = small_grid((10, 14, 12), 4, 35) * 0.4
    dy = cuda(np.random.default_rng(36).standard_normal((1, 3, 9, 11, 4)).astype(np.float32))
    grads, outs = [], []
    for store, frac in ((False, None), (True, fraction)):
        ops.set_raymarch_sample_store(store, pool_fraction=frac)
        try:
            xt = cuda(x).requires_grad_(True)
            with ops.grad_mode(mode):
                y = ops.raymarch_grid_transform(xt, M, V, P, F, (13, 9, 11))
                y.backward(dy)
        finally:
            ops.set_raymarch_sample_store(True, pool_fraction=0.25)
        grads.append(np_(xt.grad))
        outs.append(np_(y))
    assert np.array_equal(outs[0], outs[1])
    assert rel_l2(grads[1], grads[0]) <= 1e-5
    shape5 = (1, 10, 14, 12, 4)
    smp = ops._samples_buffer(shape5, 3, (13, 9, 11), True, 'cuda', pool_fraction=fraction)
    ops._raymarch_fwd(cuda(x), M, V, P, F, (13, 9, 11), 1, 0, 0, True, samples=smp)
    n = ops.stored_sample_count(smp, shape5, 3, (13, 9, 11))
    lib = ops._lib.load()
    args = (ops._lib.i64(shape5), 3, ops._lib.i32((13, 9, 11)), 1)
    cap = (smp.numel() - lib.gft_raymarch_grid_transform_samples_min_size(*args)) // 16
    taken = ops.sample_pool_cells(smp)
    assert n > 0
    if fraction == 1.0:
        assert n <= taken <= cap  # everything fit
    else:
        assert cap < n and taken >= cap - 256  # the pool ran full


def test_raymarch_sample_store_many_pairs(ops):
    """More (batch, camera) pairs than one launch table holds (2 x 9 = 18):
    the store offsets continue across the tables, and each batch slice skips
    by its own occupancy map."""
    _, _, M, V, P, F = scene((10, 14, 12), 9, (13, 9, 11))
    # two slices zero outside different boxes: each slice has its own occupancy
    x = np.zeros((2, 10, 14, 12, 4), np.float32)
    x[0, 1:5, 2:9, 6:12] = small_grid((4, 7, 6), 4, 29)[0] * 0.4
    x[1, 5:10, 7:14, 0:6] = small_grid((5, 7, 6), 4, 34)[0] * 0.4
    M2 = np.stack([M[0], M[0]]) if np.asarray(M).ndim == 3 else M
    dy = cuda(np.random.default_rng(30).standard_normal((2, 9, 9, 11, 4)).astype(np.float32))
    grads, outs = [], []
    for store in (False, True):
        ops.set_raymarch_sample_store(store)
        try:
            xt = cuda(x).requires_grad_(True)
            with ops.grad_mode('REFERENCE'):
                y = ops.raymarch_grid_transform(xt, M2, V, P, F, (13, 9, 11))
                y.backward(dy)
        finally:
            ops.set_raymarch_sample_store(True)
        grads.append(np_(xt.grad))
        outs.append(np_(y))
    assert np.array_equal(outs[0], outs[1])
    assert rel_l2(grads[1], grads[0]) <= 1e-5


def test_raymarch_not_separate_batch(ops):
    from oracle import raymarch as RM
    _, _, M, V, P, F = scene((8, 9, 7), 2, (9, 6, 5))
    x = np.concatenate([small_grid((8, 9, 7), 4, 1), small_grid((8, 9, 7), 4, 2)], 0) * 0.3
    M2 = np.concatenate([M, M], 0)
    y = ops.raymarch_grid_transform(cuda(x), M2, V, P, F, (9, 6, 5), separate_camera_batch=False)
    ref = RM.raymarch_fwd(x, M2, V, P, F, (9, 6, 5), separate_camera_batch=False)
    assert y.shape == (2, 1, 6, 5, 4)
    assert rel_l2(np_(y), ref) <= FWD_TOL


def test_raymarch_bf16_storage(ops):
    from oracle import raymarch as RM
    _, _, M, V, P, F = scene((10, 14, 12), 2, (13, 9, 11))
    x = small_grid((10, 14, 12), 4, 15) * 0.4
    y = ops.raymarch_grid_transform(cuda(x), M, V, P, F, (13, 9, 11), storage_dtype=torch.bfloat16)
    ref = RM.raymarch_fwd(x, M, V, P, F, (13, 9, 11))
    assert rel_l2(np_(y), ref) <= BF16_TOL


# ------------------------------------------------------------------ SampleGridLut
@pytest.mark.parametrize('C', [1, 2, 4])
@pytest.mark.parametrize('filt', ['NEAREST', 'LINEAR', 'MIN', 'MAX'])
@pytest.mark.parametrize('boundary', BOUNDS)
def test_lut_forward(ops, C, filt, boundary):
    from oracle import resample as R
    rng = np.random.default_rng(20)
    x = small_grid((8, 9, 7), C, 21)
    lut = np.concatenate([rng.standard_normal((2, 6, 5, 4, 3)) * 2.0, np.zeros((2, 6, 5, 4, 1))], -1).astype(np.float32)
    y = ops.sample_grid_lut(cuda(x), cuda(lut), filt, boundary)
    ref = R.sample_grid_lut(x, lut, ['NEAREST', 'LINEAR', 'MIN', 'MAX'].index(filt), BOUNDS.index(boundary))
    assert y.shape == ref.shape
    assert rel_l2(np_(y), ref) <= FWD_TOL


@pytest.mark.parametrize('mip', ['NEAREST', 'LINEAR'])
@pytest.mark.parametrize('boundary', ['BORDER', 'CLAMP'])
def test_lut_forward_mips(ops, mip, boundary):
    from oracle import resample as R
    from oracle import sampling as OS
    rng = np.random.default_rng(22)
    x = small_grid((16, 18, 14), 2, 23)
    lut = np.concatenate([rng.random((1, 7, 6, 5, 3)) * [14, 18, 16], rng.random((1, 7, 6, 5, 1)) * 3.5],
                         -1).astype(np.float32)
    y = ops.sample_grid_lut(cuda(x), cuda(lut), 'LINEAR', boundary, mip, 3, 0.25, relative_coords=False,
                            cell_center_offset=0.5)
    ref = R.sample_grid_lut(x, lut, OS.LINEAR, BOUNDS.index(boundary), ['NONE', 'NEAREST', 'LINEAR'].index(mip), 3,
                            0.25, 0.5, relative=False)
    assert rel_l2(np_(y), ref) <= FWD_TOL


@pytest.mark.parametrize('C', [1, 4])
@pytest.mark.parametrize('filt', ['LINEAR', 'NEAREST'])
@pytest.mark.parametrize('boundary', BOUNDS)
@pytest.mark.parametrize('mode', ['REFERENCE', 'EXACT'])
def test_lut_backward(ops, C, filt, boundary, mode):
    from oracle import resample as R
    rng = np.random.default_rng(24)
    x = small_grid((8, 9, 7), C, 25)
    lut = np.concatenate([rng.standard_normal((2, 8, 9, 7, 3)) * 1.5, np.zeros((2, 8, 9, 7, 1))], -1).astype(np.float32)
    dy = rng.standard_normal((1, 2, 8, 9, 7, C)).astype(np.float32)
    xt = cuda(x).requires_grad_(True)
    lt = cuda(lut).requires_grad_(True)
    with ops.grad_mode(mode):
        y = ops.sample_grid_lut(xt, lt, filt, boundary)
        y.backward(cuda(dy))
    gx, gl = R.sample_grid_lut_grad(x, dy, lut, ['NEAREST', 'LINEAR'].index(filt), BOUNDS.index(boundary),
                                    exact=(mode == 'EXACT'))
    assert rel_l2(np_(xt.grad), gx) <= GRAD_TOL
    if filt == 'LINEAR':
        assert rel_l2(np_(lt.grad), gl) <= GRAD_TOL
    else:
        assert np.all(np_(lt.grad) == 0)


# ------------------------------------------------------------------ SampleGridTransform
CMS = ['TRANSFORM_LINDEPTH', 'TRANSFORM_LINDEPTH_REVERSE', 'TRANSFORM', 'TRANSFORM_REVERSE']


def _transform_case(cm):
    from oracle import transforms as OT
    shape, res = (10, 14, 12), (13, 9, 11)
    _, _, M, V, P, F = scene(shape, 2, res)
    if cm in ('TRANSFORM_LINDEPTH_REVERSE', 'TRANSFORM_REVERSE'):
        in_shape, out_shape = res, shape
    else:
        in_shape, out_shape = shape, res
    return M, V, P, F, in_shape, out_shape, [OT.LINDEPTH, OT.LINDEPTH_REVERSE, OT.TRANSFORM, OT.TRANSFORM_REVERSE][CMS.index(cm)]


@pytest.mark.parametrize('cm', CMS)
@pytest.mark.parametrize('filt', ['NEAREST', 'LINEAR'])
@pytest.mark.parametrize('boundary', ['BORDER', 'CLAMP'])
@pytest.mark.parametrize('mip', ['NONE', 'NEAREST', 'LINEAR'])
def test_sample_transform_forward(ops, cm, filt, boundary, mip):
    from oracle import resample as R
    M, V, P, F, in_shape, out_shape, ocm = _transform_case(cm)
    x = small_grid(in_shape, 2, 30)
    y = ops.sample_grid_transform(cuda(x), M, V, P, F, out_shape, filt, boundary, mip, 2 if mip != 'NONE' else 0,
                                  0.3, cm)
    ref = R.sample_grid_transform(x, M, V, P, F, out_shape, ['NEAREST', 'LINEAR'].index(filt),
                                  ['BORDER', 'CLAMP'].index(boundary), ['NONE', 'NEAREST', 'LINEAR'].index(mip),
                                  2 if mip != 'NONE' else 0, 0.3, ocm)
    assert y.shape == ref.shape
    if filt == 'NEAREST' or mip == 'NEAREST':
        # Nearest cell / nearest level are step functions of the position: cells whose
        # fp32 position sits on a rounding tie may pick the neighbour the fp64 oracle
        # does not.  Bound the fraction of such cells; all others must agree.
        bad = np.any(np.abs(np_(y) - ref) > 1e-5, axis=-1)
        assert bad.mean() <= 0.02
        assert rel_l2(np_(y)[~bad], ref[~bad]) <= FWD_TOL
    else:
        assert rel_l2(np_(y), ref) <= FWD_TOL


@pytest.mark.parametrize('cm', ['TRANSFORM_LINDEPTH', 'TRANSFORM'])
@pytest.mark.parametrize('filt', ['NEAREST', 'LINEAR'])
@pytest.mark.parametrize('boundary', ['BORDER', 'CLAMP'])
@pytest.mark.parametrize('mip', ['NEAREST', 'LINEAR'])
@pytest.mark.parametrize('N', [1, 2])
def test_sample_transform_sparse_volume(ops, cm, filt, boundary, mip, N):
    """A volume that is zero outside a small box (volume -> frustum with mips):
    samples reading only zeros at every level, by the occupancy map of 8^3-voxel
    blocks grown by the mip footprint, skip their LOD and fetches; the result
    still matches the oracle."""
    from oracle import resample as R
    from oracle import transforms as OT
    shape, res = (96, 100, 96), (24, 30, 32)  # 12x13x12 blocks, the box in blocks 5-8
    _, _, M, V, P, F = scene(shape, 2, res)
    x = np.zeros((N,) + shape + (1,), np.float32)
    x[0, 40:64, 40:66, 40:64] = small_grid((24, 26, 24), 1, 33)[0]
    if N == 2:  # another box: each slice has its own occupancy map
        x[1, 10:30, 60:90, 50:80] = small_grid((20, 30, 30), 1, 35)[0]
        M = np.stack([M[0], M[0]])
    ocm = OT.LINDEPTH if cm == 'TRANSFORM_LINDEPTH' else OT.TRANSFORM
    y = ops.sample_grid_transform(cuda(x), M, V, P, F, res, filt, boundary, mip, 2, 0.3, cm)
    ref = R.sample_grid_transform(x, M, V, P, F, res, ['NEAREST', 'LINEAR'].index(filt),
                                  ['BORDER', 'CLAMP'].index(boundary), ['NONE', 'NEAREST', 'LINEAR'].index(mip), 2,
                                  0.3, ocm)
    assert np.abs(ref).max() > 0 and (ref == 0).mean() > 0.3
    if filt == 'NEAREST' or mip == 'NEAREST':
        bad = np.any(np.abs(np_(y) - ref) > 1e-5, axis=-1)
        assert bad.mean() <= 0.02
        assert rel_l2(np_(y)[~bad], ref[~bad]) <= FWD_TOL
    else:
        assert rel_l2(np_(y), ref) <= FWD_TOL


@pytest.mark.parametrize('cm', ['TRANSFORM_LINDEPTH_REVERSE', 'TRANSFORM_REVERSE'])
@pytest.mark.parametrize('frustum', ['coarse', 'fine'])
def test_sample_transform_reverse_lod_bound(ops, cm, frustum):
    """Frustum -> volume with mips and no bias: where every voxel step spans
    less than one frustum cell (a coarse frustum) the LOD is 0 for every
    sample and the launch may skip it; where some steps span more (a fine
    frustum) it must be computed.  Both match the oracle over the whole
    output, and the oracle's LOD range confirms which case each one is."""
    from oracle import resample as R
    from oracle import transforms as OT
    shape = (24, 28, 24)
    res = (8, 8, 8) if frustum == 'coarse' else (48, 56, 56)
    _, _, M, V, P, F = scene(shape, 2, res)
    ocm = OT.LINDEPTH_REVERSE if cm == 'TRANSFORM_LINDEPTH_REVERSE' else OT.TRANSFORM_REVERSE
    x = small_grid(res, 1, 36)
    y = ops.sample_grid_transform(cuda(x), M, V, P, F, shape, 'LINEAR', 'BORDER', 'LINEAR', 2, 0.0, cm)
    ref = R.sample_grid_transform(x, M, V, P, F, shape, 1, 0, 2, 2, 0.0, ocm)
    idx = np.stack(np.meshgrid(*[np.arange(n) + 0.5 for n in shape], indexing='ij'), -1)[..., ::-1]
    lods = [OT.sample_positions(OT.CameraXform(M[0], V[c], P[c], F[c]), ocm, idx, np.array(res[::-1]),
                                np.array(shape[::-1]), True)[..., 3].max() for c in range(2)]
    if frustum == 'coarse':
        assert max(lods) == 0.0
    else:
        assert max(lods) > 0.5
    assert np.abs(ref).max() > 0
    assert rel_l2(np_(y), ref) <= FWD_TOL


@pytest.mark.parametrize('mip', ['NEAREST', 'LINEAR'])
def test_sample_transform_dense_input_flag(ops, mip):
    """dense_input (GFT_SAMPLE_DENSE) only leaves out the occupancy map: the
    result is bit-identical, for a sparse volume too."""
    shape, res = (96, 100, 96), (24, 30, 32)
    _, _, M, V, P, F = scene(shape, 2, res)
    x = np.zeros((1,) + shape + (1,), np.float32)
    x[0, 40:64, 40:66, 40:64] = small_grid((24, 26, 24), 1, 37)[0]
    outs = [ops.sample_grid_transform(cuda(x), M, V, P, F, res, 'LINEAR', 'BORDER', mip, 2, 0.3,
                                      'TRANSFORM_LINDEPTH', dense_input=dense) for dense in (False, True)]
    assert np.abs(np_(outs[0])).max() > 0
    assert torch.equal(outs[0], outs[1])


@pytest.mark.parametrize('cm', CMS)
@pytest.mark.parametrize('boundary', BOUNDS)
@pytest.mark.parametrize('mode', ['REFERENCE', 'EXACT'])
def test_sample_transform_backward(ops, cm, boundary, mode):
    from oracle import resample as R
    M, V, P, F, in_shape, out_shape, ocm = _transform_case(cm)
    x = small_grid(in_shape, 4, 31)
    rng = np.random.default_rng(32)
    dy = rng.standard_normal((1, 2) + tuple(out_shape) + (4,)).astype(np.float32)
    with ops.grad_mode(mode):
        g = ops.sample_grid_transform_grad(cuda(x), cuda(dy), M, V, P, F, 'LINEAR', boundary,
                                           coordinate_mode=cm)
    ref = R.sample_grid_transform_grad(x, dy, M, V, P, F, BOUNDS.index(boundary), ocm, exact=(mode == 'EXACT'))
    assert rel_l2(np_(g), ref) <= GRAD_TOL


def test_lod_transform(ops):
    from oracle import resample as R
    _, cams, M, V, P, F = scene((10, 14, 12), 2, (13, 9, 11))
    MV = np.stack([M[0] @ V[i] for i in range(2)]).astype(np.float32)  # (V @ M)^T
    for inv in (False, True):
        ins, outs = ((10, 14, 12), (13, 9, 11)) if not inv else ((13, 9, 11), (10, 14, 12))
        y = ops.lod_transform(ins, MV, P, F, outs, inv)
        ref = R.lod_transform(ins, MV, P, F, outs, inv)
        assert rel_l2(np_(y), ref) <= FWD_TOL


# ------------------------------------------------------------------ ReduceGridBlend
@pytest.mark.parametrize('C', [1, 2, 4])
@pytest.mark.parametrize('blend', BLENDS)
@pytest.mark.parametrize('keep', [False, True])
def test_blend(ops, C, blend, keep):
    from oracle import blend as OB
    x = small_grid((9, 7, 6), C, 40) * 0.3
    y = ops.reduce_grid_blend(cuda(x), blend, keep)
    ref = OB.reduce_grid_blend(x, getattr(OB, blend), keep)
    assert rel_l2(np_(y), ref) <= FWD_TOL
    if blend == 'ALPHA_ADDITIVE':
        return
    rng = np.random.default_rng(41)
    dy = rng.standard_normal(ref.shape).astype(np.float32)
    for mode in ('REFERENCE', 'EXACT'):
        with ops.grad_mode(mode):
            g = ops.reduce_grid_blend_grad(cuda(dy), y, cuda(x), blend, keep)
        gref = OB.reduce_grid_blend_grad(dy, np_(y), x, getattr(OB, blend), keep, exact=(mode == 'EXACT'))
        assert rel_l2(np_(g), gref) <= GRAD_TOL


# ------------------------------------------------------------------ advection
@pytest.mark.parametrize('order,clamp', [(1, 'NONE'), (2, 'NONE'), (2, 'MC_SMOOTH'), (1, 'NEGATIVE'), (2, 'NEGATIVE')])
@pytest.mark.parametrize('boundary', BOUNDS)
@pytest.mark.parametrize('mode', ['REFERENCE', 'EXACT'])
def test_advect(ops, order, clamp, boundary, mode, shape=(9, 10, 8)):
    from oracle import advect as OA
    rng = np.random.default_rng(50)
    D, H, W = shape
    d = small_grid((D, H, W), 1, 51, positive=(clamp != 'NEGATIVE'))
    vx = (rng.standard_normal((1, D, H, W + 1, 1)) * 0.8).astype(np.float32)
    vy = (rng.standard_normal((1, D, H + 1, W, 1)) * 0.8).astype(np.float32)
    vz = (rng.standard_normal((1, D + 1, H, W, 1)) * 0.8).astype(np.float32)
    dt = 1.3
    bi = BOUNDS.index(boundary)
    dtn = cuda(d).requires_grad_(True)
    vs = [cuda(v).requires_grad_(True) for v in (vx, vy, vz)]
    with ops.grad_mode(mode):
        y = ops.advect(dtn, *vs, dt=dt, order=order, clamp=clamp, boundary=boundary)
        go = rng.standard_normal(d.shape).astype(np.float32)
        y.backward(cuda(go))
    ref = OA.warp(d[0], vx[0], vy[0], vz[0], dt, order, clamp, bi)
    assert rel_l2(np_(y)[0], ref) <= FWD_TOL
    gd, gvx, gvy, gvz = OA.warp_grad(d[0], vx[0], vy[0], vz[0], go[0], dt, order, clamp, bi, exact=(mode == 'EXACT'))
    assert rel_l2(np_(dtn.grad)[0], gd) <= GRAD_TOL
    for got, want in zip(vs, (gvx, gvy, gvz)):
        assert rel_l2(np_(got.grad)[0], want) <= GRAD_TOL


@pytest.mark.parametrize('order', [1, 2])
@pytest.mark.parametrize('boundary', BOUNDS)
def test_advect_odd_voxel_count(ops, order, boundary):
    """An odd number of voxels: the single-channel reference-mode adjoint pads
    its packed (sum, count) regions to even offsets."""
    test_advect(ops, order, 'MC_SMOOTH' if order == 2 else 'NONE', boundary, 'REFERENCE', shape=(9, 11, 7))


@pytest.mark.parametrize('C', [1, 4])
@pytest.mark.parametrize('field', ['smooth', 'integer'])
@pytest.mark.parametrize('boundary', BOUNDS)
@pytest.mark.parametrize('mode', ['REFERENCE', 'EXACT'])
def test_advect_merged_scatter(ops, C, field, boundary, mode):
    """The adjoint scatters merge the corners that consecutive voxels along x
    share: a smooth field (lookups one cell apart, nearly every lane merges)
    and an integer one (lookups on cell corners, where the ceil corner is the
    floor corner and counts 2).  Rows of 45 voxels cross the warps, the last
    block is partial, and two density slices share the velocity (the first
    slice writes the lookup gradient, the second adds to it)."""
    from oracle import advect as OA
    D, H, W = 5, 6, 45
    rng = np.random.default_rng(60 + C)
    d = np.stack([small_grid((D, H, W), C, 61 + C)[0], small_grid((D, H, W), C, 62 + C)[0]])
    if field == 'smooth':
        def comp(shape, base):
            z, y, x = np.meshgrid(*[np.arange(n, dtype=np.float64) for n in shape], indexing='ij')
            return (base + 0.05 * np.sin(0.3 * x + 0.2 * y + 0.1 * z)).astype(np.float32)[None, ..., None]
        vx, vy, vz = comp((D, H, W + 1), 0.37), comp((D, H + 1, W), -0.21), comp((D + 1, H, W), 0.13)
        dt = 1.3
    else:
        vx = np.full((1, D, H, W + 1, 1), 1.0, np.float32)
        vy = np.full((1, D, H + 1, W, 1), -1.0, np.float32)
        vz = np.zeros((1, D + 1, H, W, 1), np.float32)
        dt = 1.0
    bi = BOUNDS.index(boundary)
    dtn = cuda(d).requires_grad_(True)
    vs = [cuda(v).requires_grad_(True) for v in (vx, vy, vz)]
    go = rng.standard_normal(d.shape).astype(np.float32)
    with ops.grad_mode(mode):
        y = ops.advect(dtn, *vs, dt=dt, order=2, clamp='MC_SMOOTH', boundary=boundary)
        y.backward(cuda(go))
    gv_want = [np.zeros(v.shape[1:]) for v in (vx, vy, vz)]
    for n in range(2):
        ref = OA.warp(d[n], vx[0], vy[0], vz[0], dt, 2, 'MC_SMOOTH', bi)
        assert rel_l2(np_(y)[n], ref) <= FWD_TOL
        gd, *gv = OA.warp_grad(d[n], vx[0], vy[0], vz[0], go[n], dt, 2, 'MC_SMOOTH', bi, exact=(mode == 'EXACT'))
        assert rel_l2(np_(dtn.grad)[n], gd) <= GRAD_TOL
        for acc, g in zip(gv_want, gv):
            acc += g
    for got, want in zip(vs, gv_want):
        assert rel_l2(np_(got.grad)[0], want) <= GRAD_TOL


# ------------------------------------------------------------------ raymarch, uneven camera batches
UNEVEN = [(13, 9, 11), (7, 6, 5), (11, 12, 16)]  # (depth samples, height, width) per camera


def test_advect_backward_reuses_forward_intermediate(ops):
    """MacCormack on one fp32 slice: autograd runs the forward in the gradient
    workspace and the backward reads its semi-Lagrangian grid
    (GFT_GRAD_FORWARD_READY); the gradients equal those of a backward that
    recomputes it (float atomics: summation order only)."""
    from gft import synthetic as syn
    shape = (10, 12, 9)
    d = cuda(syn.plume_density(shape, 31))
    vx, vy, vz = (cuda(v) for v in syn.curl_velocity(shape, 32))
    dy = cuda(np.random.default_rng(33).standard_normal((1,) + shape + (1,)).astype(np.float32))
    for mode in ('REFERENCE', 'EXACT'):
        ts = [t.clone().requires_grad_(True) for t in (d, vx, vy, vz)]
        with ops.grad_mode(mode):
            y = ops.advect(*ts, dt=1.0, order=2, clamp='MC_SMOOTH', boundary='CLAMP')
            y.backward(dy)
            ref = ops._advect_bwd(d, vx, vy, vz, dy, 1.0, 2, ops.CLAMP['MC_SMOOTH'], ops.BOUNDARY['CLAMP'],
                                  ops.GRAD[mode])
        for t, r in zip(ts, ref):
            assert rel_l2(np_(t.grad).reshape(-1), np_(r).reshape(-1)) <= 1e-6


def _uneven_scene(C, seed, batch=1):
    _, _, M, V, P, F = scene((10, 14, 12), 3, (13, 9, 11))
    x = np.concatenate([small_grid((10, 14, 12), C, seed + b) for b in range(batch)], 0) * 0.4
    return x, np.concatenate([M] * batch, 0), V, P, F


@pytest.mark.parametrize('C', [1, 2, 4])
@pytest.mark.parametrize('boundary', ['BORDER', 'CLAMP'])
@pytest.mark.parametrize('batch', [1, 2])
def test_raymarch_multi_forward_equals_per_camera(ops, C, boundary, batch):
    x, M, V, P, F = _uneven_scene(C, 31, batch)
    imgs = ops.raymarch_grid_transform_multi(cuda(x), M, V, P, F, UNEVEN, 'LINEAR', boundary)
    for c, shp in enumerate(UNEVEN):
        one = ops.raymarch_grid_transform(cuda(x), M, V[c:c + 1], P[c:c + 1], F[c:c + 1], shp, 'LINEAR', boundary)
        assert imgs[c].shape == (batch, shp[1], shp[2], C)
        assert torch.equal(imgs[c], one[:, 0])


def test_raymarch_multi_forward_oracle(ops):
    from oracle import raymarch as RM
    x, M, V, P, F = _uneven_scene(4, 35)
    imgs = ops.raymarch_grid_transform_multi(cuda(x), M, V, P, F, UNEVEN)
    for c, shp in enumerate(UNEVEN):
        ref = RM.raymarch_fwd(x, M, V[c:c + 1], P[c:c + 1], F[c:c + 1], shp)
        assert rel_l2(np_(imgs[c]), ref[:, 0]) <= FWD_TOL


@pytest.mark.parametrize('mode', ['REFERENCE', 'EXACT'])
@pytest.mark.parametrize('C', [1, 4])
def test_raymarch_multi_backward_equals_sum_over_cameras(ops, mode, C):
    x, M, V, P, F = _uneven_scene(C, 41)
    rng = np.random.default_rng(42)
    dys = [cuda(rng.standard_normal((1, h, w, C)).astype(np.float32)) for _, h, w in UNEVEN]
    with ops.grad_mode(mode):
        xt = cuda(x).requires_grad_(True)
        imgs = ops.raymarch_grid_transform_multi(xt, M, V, P, F, UNEVEN)
        sum((im * dy).sum() for im, dy in zip(imgs, dys)).backward()
        g_sum = torch.zeros_like(xt)
        for c, shp in enumerate(UNEVEN):
            xc = cuda(x).requires_grad_(True)
            one = ops.raymarch_grid_transform(xc, M, V[c:c + 1], P[c:c + 1], F[c:c + 1], shp)
            one.backward(dys[c][:, None])
            g_sum += xc.grad
    assert rel_l2(np_(xt.grad), np_(g_sum)) <= 1e-5


def test_raymarch_multi_argument_errors(ops):
    from gft import _lib
    x, M, V, P, F = _uneven_scene(4, 43)
    with pytest.raises(_lib.GftInvalidArgument):
        ops.raymarch_grid_transform_multi(cuda(x), M, V, P, F, UNEVEN[:2])
    with pytest.raises(_lib.GftInvalidArgument):
        ops.raymarch_grid_transform_multi(cuda(x), M, V, P, F, [(13, 9, 11), (7, 0, 5), (11, 12, 16)])


# ------------------------------------------------------------------ raymarch, views bound to batch slices
def _views_scene(C, seed, frames=3, per_frame=6):
    """frames batch slices, each seen by its own per_frame cameras of uneven
    image sizes (18 views: two launches of up to 16)."""
    from gft import synthetic as syn
    _, _, M, _, _, _ = scene((10, 14, 12), 1, (13, 9, 11))
    x = np.concatenate([small_grid((10, 14, 12), C, seed + b) for b in range(frames)], 0) * 0.4
    Vs, Ps, Fs, shapes, cb = [], [], [], [], []
    for f in range(frames):
        cams, shp = syn.hemisphere_cameras(per_frame - 1, 11, sizes=(5, 13), radius=2.0, fov=40.0, seed=seed + 10 * f,
                                           fixed_size=9)
        V, P, F = syn.camera_params(cams)
        Vs.append(V), Ps.append(P), Fs.append(F)
        shapes += [list(s) for s in shp]
        cb += [f] * per_frame
    return x, np.concatenate([M] * frames, 0), np.concatenate(Vs), np.concatenate(Ps), np.concatenate(Fs), cb, shapes


@pytest.mark.parametrize('C', [1, 4])
def test_raymarch_views_forward_equals_per_camera(ops, C):
    x, M, V, P, F, cb, shapes = _views_scene(C, 51)
    y = ops.raymarch_grid_transform_views(cuda(x), cb, M, V, P, F, shapes)
    imgs = ops.views_split(y, shapes)
    for c, (b, shp) in enumerate(zip(cb, shapes)):
        one = ops.raymarch_grid_transform(cuda(x[b:b + 1]), M[b:b + 1], V[c:c + 1], P[c:c + 1], F[c:c + 1], shp)
        assert torch.equal(imgs[c], one[0, 0])


@pytest.mark.parametrize('mode', ['REFERENCE', 'EXACT'])
def test_raymarch_views_backward_equals_per_camera_sum(ops, mode):
    x, M, V, P, F, cb, shapes = _views_scene(4, 53)
    rng = np.random.default_rng(54)
    dys = [cuda(rng.standard_normal((h, w, 4)).astype(np.float32)) for _, h, w in shapes]
    with ops.grad_mode(mode):
        xt = cuda(x).requires_grad_(True)
        y = ops.raymarch_grid_transform_views(xt, cb, M, V, P, F, shapes)
        (y * torch.cat([d.reshape(-1, 4) for d in dys])).sum().backward()
        g = torch.zeros_like(xt)
        for c, (b, shp) in enumerate(zip(cb, shapes)):
            xc = cuda(x[b:b + 1]).requires_grad_(True)
            one = ops.raymarch_grid_transform(xc, M[b:b + 1], V[c:c + 1], P[c:c + 1], F[c:c + 1], shp)
            one.backward(dys[c][None, None])
            g[b:b + 1] += xc.grad
    assert rel_l2(np_(xt.grad), np_(g)) <= 1e-5


def test_raymarch_views_oracle_and_errors(ops):
    from gft import _lib
    from oracle import raymarch as RM
    x, M, V, P, F, cb, shapes = _views_scene(4, 57, frames=2, per_frame=3)
    y = ops.views_split(ops.raymarch_grid_transform_views(cuda(x), cb, M, V, P, F, shapes), shapes)
    for c, (b, shp) in enumerate(zip(cb, shapes)):
        ref = RM.raymarch_fwd(x[b:b + 1], M[b:b + 1], V[c:c + 1], P[c:c + 1], F[c:c + 1], shp)
        assert rel_l2(np_(y[c]), ref[0, 0]) <= FWD_TOL
    with pytest.raises(_lib.GftInvalidArgument):
        ops.raymarch_grid_transform_views(cuda(x), [0, 1, 2, 0, 1, 1], M, V, P, F, shapes)  # slice 2 of 2
    with pytest.raises(_lib.GftInvalidArgument):
        ops.raymarch_grid_transform_views(cuda(x), cb[:-1], M, V, P, F, shapes)


# ------------------------------------------------------------------ raymarch, brick layout
@pytest.mark.parametrize('C', [1, 2, 4])
@pytest.mark.parametrize('boundary', ['BORDER', 'CLAMP', 'WRAP'])
@pytest.mark.parametrize('mode', ['REFERENCE', 'EXACT'])
@pytest.mark.parametrize('sparse', [False, True])
def test_raymarch_bricked_equals_rows(ops, C, boundary, mode, sparse):
    """Odd grid sizes (padded bricks), forward bit-identical, gradient in the
    brick layout equal to the row gradient; sparse: zero outside a box whose
    faces cut through bricks, so the sample store's occupancy map of the
    bricked grid (built per brick) and of the row grid (per voxel) differ."""
    _, _, M, V, P, F = scene((9, 13, 11), 3, (13, 9, 11))
    x = small_grid((9, 13, 11), C, 51) * 0.4
    if sparse:
        box = np.zeros_like(x)
        box[:, 3:8, 5:10, 1:6] = x[:, 3:8, 5:10, 1:6]
        x = box
    dy = cuda(np.random.default_rng(52).standard_normal((1, 3, 9, 11, C)).astype(np.float32))
    xr = cuda(x).requires_grad_(True)
    xb = ops.to_bricks(cuda(x)).requires_grad_(True)
    assert torch.equal(ops.from_bricks(xb.detach(), (9, 13, 11)), xr.detach())
    with ops.grad_mode(mode):
        yr = ops.raymarch_grid_transform(xr, M, V, P, F, (13, 9, 11), 'LINEAR', boundary)
        yb = ops.raymarch_grid_transform_bricked(xb, (9, 13, 11), M, V, P, F, (13, 9, 11), boundary)
        assert torch.equal(yr, yb)
        yr.backward(dy)
        yb.backward(dy)
    assert rel_l2(np_(ops.from_bricks(xb.grad, (9, 13, 11))), np_(xr.grad)) <= 1e-6


def test_light_compose_bricked(ops):
    from gft import fused
    g = torch.Generator().manual_seed(6)
    D, H, W = 7, 10, 5
    d0 = torch.rand((1, D, H, W, 1), generator=g).cuda()
    t0 = torch.rand((1, D, H, W, 1), generator=g).cuda()
    col = torch.rand((1, D, H, W, 3), generator=g).cuda()
    gb = torch.randn((1, ops.brick_cells((D, H, W)), 4), generator=g).cuda()
    d1, t1 = d0.clone().requires_grad_(True), t0.clone().requires_grad_(True)
    yb = fused.light_compose(d1, t1, col, 0.64, 0.37, brick=True)
    d2, t2 = d0.clone().requires_grad_(True), t0.clone().requires_grad_(True)
    yr = fused.light_compose(d2, t2, col, 0.64, 0.37)
    assert torch.equal(ops.from_bricks(yb.detach(), (D, H, W)), yr.detach())
    yb.backward(gb)
    yr.backward(ops.from_bricks(gb, (D, H, W)))
    assert torch.equal(d1.grad, d2.grad) and torch.equal(t1.grad, t2.grad)
