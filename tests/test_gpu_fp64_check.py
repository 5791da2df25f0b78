"""The FP64 check step on the GPU (gft_transmittance_check,
gft_raymarch_check): the deviations it reports equal the deviations of the
FP32 results from the FP64 oracle's recomputation of the same FP32 inputs, and
the check runs inside the captured step."""
import numpy as np
import pytest
import torch

from scene_utils import scene, small_grid

pytestmark = pytest.mark.gpu


@pytest.fixture(scope='module')
def mods():
    if not torch.cuda.is_available():
        pytest.skip('no CUDA device')
    from gft import fused, ops
    return fused, ops


def _errors(got, ref):
    """(max |got - ref|, max |ref|)"""
    got = np.asarray(got, dtype=np.float64)
    ref = np.asarray(ref, dtype=np.float64)
    return float(np.abs(got - ref).max()), float(np.abs(ref).max())


def _close(a, b):
    return abs(a - b) <= 1e-6 * max(abs(b), 1e-300)


@pytest.mark.parametrize('stride', [1, 3])
def test_transmittance_check_equals_fp64_deviation(mods, stride):
    fused, _ = mods
    rng = np.random.default_rng(3)
    x = (rng.random((2, 96, 17, 13, 1)) * 0.2).astype(np.float32)
    xt = torch.from_numpy(x).cuda()
    tr = fused.transmittance(xt)
    res = fused.transmittance_check(xt, tr, stride).cpu().numpy()
    excl = np.concatenate([np.zeros_like(x[:, :1], dtype=np.float64), np.cumsum(x.astype(np.float64), axis=1)[:, :-1]],
                          axis=1)
    ref = np.exp(-excl)
    cols = np.arange(17 * 13 * 2) % stride == 0
    got = tr.cpu().numpy().astype(np.float64)
    sel = lambda a: np.moveaxis(a[..., 0], 1, -1).reshape(-1, a.shape[1])[cols]  # [columns, D]
    ea, rm = _errors(sel(got), sel(ref))
    assert ea > 0 and _close(res[0], ea) and _close(res[1], rm)
    assert res[0] / res[1] < 1e-5


@pytest.mark.parametrize('brick,dtype', [(False, torch.float32), (True, torch.float32), (True, torch.bfloat16)])
def test_raymarch_check_equals_fp64_deviation(mods, brick, dtype):
    _, ops = mods
    from oracle import raymarch as RM
    shape, res = (20, 24, 18), (40, 21, 23)
    _, _, M, V, P, F = scene(shape, 3, res)
    x = small_grid(shape, 4, 5) * 0.3
    xt = torch.from_numpy(x).cuda().to(dtype)
    xs = xt.float().cpu().numpy().astype(np.float64)  # the values the kernel reads
    if brick:
        xb = ops.to_bricks(xt.float().contiguous()).to(dtype)
        y = ops.raymarch_grid_transform_bricked(xb, shape, M, V, P, F, res)
        got = ops.raymarch_check(xb, M, V, P, F, res, y, 1, grid_shape=shape).cpu().numpy()
    else:
        y = ops.raymarch_grid_transform(xt, M, V, P, F, res)
        got = ops.raymarch_check(xt, M, V, P, F, res, y, 1).cpu().numpy()
    ref = RM.raymarch_fwd(xs, M, V, P, F, res)
    ea, rm = _errors(y.cpu().numpy()[..., 3], ref[..., 3])
    assert ea > 0
    # the kernel's and NumPy's FP64 recomputations differ by double rounding only
    assert abs(got[0] - ea) <= 1e-9 * rm and _close(got[1], rm)
    assert got[0] / got[1] < 1e-5


def test_check_step_inside_the_captured_step(mods):
    from gft.pipeline import RenderAdvectStep
    st = RenderAdvectStep('tiny', torch.device('cuda', 0), fp64_check=True, check_strides=(1, 1))
    st.setup_static(st.make_inputs())
    st.capture(warmup=3)
    st.check_buf.fill_(-1.0)
    st.replay()
    torch.cuda.synchronize()
    e = st.fp64_errors()
    for k in ('transmittance_abs', 'transmittance_rel', 'raymarch_density_abs', 'raymarch_density_rel'):
        assert 0.0 <= e[k] < 1e-5, (k, e[k])
