"""Launch-configuration knobs change how kernels are launched, not what they
compute: every candidate of every knob gives the default launch's results
(bit-identical forward raymarch; the scatters and segmented scans up to the
order of their floating-point additions), and the tuner picks one of them
and caches it."""
import numpy as np
import pytest
import torch

from scene_utils import rel_l2, scene, small_grid

pytestmark = pytest.mark.gpu


@pytest.fixture(scope='module')
def gpu():
    if not torch.cuda.is_available():
        pytest.skip('no CUDA device')
    from gft import autotune, ops
    ops.set_grad_mode('REFERENCE')
    prev = autotune.knobs()
    yield torch.device('cuda', 0)
    autotune.apply(prev)


def _np(t):
    return t.detach().float().cpu().numpy().astype(np.float64)


@pytest.mark.parametrize('mode', ['REFERENCE', 'EXACT'])
def test_persistent_raymarch_grid_equals_one_block_per_tile(gpu, mode):
    """5 views of 480x270 (5100 pixel tiles, so a persistent grid of 2-6
    blocks per SM walks many tiles per block) over a sparse 24x30x20 grid:
    forward (with the sample store) bit-identical, gradient equal."""
    from gft import autotune, ops
    shape, res = (24, 30, 20), (40, 270, 480)
    _, _, M, V, P, F = scene(shape, 5, res)
    x = small_grid(shape, 4, 9) * 0.3
    x[:, :, :10] = 0.0
    xt = torch.from_numpy(x).cuda()
    dy = torch.randn((1, 5, 270, 480, 4), device='cuda', generator=torch.Generator('cuda').manual_seed(3)) * 1e-3

    def run():
        xi = xt.clone().requires_grad_(True)
        with ops.grad_mode(mode):
            y = ops.raymarch_grid_transform(xi, M, V, P, F, res)
            y.backward(dy)
        torch.cuda.synchronize()
        return y.detach().clone(), xi.grad.detach().clone()

    with autotune.knob_settings({'raymarch_blocks_per_sm': 0}):
        y0, g0 = run()
    for v in autotune.KNOBS['raymarch_blocks_per_sm'][1][1:]:
        with autotune.knob_settings({'raymarch_blocks_per_sm': v}):
            y, g = run()
        assert torch.equal(y, y0), v
        assert rel_l2(_np(g), _np(g0)) <= 1e-6, v


@pytest.mark.parametrize('name', ['advect_threads', 'resample_threads', 'scan_segments', 'raymarch_blocks_per_sm',
                                  'weights_blocks_per_sm', 'weights_pipeline'])
def test_step_results_equal_for_every_knob_value(gpu, name):
    from gft import autotune
    from gft.pipeline import RenderAdvectStep
    st = RenderAdvectStep('cfg1', gpu)
    st.setup_static(st.make_inputs())
    with autotune.knob_settings(autotune.defaults()):
        l0, g0 = st.run_static()
        l0, g0 = float(l0.detach()), [_np(g) for g in g0]
    for v in autotune.KNOBS[name][1]:
        with autotune.knob_settings({name: v}):
            loss, grads = st.run_static()
        assert abs(float(loss.detach()) - l0) <= 1e-6 * abs(l0), (name, v)
        for a, b in zip(grads, g0):
            assert rel_l2(_np(a), b) <= 1e-5, (name, v)


@pytest.mark.parametrize('project', [False, True])
def test_pipelined_weight_pass_gradient(gpu, project):
    """GFT_KNOB_WEIGHTS_PIPELINE: the reference-normalised gradient with each
    camera's weight sums computed on the library's side stream beside the
    previous camera's scatter equals the one-pass gradient (5 views, stored
    samples; 4 channels, or projected onto two)."""
    from gft import autotune, ops
    shape, res = (24, 30, 20), (40, 135, 240)
    _, _, M, V, P, F = scene(shape, 5, res)
    x = torch.from_numpy(small_grid(shape, 4, 11) * 0.3).cuda()
    xb = ops.to_bricks(x)
    shape5 = (1,) + shape + (4,)
    smp = ops._samples_buffer(shape5, 5, res, True, gpu)
    y = ops._raymarch_fwd(xb, M, V, P, F, res, 1, 0, 0, True, grid=shape, samples=smp)
    dy = torch.randn(y.shape, device='cuda', generator=torch.Generator('cuda').manual_seed(5)) * 1e-3
    proj = np.array([0.3, -1.2, 0.7, 0.0, 0.5, 0.5, 0.5, 1.1], np.float32) if project else None
    bwd = lambda: ops._raymarch_bwd(xb, y, dy, M, V, P, F, res, 1, 0, 0, True, ops.GRAD['REFERENCE'], grid=shape,
                                    samples=smp, projection=proj)
    with autotune.knob_settings({'weights_pipeline': 0}):
        g0 = bwd()
    with autotune.knob_settings({'weights_pipeline': 1}):
        g1 = bwd()
        torch.cuda.synchronize()
        # twice in a row on the same side stream and events
        g2 = bwd()
    torch.cuda.synchronize()
    assert np.abs(_np(g0)).max() > 0
    assert rel_l2(_np(g1), _np(g0)) <= 1e-6
    assert rel_l2(_np(g2), _np(g0)) <= 1e-6


def test_pipelined_weight_pass_in_a_captured_step(gpu):
    """The side stream forks from and joins the capturing stream: a step
    captured with the pipeline knob replays to the eager default step's loss
    and gradients."""
    from gft import autotune
    from gft.pipeline import RenderAdvectStep
    st = RenderAdvectStep('cfg1', gpu)
    st.setup_static(st.make_inputs())
    with autotune.knob_settings(autotune.defaults()):
        l0, g0 = st.run_static()
        l0, g0 = float(l0.detach()), [_np(g) for g in g0]
    with autotune.knob_settings({'weights_pipeline': 1}):
        cap = RenderAdvectStep('cfg1', gpu)
        cap.setup_static(cap.make_inputs())
        cap.capture(warmup=2)
        for _ in range(2):
            loss, grads = cap.replay()
        torch.cuda.synchronize()
    assert abs(float(loss.detach()) - l0) <= 1e-6 * abs(l0)
    for a, b in zip(grads, g0):
        assert rel_l2(_np(a), b) <= 1e-5


def test_tuner_picks_a_candidate_and_caches_it(gpu):
    from gft import autotune
    from gft.pipeline import RenderAdvectStep
    st = RenderAdvectStep('cfg1', gpu, autotune=True)
    st.setup_static(st.make_inputs())
    st.capture(warmup=2)
    for name, (_, cands, _) in autotune.KNOBS.items():
        assert st.knobs[name] in cands and autotune.get_knob(name) == st.knobs[name]
        assert set(st.tune_log[name]) == {str(c) for c in cands}
    # the same workload again: the cached choice, no timing
    again = RenderAdvectStep('cfg1', gpu, autotune=True)
    again.setup_static(again.make_inputs())
    again.capture(warmup=1)
    assert again.knobs == st.knobs and again.tune_log == {}
    loss, _ = again.replay()
    torch.cuda.synchronize()
    assert np.isfinite(float(loss.detach()))
