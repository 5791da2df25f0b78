"""The benchmark step and the checkpointed transport chain on a tiny config:
graph replay equals eager execution, checkpointed gradients equal the plain
ones, batched equals plain, and the step gradient matches the oracle chain."""
import numpy as np
import pytest
import torch

from scene_utils import rel_l2

pytestmark = pytest.mark.gpu


@pytest.fixture(scope='module')
def gpu():
    if not torch.cuda.is_available():
        pytest.skip('no CUDA device')
    from gft import ops
    ops.set_grad_mode('REFERENCE')
    return torch.device('cuda', 0)


def _np(t):
    return t.detach().cpu().numpy().astype(np.float64)


def test_graph_replay_equals_eager(gpu):
    from gft.pipeline import RenderAdvectStep
    s = RenderAdvectStep('tiny', gpu)
    s.setup_static(s.make_inputs())
    loss_e, grads_e = s.run_static()
    loss_e, grads_e = float(loss_e), [_np(g) for g in grads_e]
    s.capture(warmup=3)
    loss_g, grads_g = s.replay()
    torch.cuda.synchronize()
    assert abs(float(loss_g) - loss_e) <= 1e-5 * abs(loss_e)
    for a, b in zip(grads_g, grads_e):
        assert rel_l2(_np(a), b) <= 1e-4


def test_capture_while_an_eager_step_is_alive(gpu):
    """Capturing the step while the autograd graph of an eager step through
    the same static inputs is still referenced (the static inputs become
    fresh leaves on the same memory)."""
    from gft.pipeline import RenderAdvectStep
    s = RenderAdvectStep('tiny', gpu)
    d_before = s.setup_static(s.make_inputs())[0]
    loss_e, grads_e = s.run_static()
    s.capture(warmup=3)
    assert s.s_d.data_ptr() == d_before.data_ptr()
    loss_g, grads_g = s.replay()
    torch.cuda.synchronize()
    assert abs(float(loss_g) - float(loss_e)) <= 1e-5 * abs(float(loss_e))
    for a, b in zip(grads_g, grads_e):
        assert rel_l2(_np(a), _np(b)) <= 1e-4


def test_streamed_steps_equal_single_steps(gpu):
    """StreamedSteps (inputs copied while the previous step runs, losses read
    one step late) gives each step the loss and gradients of running that
    step alone on the same inputs."""
    from gft.pipeline import RenderAdvectStep, StreamedSteps
    s = RenderAdvectStep('tiny', gpu)
    frames = [s.make_inputs(frame=f) for f in range(3)]
    ref = []
    for inp in frames:
        r = RenderAdvectStep('tiny', gpu)
        r.setup_static(inp)
        loss, grads = r.run_static()
        ref.append((float(loss), [_np(g) for g in grads]))
    streamed = StreamedSteps(s, frames[0])
    hosts = [StreamedSteps.host_inputs(inp) for inp in frames]
    order = [0, 1, 2, 1, 0]
    losses = streamed.run([hosts[i] for i in order])
    assert len(losses) == len(order)
    for j, i in enumerate(order):
        assert abs(losses[j] - ref[i][0]) <= 1e-5 * abs(ref[i][0])
    # the gradients of the last step (slot 0) before that slot runs again
    torch.cuda.synchronize()
    for a, b in zip(streamed.grads(len(order) - 1), ref[order[-1]][1]):
        assert rel_l2(_np(a), b) <= 1e-4


def test_batched_equals_plain(gpu):
    from gft.pipeline import RenderAdvectStep
    a = RenderAdvectStep('tiny', gpu, mode='batched')
    inp = a.make_inputs()
    a.setup_static(inp)
    b = RenderAdvectStep('tiny', gpu, mode='plain')
    b.setup_static(inp)
    la, ga = a.run_static()
    lb, gb = b.run_static()
    assert abs(float(la) - float(lb)) <= 1e-5 * abs(float(lb))
    for x, y in zip(ga, gb):
        assert rel_l2(_np(x), _np(y)) <= 1e-4


@pytest.mark.parametrize('order', [1, 2])
def test_bf16_storage_step_vs_fp64(gpu, order):
    """The BF16-storage step (loss and all four gradients) against the FP64
    step oracle at the BF16 tolerance, 1e-2 rel-L2, outside the voxels where
    the reference's advection adjoint is discontinuous in the lookups."""
    import tie_masks as TM
    from scene_utils import step_scene
    from gft.pipeline import RenderAdvectStep
    from oracle import step as OS
    st = RenderAdvectStep('tiny', gpu, storage_dtype=torch.bfloat16, order=order)
    inp = st.make_inputs()
    st.setup_static(inp)
    loss, grads = st.run_static()
    d0 = inp['d_prev'][0].astype(np.float64)
    vel = [inp[k].astype(np.float64) for k in ('vx', 'vy', 'vz')]
    ref_loss, _, ref_grads = OS.step(step_scene(st), d0, *vel, inp['target'])
    assert abs(float(loss.detach()) - ref_loss) <= 1e-2 * abs(ref_loss)
    dmask, vmask = TM.advect_masks(d0, *vel, order=order, clamp=st.clamp, reference=True)
    masks = (dmask,) + TM.face_masks(vmask)
    for name, g, r, m in zip(('density', 'vel_x', 'vel_y', 'vel_z'), grads, ref_grads, masks):
        mm = np.broadcast_to(m.reshape(m.shape + (1,) * (r.ndim - m.ndim)), r.shape)
        e = rel_l2(np.where(mm, 0.0, _np(g).reshape(r.shape)), np.where(mm, 0.0, r))
        assert e <= 1e-2, '%s gradient rel-L2 %.3g' % (name, e)


@pytest.mark.parametrize('tonemap', ['CLIP_NEGATIVE', 'SATURATE', 'NORMALIZE'])
def test_tonemapped_step_vs_fp64(gpu, tonemap):
    """The captured step with the renderer's tonemapping folded into its loss
    against the FP64 step oracle with the same tonemapping (FP32 tolerances,
    outside the advection adjoint's discontinuities)."""
    import tie_masks as TM
    from scene_utils import step_scene
    from gft.pipeline import RenderAdvectStep
    from oracle import step as OS
    st = RenderAdvectStep('tiny', gpu, tonemap=tonemap)
    inp = st.make_inputs()
    st.setup_static(inp)
    st.capture(warmup=3)
    loss, grads = st.replay()
    torch.cuda.synchronize()
    d0 = inp['d_prev'][0].astype(np.float64)
    vel = [inp[k].astype(np.float64) for k in ('vx', 'vy', 'vz')]
    ref_loss, _, ref_grads = OS.step(step_scene(st), d0, *vel, inp['target'])
    assert abs(float(loss) - ref_loss) <= 1e-5 * abs(ref_loss)
    dmask, vmask = TM.advect_masks(d0, *vel, order=st.order, clamp=st.clamp, reference=True)
    masks = (dmask,) + TM.face_masks(vmask)
    for name, g, r, m in zip(('density', 'vel_x', 'vel_y', 'vel_z'), grads, ref_grads, masks):
        mm = np.broadcast_to(m.reshape(m.shape + (1,) * (r.ndim - m.ndim)), r.shape)
        e = rel_l2(np.where(mm, 0.0, _np(g).reshape(r.shape)), np.where(mm, 0.0, r))
        assert e <= 1e-4, '%s gradient rel-L2 %.3g' % (name, e)


def test_checkpointed_chain_gradients(gpu):
    from gft.chain import TransportChain
    from gft.pipeline import RenderAdvectStep
    from gft import synthetic as syn
    s = RenderAdvectStep('tiny', gpu)
    T = 5
    d0 = torch.from_numpy(syn.plume_density(s.shape, 3)).to(gpu)
    vels = []
    for t in range(T - 1):
        vx, vy, vz = syn.curl_velocity(s.shape, 10 + t)
        vels.append(tuple(torch.from_numpy(v).to(gpu).requires_grad_(True) for v in (vx, vy, vz)))
    with torch.no_grad():
        targets = [s.render(torch.from_numpy(syn.plume_density(s.shape, 30 + t, t)).to(gpu))[..., :3] for t in range(T)]
    res = []
    for ck in (True, False):
        d = d0.clone().requires_grad_(True)
        chain = TransportChain(s, frames=T, checkpoint_every=2)
        loss = chain.loss(d, vels, targets, use_checkpoints=ck)
        g = torch.autograd.grad(loss, [d] + [v for tr in vels for v in tr])
        res.append((float(loss), [_np(x) for x in g]))
    assert abs(res[0][0] - res[1][0]) <= 1e-6 * abs(res[1][0])
    for a, b in zip(res[0][1], res[1][1]):
        assert rel_l2(a, b) <= 1e-4


def test_uneven_batch_step_equals_per_frame_steps(gpu):
    """The uneven-view batch step (frames x their own views in one
    raymarch_grid_transform_views call, batched shadow and light composition,
    one CUDA graph) equals the frames computed one at a time: the loss is the
    pixel-weighted mean of the per-frame losses and each frame's gradient the
    per-frame gradient scaled by its share of the pixels."""
    from gft.pipeline import UnevenBatchStep
    kw = dict(views=3, shape=(12, 16, 10), samples=14, device=gpu, shadow=(10, 10, 10), mips=2, sizes=(6, 12))
    both = UnevenBatchStep(frames=2, seed=70, **kw)
    rng = np.random.default_rng(71)
    d = (rng.random((2, 12, 16, 10, 1)) * 0.3).astype(np.float32)
    tgt = (rng.random((both.pixels, 3)) * 0.2).astype(np.float32)
    both.setup_static({'d': d, 'target': tgt})
    both.capture(warmup=2)
    loss, g = both.replay()
    torch.cuda.synchronize()
    loss, g = float(loss.detach()), _np(g)
    parts, grads, off = [], [], 0
    for f in range(2):
        one = UnevenBatchStep(frames=1, seed=70 + f, **kw)
        n = one.pixels
        one.setup_static({'d': d[f:f + 1], 'target': tgt[off:off + n]})
        lf, gf = one.step(one.s_d, one.s_t)
        parts.append((float(lf.detach()), n))
        grads.append(_np(gf) * n)
        off += n
    total = sum(n for _, n in parts)
    assert abs(loss - sum(l * n for l, n in parts) / total) <= 1e-5 * abs(loss)
    assert rel_l2(g, np.concatenate(grads, 0) / total) <= 1e-5
