"""One differentiable render + advect iteration of the global-transport
reconstruction, built on gft.ops (the path of Renderer.render_density,
SpotLight.grid_lighting and VelocityGrid.warp of the reference).

    d      = warp(d_prev, v)                    MacCormack + MC_SMOOTH, CLAMP
    shadow = exp(-shift(cumsum(sample(d))))     light frustum, LINDEPTH, mips
    light  = d * (back_project(shadow) * falloff * c * i + ambient)
    img    = raymarch(concat(light, d) * depth_step, cameras)   BEER_LAMBERT
    loss   = mean((img.rgb + bkg * exp(-img.a) - target)^2)

``batched``: all cameras in one raymarch launch, fused advection, the
transmittance, light composition and image loss as single kernels
(gft.fused), and the whole forward + backward captured in one CUDA graph.
``plain``: the reference's launch structure -- one raymarch launch per camera,
advection composed from four SampleGridLut calls plus elementwise ops, the
shadow, lighting and loss composed from tensor ops, no graph.
All constants are device tensors created up front so the step is capturable.
"""
import numpy as np
import torch

from . import fused
from . import ops
from . import synthetic as syn
from phitest.render.lighting import SpotLight
from phitest.render.transform import Transform


class RenderSettings:
    """The Renderer fields the shadow pass reads (renderer.py:64-88)."""

    def __init__(self, num_mips=3):
        self.filter_mode = 'LINEAR'
        self.boundary_mode = 'BORDER'
        self.mip_mode = 'LINEAR'
        self.num_mips = num_mips
        self.mip_bias = 0.0
        self.gradient_mip_bias_add = 0.0
        self.blend_mode = 'BEER_LAMBERT'


def _fresh_leaves(*ts):
    """New leaf tensors on the same storage (the graph's static inputs keep
    their memory).  A leaf's gradient accumulator records the stream of its
    first use and lives as long as any autograd graph through the leaf; if
    an eager step on the default stream still holds one, a capture of the
    step on another stream would wait on the default stream, which CUDA
    refuses during capture."""
    return tuple(t.detach().requires_grad_(t.requires_grad) for t in ts)


CONFIGS = {
    # multi-view frame: 5 views of 480x270 (height x width), 192 samples, 3 mips, spot light + shadow volume
    'cfg2': dict(grid=(128, 227, 128), views=5, image=(480, 270), samples=192, mips=3,
                 shadow=(256, 196, 196), seed=2000),
    # 64^3 single-view case for quick runs / CPU timing
    'cfg1': dict(grid=(64, 64, 64), views=1, image=(128, 128), samples=64, mips=3,
                 shadow=(64, 64, 64), seed=1000),
    # stress grid 256x455x256, 5 views of 960x540 (height x width), 256 samples (one frame)
    'cfg5': dict(grid=(256, 455, 256), views=5, image=(960, 540), samples=256, mips=4,
                 shadow=(256, 196, 196), seed=5000),
    # tiny case for tests
    'tiny': dict(grid=(10, 12, 9), views=2, image=(9, 11), samples=12, mips=2,
                 shadow=(8, 8, 8), seed=7),
}


class RenderAdvectStep:
    """One render + advect iteration (see the module docstring).  storage_dtype
    (torch.bfloat16) stores the raymarch input in bf16; advect_storage_dtype
    does the same for the advection's input density (default fp32: the
    advection's gathers are latency-bound, so bf16 saves little there, and an
    fp32 input lets the adjoint reuse the forward's intermediate grid and
    differentiate at the fp32 density)."""

    def __init__(self, config='cfg2', device='cuda', storage_dtype=None, mode='batched', order=None,
                 fp64_check=False, check_strides=(7, 257), autotune=False, tonemap='NONE',
                 advect_storage_dtype=None):
        self.config_name = config if isinstance(config, str) else None
        self.advect_storage_dtype = advect_storage_dtype
        # tonemapping of the composited images before the loss (renderer.py:639-640)
        self.tonemap = str(tonemap).upper()
        cfg = dict(CONFIGS[config] if isinstance(config, str) else config)
        if order is not None:
            cfg['order'] = int(order)
        self.cfg = cfg
        self.order = int(cfg.get('order', 2))  # 1 semi-Lagrangian, 2 MacCormack (+ MC_SMOOTH)
        self.clamp = 'MC_SMOOTH' if self.order == 2 else 'NONE'
        self.dev = torch.device(device)
        self.storage_dtype = storage_dtype
        self.mode = mode
        D, H, W = cfg['grid']
        self.shape = (D, H, W)
        Hi, Wi = cfg['image']
        self.res = (cfg['samples'], Hi, Wi)
        self.gt = syn.grid_transform(self.shape)
        self.cams = syn.arc_cameras(cfg['views'], self.res, radius=2.5, fov=30.0)
        self.M = syn.model_matrix(self.gt)
        self.V, self.P, self.F = syn.camera_params(self.cams)
        self.depth_step = float(self.cams[0].depth_step)
        # spot light with shadow volume + ambient (lighting set-up of reconstruct_sequence.py:696-705)
        self.spot = SpotLight(Transform(translation=[0, 0, 2.0], parent=Transform(rotation_deg=[-40, 0, 0])),
                              intensity=0.85, cast_shadows=True, shadow_clip=[0.85, 3.15], range_scale=0.825,
                              angle_deg=60.0, shadow_resolution=list(cfg['shadow']), cone_mask=False)
        self.ambient = 0.64
        self.rs = RenderSettings(cfg['mips'])
        self.Vs, self.Ps, self.Fs = syn.camera_params([self.spot.shadow_cam])
        self.shadow_step = float(self.spot.shadow_cam.depth_step)
        self.shadow_res = tuple(cfg['shadow'])
        fall = self.spot.falloff(_Holder(self.gt), self.dev)  # [D,H,W,1]
        col = torch.tensor(self.spot.c * np.float32(self.spot.i), dtype=torch.float32, device=self.dev)
        self.falloff_col = (fall * col)[None].contiguous()  # [1,D,H,W,3]
        # the same light factored (falloff x colour) for the fused render
        self.light = (fall.contiguous(), col.cpu().numpy())
        self.bkg_host = np.array([0.0, 0.5, 1.0], dtype=np.float32)
        self.bkg = torch.from_numpy(self.bkg_host).to(self.dev)
        self.graph = None
        # launch-configuration knobs chosen by gft.autotune before the capture
        self.autotune = bool(autotune)
        self.knobs, self.tune_log = None, {}
        # FP64 check step (batched mode): double-precision recomputation of the
        # shadow transmittance (every check_strides[0]-th light-frustum column)
        # and of the raymarch's accumulated density (every check_strides[1]-th
        # ray) of each forward, into a device buffer read by fp64_errors()
        self.fp64_check = bool(fp64_check) and mode != 'plain'
        self.check_strides = tuple(int(v) for v in check_strides)
        self.check_buf = torch.zeros(4, dtype=torch.float64, device=self.dev) if self.fp64_check else None

    # --------------------------------------------------------------- inputs
    def make_inputs(self, frame=0, target_seed_offset=7):
        """Seeded density (previous frame), staggered velocity and target images
        (rendered from a perturbed plume with the same path)."""
        seed = self.cfg['seed'] + frame
        d_prev = syn.plume_density(self.shape, seed, frame)
        vx, vy, vz = syn.curl_velocity(self.shape, seed + 500)
        with torch.no_grad():
            dt = torch.from_numpy(syn.plume_density(self.shape, seed + target_seed_offset, frame + 1)).to(self.dev)
            tgt = self.render(dt)[..., :3].contiguous()
        return dict(d_prev=d_prev, vx=vx[0], vy=vy[0], vz=vz[0], target=tgt.cpu().numpy())

    # --------------------------------------------------------------- pieces
    def advect(self, d_prev, vx, vy, vz):
        if self.mode == 'plain':
            return advect_composed(d_prev, vx, vy, vz, dt=1.0, order=self.order, clamp=self.clamp, boundary='CLAMP')
        return ops.advect(d_prev, vx, vy, vz, dt=1.0, order=self.order, clamp=self.clamp, boundary='CLAMP',
                          storage_dtype=self.advect_storage_dtype)

    def shadow(self, d):
        from phitest.render.renderer import _InverseSampleGrad
        sh = _InverseSampleGrad.apply(d * self.shadow_step, self.M, self.Vs, self.Ps, self.Fs, self.shadow_res,
                                      'TRANSFORM_LINDEPTH', 'TRANSFORM_LINDEPTH_REVERSE', self.rs, None)
        if self.mode == 'plain':
            sh = ops.reduce_grid_blend(sh[0], 'BEER_LAMBERT', keep_dims=True)
            sh = torch.cat([torch.zeros_like(sh[:, :1]), sh[:, :-1]], dim=1)  # BORDER shift
            tr = torch.exp(-sh)
        else:
            tr = fused.transmittance(sh.squeeze(0))  # a view: no zero-fill in the backward
            if self.fp64_check:
                fused.transmittance_check(sh.squeeze(0).detach(), tr.detach(), self.check_strides[0],
                                          out=self.check_buf[0:2])
        trv = _InverseSampleGrad.apply(tr, self.M, self.Vs, self.Ps, self.Fs, self.shape,
                                       'TRANSFORM_LINDEPTH_REVERSE', 'TRANSFORM_LINDEPTH', self.rs, None)
        return trv.squeeze(0)  # [1,D,H,W,1]

    def render(self, d):
        if self.mode == 'plain':
            light = d * (self.shadow(d) * self.falloff_col + self.ambient)
            data = torch.cat([light, d], dim=-1) * self.depth_step
            imgs = [ops.raymarch_grid_transform(data, self.M, self.V[i:i + 1], self.P[i:i + 1], self.F[i:i + 1],
                                                self.res) for i in range(len(self.V))]
            img = torch.cat(imgs, dim=1)
        else:
            # the light composition writes the raymarch input directly, in the
            # brick layout and the storage type
            img, xs = fused.render_bricked(d, self.shadow(d), self.light, self.ambient, self.depth_step,
                                           self.M, self.V, self.P, self.F, self.res,
                                           storage_dtype=self.storage_dtype)
            if self.fp64_check:
                ops.raymarch_check(xs, self.M, self.V, self.P, self.F, self.res, img.detach(), self.check_strides[1],
                                   grid_shape=self.shape, out=self.check_buf[2:4])
        return img.squeeze(0)  # [V,H,W,4]

    def fp64_errors(self):
        """Largest deviations of the last forward's FP32 results from their FP64
        recomputation (needs fp64_check=True): transmittance and raymarch
        density, absolute and relative to the largest FP64 value (max norm)."""
        v = self.check_buf.cpu().tolist()
        rel = lambda e, m: e / m if m > 0 else 0.0
        return {'transmittance_abs': v[0], 'transmittance_rel': rel(v[0], v[1]), 'raymarch_density_abs': v[2],
                'raymarch_density_rel': rel(v[2], v[3]),
                'strides': {'transmittance_columns': self.check_strides[0], 'raymarch_rays': self.check_strides[1]}}

    def loss(self, d_prev, vx, vy, vz, target):
        if self.mode != 'plain' and torch.is_grad_enabled() and ops.get_grad_mode() == 'REFERENCE':
            # the raymarch gradient's geometry-only weight pass overlaps advection and shadow
            ops.prefetch_raymarch_weights(tuple(d_prev.shape[:4]) + (4,), self.M, self.V, self.P, self.F, self.res,
                                          device=d_prev.device, for_camera_sums=True)
        d = self.advect(d_prev, vx, vy, vz)
        img = self.render(d)
        if self.mode != 'plain':
            return fused.image_loss(img, target, self.bkg_host, self.tonemap)
        rgb = img[..., :3] + self.bkg * torch.exp(-img[..., 3:])
        return torch.mean((tonemap_tensor(rgb, self.tonemap) - target) ** 2)

    def step(self, d_prev, vx, vy, vz, target):
        """Forward + backward; returns (loss, (g_d_prev, g_vx, g_vy, g_vz))."""
        loss = self.loss(d_prev, vx, vy, vz, target)
        grads = torch.autograd.grad(loss, [d_prev, vx, vy, vz])
        return loss, grads

    # --------------------------------------------------------------- graphs
    def setup_static(self, inputs):
        dev = self.dev
        self.s_d = torch.from_numpy(inputs['d_prev']).to(dev).requires_grad_(True)
        self.s_vx = torch.from_numpy(inputs['vx'][None]).to(dev).requires_grad_(True)
        self.s_vy = torch.from_numpy(inputs['vy'][None]).to(dev).requires_grad_(True)
        self.s_vz = torch.from_numpy(inputs['vz'][None]).to(dev).requires_grad_(True)
        self.s_t = torch.from_numpy(inputs['target']).to(dev)
        return (self.s_d, self.s_vx, self.s_vy, self.s_vz, self.s_t)

    def capture(self, warmup=3):
        """Captures step() on the static inputs into one CUDA graph (after
        tuning the launch-configuration knobs on them, with autotune)."""
        self.s_d, self.s_vx, self.s_vy, self.s_vz = _fresh_leaves(self.s_d, self.s_vx, self.s_vy, self.s_vz)
        args = (self.s_d, self.s_vx, self.s_vy, self.s_vz, self.s_t)
        if self.autotune:
            from . import autotune as _at
            self.knobs = _at.tune(lambda: self.step(*args), key=_at.step_key(self), log=self.tune_log)
        side = torch.cuda.Stream(self.dev)
        side.wait_stream(torch.cuda.current_stream(self.dev))
        with torch.cuda.stream(side):
            for _ in range(warmup):
                self.step(*args)
        torch.cuda.current_stream(self.dev).wait_stream(side)
        torch.cuda.synchronize(self.dev)
        self.graph = torch.cuda.CUDAGraph()
        with torch.cuda.graph(self.graph):
            self.g_loss, self.g_grads = self.step(*args)
        torch.cuda.synchronize(self.dev)
        return self.graph

    def replay(self):
        self.graph.replay()
        return self.g_loss, self.g_grads

    def run_static(self):
        if self.graph is not None:
            return self.replay()
        return self.step(self.s_d, self.s_vx, self.s_vy, self.s_vz, self.s_t)


class UnevenBatchStep:
    """A batch of frames rendered by views bound to their frame (the uneven-view
    workload): per frame one fixed view plus ``views`` seeded cameras on the
    upper hemisphere with square images of 64-256 pixels, all with ``samples``
    depth samples; each frame lit by the spot light with its shadow pass; loss =
    mean squared difference of every view's image (background composite) to its
    target; forward + backward to every frame's density.  The raymarch of all
    frames' views runs as gft.ops.raymarch_grid_transform_views (16 views per
    launch), the shadow pass and the light composition batched over the frames,
    the whole step capturable in one CUDA graph.

    clip_cameras: each camera's top/right/bottom/left narrowed to the density
    grid's world bounding box (Camera.copy_clipped_to_world_coords with
    preserve_clip, so the depth step stays that of the original camera), as the
    reference fits its render cameras to the density's hull, so fewer rays
    miss the grid."""

    def __init__(self, frames=64, views=8, shape=(96, 170, 96), samples=128, device='cuda', storage_dtype=None,
                 clip_cameras=True, seed=4000, shadow=(128, 128, 128), mips=3, sizes=(64, 256)):
        self.dev = torch.device(device)
        self.knobs = None
        self.frames = int(frames)
        self.shape = tuple(shape)
        self.storage_dtype = storage_dtype
        self.gt = syn.grid_transform(self.shape)
        D, H, W = self.shape
        corners = self.gt.transform_AABB([0, 0, 0], [W, H, D], True)
        Vs, Ps, Fs, self.shapes, self.camera_batch, steps = [], [], [], [], [], []
        for f in range(self.frames):
            cams, shp = syn.hemisphere_cameras(views, samples, sizes=sizes, seed=seed + f)
            if clip_cameras:
                cams = [c.copy_clipped_to_world_coords(corners, preserve_clip=True)[0] for c in cams]
            V, P, F = syn.camera_params(cams)
            Vs.append(V), Ps.append(P), Fs.append(F)
            self.shapes += [list(s) for s in shp]
            self.camera_batch += [f] * len(cams)
            steps += [c.depth_step for c in cams]
        self.V, self.P, self.F = np.concatenate(Vs), np.concatenate(Ps), np.concatenate(Fs)
        self.depth_step = float(steps[0])
        if not np.allclose(steps, self.depth_step):
            raise ValueError('the views of a batch must share one depth step')
        self.M = np.concatenate([syn.model_matrix(self.gt)] * self.frames)
        self.spot = SpotLight(Transform(translation=[0, 0, 2.0], parent=Transform(rotation_deg=[-40, 0, 0])),
                              intensity=0.85, cast_shadows=True, shadow_clip=[0.85, 3.15], range_scale=0.825,
                              angle_deg=60.0, shadow_resolution=list(shadow), cone_mask=False)
        self.ambient = 0.64
        self.rs = RenderSettings(mips)
        self.Vs, self.Ps, self.Fs = syn.camera_params([self.spot.shadow_cam])
        self.shadow_step = float(self.spot.shadow_cam.depth_step)
        self.shadow_res = tuple(shadow)
        fall = self.spot.falloff(_Holder(self.gt), self.dev)
        col = torch.tensor(self.spot.c * np.float32(self.spot.i), dtype=torch.float32, device=self.dev)
        self.falloff_col = (fall * col)[None].contiguous()
        self.bkg_host = np.array([0.0, 0.5, 1.0], dtype=np.float32)
        self.pixels = sum(h * w for _, h, w in self.shapes)
        self.graph = None

    def make_inputs(self, seed=0, target_seed_offset=7):
        """Seeded frame densities [F, D, H, W, 1] (plumes rising with the frame)
        and targets [pixels, 3] rendered from perturbed plumes."""
        d = np.concatenate([syn.plume_density(self.shape, seed + f, f) for f in range(self.frames)], 0)
        dt = np.concatenate([syn.plume_density(self.shape, seed + f + target_seed_offset, f + 1)
                             for f in range(self.frames)], 0)
        with torch.no_grad():
            tgt = self.render(torch.from_numpy(dt).to(self.dev))[..., :3].contiguous()
        return dict(d=d, target=tgt.cpu().numpy())

    def shadow(self, d):
        from phitest.render.renderer import _InverseSampleGrad
        sh = _InverseSampleGrad.apply(d * self.shadow_step, self.M, self.Vs, self.Ps, self.Fs, self.shadow_res,
                                      'TRANSFORM_LINDEPTH', 'TRANSFORM_LINDEPTH_REVERSE', self.rs, None)
        tr = fused.transmittance(sh[:, 0])
        trv = _InverseSampleGrad.apply(tr, self.M, self.Vs, self.Ps, self.Fs, self.shape,
                                       'TRANSFORM_LINDEPTH_REVERSE', 'TRANSFORM_LINDEPTH', self.rs, None)
        return trv[:, 0]  # [F,D,H,W,1]

    def render(self, d):
        """Images of all views, [pixels, 4], the views one after another."""
        data = fused.light_compose(d, self.shadow(d), self.falloff_col, self.ambient, self.depth_step)
        return ops.raymarch_grid_transform_views(data, self.camera_batch, self.M, self.V, self.P, self.F,
                                                 self.shapes, storage_dtype=self.storage_dtype)

    def step(self, d, target):
        loss = fused.image_loss(self.render(d), target, self.bkg_host)
        (g,) = torch.autograd.grad(loss, [d])
        return loss, g

    def setup_static(self, inputs):
        self.s_d = torch.from_numpy(inputs['d']).to(self.dev).requires_grad_(True)
        self.s_t = torch.from_numpy(inputs['target']).to(self.dev)

    def capture(self, warmup=3, autotune=False, tune_log=None):
        """Captures step() into one CUDA graph (after tuning the
        launch-configuration knobs on it, with autotune; the chosen values
        stay set and are kept in self.knobs)."""
        (self.s_d,) = _fresh_leaves(self.s_d)
        if autotune:
            from . import autotune as _at
            self.knobs = _at.tune(lambda: self.step(self.s_d, self.s_t), key=_at.step_key(self), log=tune_log)
        side = torch.cuda.Stream(self.dev)
        side.wait_stream(torch.cuda.current_stream(self.dev))
        with torch.cuda.stream(side):
            for _ in range(warmup):
                self.step(self.s_d, self.s_t)
        torch.cuda.current_stream(self.dev).wait_stream(side)
        torch.cuda.synchronize(self.dev)
        self.graph = torch.cuda.CUDAGraph()
        with torch.cuda.graph(self.graph):
            self.g_loss, self.g_grad = self.step(self.s_d, self.s_t)
        torch.cuda.synchronize(self.dev)

    def replay(self):
        self.graph.replay()
        return self.g_loss, self.g_grad


class StreamedSteps:
    """Runs the graph-captured step over a stream of host inputs with the
    transfers overlapped: two captured copies of the step, each with its own
    input slot, alternate; the host-to-device copy of step i+1's inputs (from
    pinned host memory, on a copy stream) runs while step i computes, and each
    step's loss is copied back to pinned host memory on the compute stream and
    read by the host one step later, so the host never stalls the device.
    Every step still copies its own inputs and reads its own loss.

    step: a RenderAdvectStep (batched mode) whose configuration both slots
    use; example: inputs as make_inputs returns them (to set up the slots)."""

    KEYS = ('d', 'vx', 'vy', 'vz', 't')

    def __init__(self, step, example, warmup=3):
        self.dev = step.dev
        self.slots = [step, RenderAdvectStep(step.config_name or step.cfg, step.dev, storage_dtype=step.storage_dtype,
                                             mode=step.mode, order=step.order,
                                             advect_storage_dtype=step.advect_storage_dtype)]
        for st in self.slots:
            st.setup_static(example)
            st.capture(warmup=warmup)
        self.copy_stream = torch.cuda.Stream(self.dev)
        self.copied = [torch.cuda.Event() for _ in self.slots]
        self.done = [torch.cuda.Event() for _ in self.slots]
        self.loss_ready = [torch.cuda.Event() for _ in self.slots]
        self.loss_host = [torch.empty(1, dtype=torch.float32).pin_memory() for _ in self.slots]
        for ev in self.done:
            ev.record(torch.cuda.current_stream(self.dev))

    @staticmethod
    def host_inputs(inputs):
        """Pinned host tensors of make_inputs' arrays, keyed d, vx, vy, vz, t."""
        import numpy as _np
        arrays = (inputs['d_prev'], inputs['vx'][None], inputs['vy'][None], inputs['vz'][None], inputs['target'])
        return {k: torch.from_numpy(_np.ascontiguousarray(a)).pin_memory() for k, a in zip(StreamedSteps.KEYS, arrays)}

    @staticmethod
    def h2d_bytes(host):
        return sum(v.numel() * v.element_size() for v in host.values())

    def _enqueue(self, i, host):
        k = i % len(self.slots)
        st = self.slots[k]
        dsts = (st.s_d, st.s_vx, st.s_vy, st.s_vz, st.s_t)
        cur = torch.cuda.current_stream(self.dev)
        with torch.cuda.stream(self.copy_stream), torch.no_grad():
            self.copy_stream.wait_event(self.done[k])  # the slot's previous step has consumed its inputs
            for key, dst in zip(self.KEYS, dsts):
                dst.copy_(host[key], non_blocking=True)
            self.copied[k].record(self.copy_stream)
        cur.wait_event(self.copied[k])
        loss, _ = st.replay()
        self.done[k].record(cur)
        self.loss_host[k].copy_(loss.detach().reshape(1), non_blocking=True)
        self.loss_ready[k].record(cur)

    def _read(self, i):
        k = i % len(self.slots)
        self.loss_ready[k].synchronize()
        return float(self.loss_host[k][0])

    def run(self, host_inputs):
        """Steps over an iterable of host_inputs() dicts; returns the losses."""
        losses = []
        i = -1
        for i, host in enumerate(host_inputs):
            self._enqueue(i, host)
            if i >= 1:
                losses.append(self._read(i - 1))
        if i >= 0:
            losses.append(self._read(i))
        return losses

    def grads(self, i):
        """Gradients of step i (valid until that slot runs again, two steps later)."""
        return self.slots[i % len(self.slots)].g_grads


class _Holder:
    """GridTransform view used for the falloff computation."""

    def __init__(self, gt):
        self.gt = gt
        self.grid_size = gt.grid_size

    def cell_size_world(self):
        return self.gt.cell_size_world()

    def grid_size_world(self):
        return self.gt.grid_size_world()

    def get_inverse_transform(self):
        return self.gt.get_inverse_transform()


def centered_lut(vx, vy, vz, dt):
    """lut = -dt * centred velocity with a zero LOD channel (data_structures.py:819-868,
    renderer.py:449-455), from staggered [1,D,H,W+1,1], [1,D,H+1,W,1], [1,D+1,H,W,1]."""
    cx = (vx[:, :, :, 1:] + vx[:, :, :, :-1]) * 0.5
    cy = (vy[:, :, 1:] + vy[:, :, :-1]) * 0.5
    cz = (vz[:, 1:] + vz[:, :-1]) * 0.5
    v = torch.cat([cx, cy, cz], dim=-1) * (-dt)
    return torch.nn.functional.pad(v, (0, 1))


def tonemap_tensor(image, mode='NONE'):
    """The renderer's tonemapping as tensor ops (phitest/render/renderer.py:528-541)."""
    if mode == 'NONE':
        return image
    if mode == 'CLIP_NEGATIVE':
        return torch.clamp_min(image, 0)
    if mode == 'SATURATE':
        return torch.clamp(image, 0, 1)
    if mode == 'NORMALIZE':
        mn = torch.min(image)
        image = torch.where(mn < 0, image - mn, image)
        mx = torch.max(image)
        return torch.where(mx > 0, image / mx, image)
    raise ValueError(mode)


def advect_composed(d, vx, vy, vz, dt=1.0, order=2, clamp='MC_SMOOTH', boundary='CLAMP'):
    """VelocityGrid.warp as the reference composes it (data_structures.py:870-905):
    SampleGridLut calls and elementwise ops.  Velocity components carry a leading
    batch dim of 1 ([1,D,H,W+1,1], ...)."""
    lut = centered_lut(vx, vy, vz, dt)

    def look(x, l, filt='LINEAR'):
        return ops.sample_grid_lut(x, l, filt, boundary, separate_camera_batch=False, relative_coords=True)[:, 0]

    fwd = look(d, lut)
    if order == 1:
        out = fwd
    else:
        back = look(fwd, -lut)
        corr = fwd + 0.5 * (d - back)
        if clamp in ('MC', 'MC_SMOOTH'):
            mn = look(d, lut, 'MIN')
            mx = look(d, lut, 'MAX')
            oob = torch.logical_or(corr < mn, corr > mx)
            corr = torch.where(oob, fwd, corr)
        out = corr
    if clamp == 'NEGATIVE':
        out = torch.clamp_min(out, 0)
    return out
