"""Renderer with the reference's API (phitest/render/renderer.py) on torch tensors.

Data are CUDA tensors in NDHWC; the sampling, blending and raymarching ops run
in libgft.so.  Method names, arguments and composition follow the reference
(renderer.py:64-651); TensorFlow elementwise ops become torch ops.
"""
import contextlib
import logging
from collections.abc import Iterable

import numpy as np
import torch

from gft import ops as _gops
from .cuda.ops_loader import blending_ops, raymarching_ops, sampling_ops
from .transform import GridTransform


class Profiler(object):
    """Minimal stand-in for phitest.render.profiling.Profiler: ``sample(name)``
    context managers (the wall-clock profiler itself is host tooling)."""

    def sample(self, name):
        return contextlib.nullcontext()


class _InverseSampleGrad(torch.autograd.Function):
    """SampleGridTransform with the reference's ``sample_gradients`` backward
    (renderer.py:200-227, :246-272): dx = sum over views of dy resampled through
    the inverse transform (with mips and bias + fast_gradient_mip_bias_add)."""

    @staticmethod
    def forward(ctx, x, M, V, P, F, out_shape, cm, inv_cm, r, storage_dtype):
        y = _gops.sample_grid_transform(x.detach(), M, V, P, F, out_shape, interpolation=r.filter_mode,
                                        boundary=r.boundary_mode, mipmapping=r.mip_mode, num_mipmaps=r.num_mips,
                                        mip_bias=r.mip_bias, coordinate_mode=cm, storage_dtype=storage_dtype)
        ctx.args = (tuple(x.shape), M, V, P, F, inv_cm, r)
        return y

    @staticmethod
    def backward(ctx, dy):
        in_shape, M, V, P, F, inv_cm, r = ctx.args
        batch = len(M)
        views = len(V)
        dx = []
        dy = dy.contiguous()
        for i in range(batch):
            m_views = np.stack([np.asarray(M[i], dtype=np.float32)] * views)
            dxv = _gops.sample_grid_transform(dy[i], m_views, V, P, F, in_shape[1:4], interpolation=r.filter_mode,
                                              boundary=r.boundary_mode, mipmapping=r.mip_mode,
                                              num_mipmaps=r.num_mips, mip_bias=r.mip_bias + r.gradient_mip_bias_add,
                                              coordinate_mode=inv_cm, separate_camera_batch=False,
                                              dense_input=True)  # V1DHWC (a gradient: dense)
            dx.append(torch.sum(dxv, dim=0) if views > 1 else dxv[0])  # 1DHWC (one view: the slice itself)
        dx = torch.cat(dx, dim=0) if batch > 1 else dx[0]
        return (dx,) + (None,) * 9


class Renderer(object):
    def __init__(self, profiler=None, filter_mode='LINEAR', boundary_mode='BORDER', mipmapping='LINEAR', num_mips=2,
                 mip_bias=0.0, sample_gradients=False, fast_gradient_mip_bias_add=0.0, blend_mode='BEER_LAMBERT',
                 name='Renderer', **kwargs):
        self.log = logging.getLogger(name)
        self.cameras = []
        self.profiler = profiler if profiler is not None else Profiler()
        self.blending = blending_ops
        self.filter_mode = filter_mode
        self.boundary_mode = boundary_mode
        self.mip_mode = mipmapping
        self.num_mips = num_mips
        self.mip_bias = mip_bias
        self.gradient_mip_bias_add = fast_gradient_mip_bias_add
        self.sample_gradients = sample_gradients
        self.blend_mode = blend_mode
        if 'luma' in kwargs:
            self.luma = kwargs['luma']
        self.allow_fused = kwargs.get('fused', False)
        self.scattering_ratio = kwargs.get('scattering_ratio', 1.0)
        # GB300 extension: storage dtype of the sampled grids (None = as given)
        self.storage_dtype = kwargs.get('storage_dtype', None)

    @property
    def can_render_fused(self):
        return self.allow_fused and (self.blend_mode in ['BEER_LAMBERT', 'ADDITIVE', 'ALPHA_ADDITIVE', 'ALPHA'])

    def _sort_cameras(self, cameras):
        def split_by_size(cams):
            sizes = []
            for cam in cams:
                if cam.transform.grid_size not in sizes:
                    sizes.append(cam.transform.grid_size)
            return [(size, [cam for cam in cams if cam.transform.grid_size == size]) for size in sizes]
        static_cams = split_by_size([c for c in cameras if c.static is not None])
        non_static_cams = split_by_size([c for c in cameras if c.static is None])
        return non_static_cams, static_cams

    def _get_camera_params_batch(self, cameras):
        M_V = [camera.view_matrix().transpose() for camera in cameras]
        M_P = [camera.projection_matrix().transpose() for camera in cameras]
        F = [camera.frustum() for camera in cameras]
        return M_V, M_P, F

    def get_camera_LuT(self, grid_transform, cam, inverse=False):
        M_model = grid_transform.get_transform_matrix().transpose()
        V, P, F = self._get_camera_params_batch([cam])
        MV = [M_model @ v for v in V]
        if inverse:
            in_shape, out_shape = cam.transform.grid_size, grid_transform.grid_size
        else:
            in_shape, out_shape = grid_transform.grid_size, cam.transform.grid_size
        return sampling_ops.lod_transform(input_shape=in_shape, matrix_mv=MV, matrix_p=P, frustum_params=F,
                                          output_shape=out_shape, inverse_transform=inverse)

    def _sample_transform(self, data, from_transformations, to_transformations, inverse=False, fix_scale_center=False):
        """TRANSFORM / TRANSFORM_REVERSE resampling between grids (renderer.py:186-236)."""
        with self.profiler.sample('sample_transform'):
            CM = {False: 'TRANSFORM', True: 'TRANSFORM_REVERSE'}
            M = [t.get_transform_matrix().transpose() for t in from_transformations]
            if fix_scale_center:
                V = [(GridTransform(t.grid_size, scale=[2, 2, 2], center=True, normalize='ALL').get_transform_matrix()
                      @ t.get_inverse_transform()).transpose() for t in to_transformations]
            else:
                V = [t.get_inverse_transform().transpose() for t in to_transformations]
            P = [t.identity_matrix() for t in to_transformations]
            F = [[-1, 1, -1, 1, 1, -1] for t in to_transformations]
            out_shape = from_transformations[0].grid_size if inverse else to_transformations[0].grid_size
            if self.sample_gradients:
                return _InverseSampleGrad.apply(data, M, V, P, F, out_shape, CM[inverse], CM[not inverse], self,
                                                self.storage_dtype)
            return sampling_ops.sample_grid_transform(input=data, matrix_m=M, matrix_v=V, matrix_p=P, frustum_params=F,
                                                      output_shape=out_shape, interpolation=self.filter_mode,
                                                      boundary=self.boundary_mode, mipmapping=self.mip_mode,
                                                      num_mipmaps=self.num_mips, mip_bias=self.mip_bias,
                                                      coordinate_mode=CM[inverse], storage_dtype=self.storage_dtype)

    def _sample_camera_transform(self, data, transformations, cameras, inverse=False):
        """LINDEPTH frustum resampling (renderer.py:240-281)."""
        with self.profiler.sample('sample_camera_transform'):
            CM = {False: 'TRANSFORM_LINDEPTH', True: 'TRANSFORM_LINDEPTH_REVERSE'}
            M = [t.get_transform_matrix().transpose() for t in transformations]
            V, P, F = self._get_camera_params_batch(cameras)
            out_shape = transformations[0].grid_size if inverse else cameras[0].transform.grid_size
            if self.sample_gradients:
                return _InverseSampleGrad.apply(data, M, V, P, F, out_shape, CM[inverse], CM[not inverse], self,
                                                self.storage_dtype)
            return sampling_ops.sample_grid_transform(input=data, matrix_m=M, matrix_v=V, matrix_p=P, frustum_params=F,
                                                      output_shape=out_shape, interpolation=self.filter_mode,
                                                      boundary=self.boundary_mode, mipmapping=self.mip_mode,
                                                      num_mipmaps=self.num_mips, mip_bias=self.mip_bias,
                                                      coordinate_mode=CM[inverse], storage_dtype=self.storage_dtype)

    def _raymarch_camera_transform(self, data, transformations, cameras, **kwargs):
        with self.profiler.sample('raymarch_camera_transform'):
            M = [t.get_transform_matrix().transpose() for t in transformations]
            V, P, F = self._get_camera_params_batch(cameras)
            return raymarching_ops.raymarch_grid_transform(
                input=data, matrix_m=M, matrix_v=V, matrix_p=P, frustum_params=F,
                output_shape=cameras[0].transform.grid_size,
                interpolation=kwargs.get('filter_mode', self.filter_mode),
                boundary=kwargs.get('boundary_mode', self.boundary_mode),
                blending_mode=kwargs.get('blend_mode', self.blend_mode), storage_dtype=self.storage_dtype)

    @staticmethod
    def _check_batch(data, transformations, cameras):
        if data.dim() != 5:
            raise ValueError('data must be 5D (NDHWC)')
        if not isinstance(transformations, Iterable):
            transformations = [transformations]
            if data.shape[0] != 1:
                raise ValueError('transformation and data batch size mismatch.')
            no_batch = True
        else:
            if len(transformations) != data.shape[0]:
                raise ValueError('transformation and data batch size mismatch.')
            no_batch = False
        if not isinstance(cameras, Iterable):
            cameras = [cameras]
        if len(cameras) > 1 and not all(cam.transform.grid_size == cameras[0].transform.grid_size for cam in cameras[1:]):
            raise ValueError('all cameras must have the same resolution (DHW). (use Renderer._sort_cameras() for batching.)')
        return transformations, cameras, no_batch

    @staticmethod
    def _step_scale(data, use_step_channel, cameras, allow_post):
        """Depth-step pre-multiplication of renderer.py:355-376 / :420-437."""
        C = data.shape[-1]
        if use_step_channel is None or (not np.isscalar(use_step_channel) and list(use_step_channel) == []):
            return data, None
        if np.isscalar(use_step_channel):
            return data * use_step_channel, None
        step_channel = sorted([_ % C for _ in use_step_channel if -C <= _ < C])
        depth_steps = [cam.depth_step for cam in cameras]
        if all(step == depth_steps[0] for step in depth_steps):
            if step_channel == list(range(C)):
                return data * depth_steps[0], None
            scale = torch.tensor([(depth_steps[0] if _ in step_channel else 1) for _ in range(C)], dtype=torch.float32,
                                 device=data.device)
            return data * scale, None
        if not allow_post:
            raise ValueError('All cameras must have the same step size for batched rendering.')
        return data, (step_channel, depth_steps)

    def sample_camera(self, data, transformations, cameras, inverse=False, allow_static=True, force_static=False,
                      use_step_channel=None):
        transformations, cameras, no_batch = self._check_batch(data, transformations, cameras)
        data, post = self._step_scale(data, use_step_channel, cameras, allow_post=True)
        sampled = self._sample_camera_transform(data, transformations, cameras, inverse)  # NVDHWC
        if post is not None:
            step_channel, depth_steps = post
            C = sampled.shape[-1]
            step = torch.tensor([[(s if _ in step_channel else 1.0) for _ in range(C)] for s in depth_steps],
                                dtype=torch.float32, device=sampled.device).view(1, len(depth_steps), 1, 1, 1, C)
            sampled = sampled * step
        return sampled.squeeze(0) if no_batch else sampled

    def raymarch_camera(self, data, transformations, cameras, use_step_channel=None, **raymarch_kwargs):
        transformations, cameras, no_batch = self._check_batch(data, transformations, cameras)
        data, _ = self._step_scale(data, use_step_channel, cameras, allow_post=False)
        sampled = self._raymarch_camera_transform(data, transformations, cameras, **raymarch_kwargs)
        return sampled.squeeze(0) if no_batch else sampled

    def _sample_LuT(self, data, luts, combined_batch=False, relative=False, normalized=False, cell_center_offset=0.0):
        """Lookup resampling, e.g. for warping (renderer.py:445-460)."""
        with self.profiler.sample('sample_LuT'):
            if luts.shape[-1] == 3:  # pad LoD 0
                luts = torch.nn.functional.pad(luts, (0, 1))
            if luts.shape[-1] != 4:
                raise ValueError('lookup table must have 3 or 4 channels')
            resampled = sampling_ops.sample_grid_lut(input=data, lookup=luts.contiguous(), interpolation=self.filter_mode,
                                                     boundary=self.boundary_mode, mipmapping=self.mip_mode,
                                                     num_mipmaps=self.num_mips, mip_bias=self.mip_bias,
                                                     coordinate_mode='LOOKUP', separate_camera_batch=not combined_batch,
                                                     cell_center_offset=cell_center_offset, relative_coords=relative,
                                                     normalized_coords=normalized)
        return resampled.squeeze(1) if combined_batch else resampled

    def _blend_grid(self, data, blend_mode=None, keep_dims=False):
        """Depth blending of a frustum grid (renderer.py:463-526)."""
        with self.profiler.sample('_blend_grid'):
            if blend_mode is None:
                blend_mode = self.blend_mode
            bm = blend_mode.upper()
            if bm == 'MAX':
                return torch.amax(data, dim=-4, keepdim=keep_dims)
            if bm == 'MEAN':
                return torch.mean(data, dim=-4, keepdim=keep_dims)
            if bm == 'MIN':
                return torch.amin(data, dim=-4, keepdim=keep_dims)
            if bm == 'BEER_LAMBERT':
                if data.shape[-1] == 1:
                    return torch.cumsum(data, dim=-4) if keep_dims else torch.sum(data, dim=-4)
                light, density = torch.split(data, [data.shape[-1] - 1, 1], dim=-1)
                dens_sum = torch.cumsum(density, dim=-4)
                if keep_dims:
                    return torch.cat([torch.cumsum(light * torch.exp(-dens_sum), dim=-4), dens_sum], dim=-1)
                return torch.cat([torch.sum(light * torch.exp(-dens_sum), dim=-4), dens_sum[..., -1, :, :, :]], dim=-1)
            shape = data.shape
            flat = data.reshape((-1,) + tuple(shape[-4:]))
            y = blending_ops.reduce_grid_blend(flat, blend_mode, keep_dims)
            return y.reshape(tuple(shape[:-4]) + tuple(y.shape[1:]))

    def _tonemap(self, image, mode='NONE', **kwargs):
        mode = mode.upper()
        if mode == 'NONE':
            return image
        if mode == 'CLIP_NEGATIVE':
            return torch.clamp_min(image, 0)
        if mode == 'SATURATE':
            return torch.clamp(image, 0, 1)
        if mode == 'NORMALIZE':
            mn = torch.min(image)
            if mn < 0:
                image = image - mn
            mx = torch.max(image)
            return image / mx if mx > 0 else image
        raise ValueError(mode)

    def _apply_custom_ops(self, tensor, custom_ops, name):
        result = tensor
        if custom_ops is not None and name in custom_ops:
            ops = custom_ops[name]
            if isinstance(ops, Iterable):
                for op in ops:
                    result = op(result)
            else:
                result = ops(result)
        return result

    def _render_cameras(self, light_density, grid_transform, cameras, camera_size, custom_ops=None):
        light_density = self._apply_custom_ops(light_density, custom_ops, 'GRID')
        step = [0, 1, 2, 3] if self.blend_mode not in ['MAX', 'MEAN', 'MIN'] else None
        if self.can_render_fused and ((custom_ops is None) or ('FRUSTUM' not in custom_ops)):
            with self.profiler.sample('Sampling & Reduction'):
                image_hdr = self.raymarch_camera(light_density, grid_transform, cameras, use_step_channel=step)
        else:
            with self.profiler.sample('Sampling'):
                frustum_grid = self.sample_camera(light_density, grid_transform, cameras, False, use_step_channel=step)
            frustum_grid = self._apply_custom_ops(frustum_grid, custom_ops, 'FRUSTUM')
            with self.profiler.sample('Reduction'):
                image_hdr = self._blend_grid(frustum_grid, self.blend_mode)
        return self._apply_custom_ops(image_hdr, custom_ops, 'IMAGE')

    def _build_light_grid(self, density_transform, light_list, monochrome=False):
        from .lighting import Light
        with self.profiler.sample('Lighting'):
            if len(light_list) == 0:
                raise ValueError('light list is empty')
            D, H, W = density_transform.grid_size
            c = 1 if monochrome else 3
            dens = density_transform.data
            light_data = torch.zeros((1, D, H, W, c), dtype=torch.float32, device=dens.device)
            for i, light in enumerate(light_list):
                if isinstance(light, Light):
                    light_grid = light.grid_lighting(density_transform, self)
                    if monochrome and not light.monochrome:
                        light_grid = torch.sum(light_grid * torch.tensor(self.luma, dtype=torch.float32,
                                                                         device=dens.device), dim=-1, keepdim=True)
                    if not monochrome and light.monochrome:
                        light_grid = light_grid.expand(1, D, H, W, c)
                elif isinstance(light, (torch.Tensor, np.ndarray)):
                    lt = torch.as_tensor(light, dtype=torch.float32, device=dens.device)
                    if lt.shape[-1] == 3 and monochrome:
                        lt = torch.sum(lt * torch.tensor(self.luma, device=dens.device), dim=-1, keepdim=True)
                    light_grid = lt.expand(1, D, H, W, c)
                else:
                    raise ValueError("Type of light {} '{}' is not supported.".format(i, type(light).__name__))
                light_data = light_data + light_grid
        return light_data

    def resample_grid3D_aligned(self, data, target_shape, align_x='BORDER', align_y='BORDER', align_z='BORDER'):
        """Resize a grid with the TRANSFORM sampler (renderer.py:653-690).
        align: BORDER, CENTER, STAGGER_INPUT or STAGGER_OUTPUT per axis."""
        if data.dim() != 5 or len(target_shape) != 3:
            raise ValueError('input must be NDHWC and target_shape DHW')
        N, D, H, W, _ = data.shape
        tz, ty, tx = target_shape

        def get_scale(align, in_size, out_size):
            a = align.upper()
            if a == 'BORDER':
                return 2. / in_size
            if a == 'CENTER':
                return 2. / out_size * (out_size - 1.) / (in_size - 1.)
            if a == 'STAGGER_INPUT':
                return 2. / (in_size - 1.)
            if a == 'STAGGER_OUTPUT':
                return 2. / (in_size + 1.)
            raise ValueError('unknown alignment {}'.format(align))
        in_scale = [get_scale(align_x, W, tx), get_scale(align_y, H, ty), get_scale(align_z, D, tz)]
        in_transform = GridTransform([D, H, W], scale=in_scale, center=True)
        target_transform = GridTransform(list(target_shape))
        return self._sample_transform(data, [in_transform] * N, [target_transform]).squeeze(1)

    def resample_grid3D_offset(self, data, offsets, target_shape):
        """Shift-resample with constant per-batch offsets through the lookup
        sampler (renderer.py:693-709).  offsets (K,3) -> [N, K, D, H, W, C]."""
        offs = torch.as_tensor(np.asarray(offsets, dtype=np.float32), device=data.device)
        if offs.dim() != 2 or offs.shape[1] != 3:
            raise ValueError('Shape of offsets must be (N,3), is %s' % (tuple(offs.shape),))
        if len(target_shape) != 3:
            raise ValueError('target_shape must be (3,), is %s' % (target_shape,))
        offs = torch.nn.functional.pad(offs, (0, 1)).view(offs.shape[0], 1, 1, 1, 4)
        lut = offs.expand([offs.shape[0]] + list(target_shape) + [4]).contiguous()
        return self._sample_LuT(data, lut, relative=True)

    def render_density(self, density_transform, light_list, camera_list, cut_alpha=True, background=None,
                       monochrome=False, split_cameras=False, custom_ops=None, tonemapping='NONE'):
        """Light grid + concat density + per-resolution camera batches + background
        composite (renderer.py:603-651).  Returns one image tensor per camera."""
        with self.profiler.sample('Render'):
            light_data = self._build_light_grid(density_transform, light_list, monochrome)
            data = torch.cat([light_data, density_transform.data], dim=-1)
            cam_images = [None] * len(camera_list)
            non_static, static = self._sort_cameras(camera_list)
            for cam_size, cams in non_static + static:
                if split_cameras:
                    images = torch.cat([self._render_cameras(data, density_transform, [cam], cam_size, custom_ops)
                                        for cam in cams], dim=0)
                else:
                    images = self._render_cameras(data, density_transform, cams, cam_size, custom_ops)
                t = torch.exp(-images[..., -1:])
                if cut_alpha:
                    images = images[..., :-1]
                if background is not None:
                    bkgs = torch.stack([torch.as_tensor(background[camera_list.index(cam)], dtype=torch.float32,
                                                        device=images.device).expand(images.shape[1:])
                                        for cam in cams])
                    images = images + bkgs * t
                images = self._tonemap(images, mode=tonemapping)
                for img, cam in zip(torch.split(images, 1), cams):
                    if cam.scissor_pad is not None:
                        pads = []
                        for p in reversed(list(cam.scissor_pad)):
                            pads += list(p)
                        img = torch.nn.functional.pad(img, pads)
                    cam_images[camera_list.index(cam)] = img
            return cam_images
