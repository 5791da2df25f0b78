"""Lights with the reference's API (phitest/render/lighting.py) on torch tensors."""
import numpy as np
import torch

from .camera import Camera
from .transform import GridTransform


def _density(density_transform):
    return density_transform.data


class Light(object):
    """Ambient light: density * colour * intensity (lighting.py:10-26)."""

    def __init__(self, color=(1., 1., 1.), intensity=1.):
        self.c = np.asarray(color, dtype=np.float32)
        self.i = intensity

    @property
    def monochrome(self):
        return np.isscalar(self.c) or np.asarray(self.c).shape == (1,)

    def _color(self, dev):
        return torch.as_tensor(self.c * np.float32(self.i), dtype=torch.float32, device=dev)

    def grid_lighting(self, density_transform, renderer=None, scattering_func=None):
        d = _density(density_transform)
        return d * self._color(d.device)


class PointLight(Light):
    """Inverse-square-like falloff 1/(1+(r*s)^2) in world-scaled grid units
    (lighting.py:49-71)."""

    def __init__(self, transform, color=(1., 1., 1.), intensity=1., range_scale=1, range_limit=0):
        super().__init__(color, intensity)
        self.t = transform
        self.r = range_limit
        self.s = range_scale

    def falloff(self, density_transform, device):
        D, H, W = density_transform.grid_size
        cs = density_transform.cell_size_world()
        gs = density_transform.grid_size_world()
        light_pos_ws = self.t.position_global()
        pos_os = (density_transform.get_inverse_transform() @ light_pos_ws)[:3]
        pos_scaled = pos_os * cs
        xs = torch.linspace(0.5 * cs[0], gs[0] - 0.5 * cs[0], W, dtype=torch.float32, device=device)
        ys = torch.linspace(0.5 * cs[1], gs[1] - 0.5 * cs[1], H, dtype=torch.float32, device=device)
        zs = torch.linspace(0.5 * cs[2], gs[2] - 0.5 * cs[2], D, dtype=torch.float32, device=device)
        rel = torch.stack(torch.meshgrid(zs - float(pos_scaled[2]), ys - float(pos_scaled[1]),
                                         xs - float(pos_scaled[0]), indexing='ij'), dim=-1)
        r = torch.linalg.norm(rel, dim=-1, keepdim=True)
        return 1.0 / (1.0 + torch.pow(r * self.s, 2.0))  # [D,H,W,1]

    def grid_lighting(self, density_transform, renderer=None, scattering_func=None):
        d = _density(density_transform)
        return d * (self.falloff(density_transform, d.device) * self._color(d.device))


class SpotLight(PointLight):
    """Point light with a light-frustum shadow pass (lighting.py:73-147)."""

    def __init__(self, transform, color=(1., 1., 1.), intensity=1., range_scale=1, range_limit=0, angle_deg=45,
                 cast_shadows=False, shadow_resolution=(64, 64, 64), shadow_clip=(1, 10), cone_mask=True, static=None):
        super().__init__(transform, color, intensity, range_scale, range_limit)
        self.a = angle_deg
        self.cast_shadows = cast_shadows
        self.shadow_resolution = list(shadow_resolution)
        self.shadow_cam = Camera(GridTransform.from_transform(transform, self.shadow_resolution), shadow_clip,
                                 fov=self.a, static=static)
        self.cone_mask = cone_mask

    def _get_shadow_mask(self, device):
        a = torch.linspace(-1., 1., self.shadow_resolution[1], device=device)
        b = torch.linspace(-1., 1., self.shadow_resolution[2], device=device)
        m = torch.stack(torch.meshgrid(a, b, indexing='ij'), dim=-1)
        return (torch.linalg.norm(m, dim=-1, keepdim=True) <= 1).float()

    def _render_shadow_map(self, density_transform, renderer):
        d = _density(density_transform)
        if self.cast_shadows:
            shadow = renderer.sample_camera(d, density_transform, self.shadow_cam, inverse=False, use_step_channel=[0])
            shadow = renderer.blending.reduce_grid_blend(shadow, renderer.blend_mode, keep_dims=True)
            # shift by one cell into depth (lighting.py:114-126)
            if renderer.boundary_mode == 'BORDER':
                pad = torch.zeros_like(shadow[..., :1, :, :, :])
            elif renderer.boundary_mode == 'CLAMP':
                pad = shadow[..., :1, :, :, :]
            elif renderer.boundary_mode == 'WRAP':
                pad = shadow[..., -1:, :, :, :]
            else:
                raise ValueError('Unknow boundary_mode %s' % renderer.boundary_mode)
            shadow = torch.cat([pad, shadow[..., :-1, :, :, :]], dim=-4)
            if renderer.blend_mode == 'BEER_LAMBERT':
                transmission = torch.exp(-shadow)
            elif renderer.blend_mode == 'ALPHA':
                transmission = 1 - torch.clamp(shadow, 0, 1)
            else:
                raise ValueError("Unknown blend_mode '{}'".format(renderer.blend_mode))
        else:
            transmission = torch.ones([1] + self.shadow_resolution + [1], dtype=torch.float32, device=d.device)
        if self.cone_mask:
            transmission = transmission * self._get_shadow_mask(d.device)
        transmission = renderer.sample_camera(transmission.contiguous(), density_transform, self.shadow_cam,
                                              inverse=True, use_step_channel=None)
        return transmission.squeeze(0)

    def grid_lighting(self, density_transform, renderer, scattering_func=None):
        light = self._render_shadow_map(density_transform, renderer)
        return light * super().grid_lighting(density_transform, renderer=renderer, scattering_func=scattering_func)
