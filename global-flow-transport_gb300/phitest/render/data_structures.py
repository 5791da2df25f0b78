"""Density / velocity grids and frame sequences with the reference's transport
API (phitest/render/data_structures.py), on torch CUDA tensors.

Only the members on the render + advect path are kept: staggered velocity
layout, centring, warping of densities (fused into one CUDA pass per stage via
gft.ops.advect) and of velocities (per staggered component, composed from the
lookup sampler like the reference), the frame-chain forward advection, and the
.npz state files of the reference (DensityGrid / VelocityGrid / State /
Sequence save and from_file, same keys and directory layout), so that a
reconstruction saved by either can resume on the other.  Statistics and
optimisation helpers are out of scope.
"""
import copy
import logging
import os

import numpy as np
import torch

LOG = logging.getLogger('Structs')


def _numpy(t):
    if isinstance(t, torch.Tensor):
        return t.detach().float().cpu().numpy()
    return np.asarray(t)

from gft import ops as _gops


def _spatial(t):
    return list(t.shape[-4:-1])


class DensityGrid:
    """data_structures.py:140-330 (subset).  ``d`` is [1, D, H, W, 1]."""

    def __init__(self, shape, d=None, inflow=None, inflow_offset=None, scale_renderer=None, device=None, hull=None,
                 inflow_mask=None, **kwargs):
        self.shape = list(shape)
        if isinstance(d, np.ndarray):
            d = torch.from_numpy(np.ascontiguousarray(d, dtype=np.float32))
        dev = torch.device(device) if device is not None else (d.device if d is not None else torch.device('cuda'))
        self._d = d.to(dev) if d is not None else torch.zeros([1] + self.shape + [1], dtype=torch.float32, device=dev)
        as_t = lambda v: torch.from_numpy(np.ascontiguousarray(v, dtype=np.float32)).to(dev) \
            if isinstance(v, np.ndarray) else v
        self.inflow = as_t(inflow)
        self.inflow_offset = list(inflow_offset) if inflow_offset is not None else None
        self.inflow_mask = as_t(inflow_mask)
        self.hull = as_t(hull)
        self.scale_renderer = scale_renderer

    def save(self, path):
        """Compressed .npz as the reference writes it (data_structures.py:332-353):
        the density [1, D, H, W, 1] as the positional array 'arr_0', plus 'hull',
        'inflow', 'inflow_mask' and 'inflow_offset' where present."""
        save = {}
        if self.hull is not None:
            save['hull'] = _numpy(self.hull)
        if self.inflow is not None:
            save['inflow'] = _numpy(self.inflow)
            if self.inflow_mask is not None:
                save['inflow_mask'] = _numpy(self.inflow_mask)
            save['inflow_offset'] = np.asarray(self.inflow_offset)
        np.savez_compressed(path, _numpy(self._d), **save)

    @classmethod
    def from_file(cls, path, scale_renderer=None, hull=None, inflow=None, inflow_offset=None, inflow_mask=None,
                  device=None, **kwargs):
        """Loads a density .npz (data_structures.py:174-194); None (with a
        warning) when it cannot be read."""
        try:
            with np.load(path) as f:
                d = f['arr_0']
                if 'hull' in f and hull is None:
                    hull = f['hull']
                if 'inflow' in f and inflow is None:
                    inflow = f['inflow']
                    if 'inflow_mask' in f and inflow_mask is None:
                        inflow_mask = f['inflow_mask']
                    if 'inflow_offset' in f and inflow_offset is None:
                        inflow_offset = f['inflow_offset'].tolist()
                grid = cls(list(d.shape[-4:-1]), d=d, inflow=inflow, inflow_offset=inflow_offset,
                           scale_renderer=scale_renderer, device=device, hull=hull, inflow_mask=inflow_mask)
        except Exception:
            LOG.warning("Failed to load density from '%s':", path, exc_info=True)
            return None
        return grid

    @property
    def d(self):
        return self._d

    def assign(self, d):
        self._d = d

    def with_inflow(self):
        """Density with the inflow region added (data_structures.py:223-233)."""
        if self.inflow is None:
            return self._d
        z, y, x = self.inflow_offset
        s = list(self.inflow.shape[-4:-1])
        pad = (0, 0, x, self.shape[2] - x - s[2], y, self.shape[1] - y - s[1], z, self.shape[0] - z - s[0])
        return self._d + torch.nn.functional.pad(self.inflow, pad)

    def warped(self, vel_grid, order=1, dt=1.0, clamp='NONE'):
        """data_structures.py:263-266."""
        if not isinstance(vel_grid, VelocityGrid):
            raise ValueError('Invalid velocity grid')
        return vel_grid.warp(self.with_inflow(), order=order, dt=dt, clamp=clamp)

    def copy_warped(self, vel_grid, order=1, dt=1.0, clamp='NONE', **kwargs):
        return DensityGrid(self.shape, d=self.warped(vel_grid, order, dt, clamp), scale_renderer=self.scale_renderer)


class VelocityGrid:
    """Staggered velocity grid (data_structures.py:380-1072, subset)."""

    @staticmethod
    def component_shapes(centered_shape):
        x_shape = list(centered_shape)
        x_shape[2] += 1
        y_shape = list(centered_shape)
        y_shape[1] += 1
        z_shape = list(centered_shape)
        z_shape[0] += 1
        return x_shape, y_shape, z_shape

    def __init__(self, centered_shape, std=0.1, x=None, y=None, z=None, scale_renderer=None, warp_renderer=None,
                 device=None, **kwargs):
        self.centered_shape = list(centered_shape)
        self.x_shape, self.y_shape, self.z_shape = VelocityGrid.component_shapes(self.centered_shape)
        dev = torch.device(device) if device is not None else torch.device('cuda')
        gen = torch.Generator(device='cpu').manual_seed(kwargs.get('seed', 0))

        def init(v, shape):
            if isinstance(v, np.ndarray):
                v = torch.from_numpy(np.ascontiguousarray(v, dtype=np.float32)).to(dev)
            if v is not None:
                if list(v.shape[-4:-1]) != shape or v.shape[-1] != 1:
                    raise ValueError('Invalid shape of velocity component on assignment')
                return v
            return ((torch.rand([1] + shape + [1], generator=gen) * 2 - 1) * abs(std)).to(dev)
        self._x = init(x, self.x_shape)
        self._y = init(y, self.y_shape)
        self._z = init(z, self.z_shape)
        self.scale_renderer = scale_renderer
        self.warp_renderer = warp_renderer
        self.lod_pad = torch.zeros([1] + self.centered_shape + [1], dtype=torch.float32, device=self._x.device)

    @classmethod
    def from_centered(cls, centered, scale_renderer=None, **kwargs):
        """Staggered grid from a centred [1,D,H,W,3] field, each component
        resampled onto its face grid with the TRANSFORM sampler
        (from_centered / _centered_to_staggered, data_structures.py:475-484, :750-768)."""
        from .transform import GridTransform
        shape = _spatial(centered)
        xs, ys, zs = cls.component_shapes(shape)
        comps = []
        for i, cs in enumerate((xs, ys, zs)):
            src = GridTransform(shape, scale=[2. / _ for _ in cs[::-1]], center=True)
            comps.append(scale_renderer._sample_transform(centered[..., i:i + 1].contiguous(), [src],
                                                          [GridTransform(cs)]).squeeze(1))
        return cls(shape, x=comps[0], y=comps[1], z=comps[2], scale_renderer=scale_renderer, device=centered.device,
                   **kwargs)

    def save(self, path):
        """Compressed .npz as the reference writes it (data_structures.py:680-681):
        'centered_shape', 'vel_x', 'vel_y', 'vel_z'."""
        np.savez_compressed(path, centered_shape=np.asarray(self.centered_shape), vel_x=_numpy(self._x),
                            vel_y=_numpy(self._y), vel_z=_numpy(self._z))

    @classmethod
    def from_file(cls, path, scale_renderer=None, warp_renderer=None, device=None, **kwargs):
        """Loads a velocity .npz (data_structures.py:487-504), including the
        legacy layout without 'centered_shape'; None (with a warning) when it
        cannot be read."""
        try:
            with np.load(path) as vel:
                if 'centered_shape' not in vel:  # legacy: derived from the x component
                    shape = list(vel['vel_x'].shape)
                    shape[-2] -= 1
                    shape = shape[1:-1]
                else:
                    shape = vel['centered_shape'].tolist()
                grid = cls(shape, x=vel['vel_x'].astype(np.float32), y=vel['vel_y'].astype(np.float32),
                           z=vel['vel_z'].astype(np.float32), scale_renderer=scale_renderer,
                           warp_renderer=warp_renderer, device=device, **kwargs)
        except Exception:
            LOG.warning("Failed to load velocity from '%s':", path, exc_info=True)
            return None
        return grid

    @property
    def x(self):
        return self._x

    @property
    def y(self):
        return self._y

    @property
    def z(self):
        return self._z

    def assign(self, x, y, z):
        self._x, self._y, self._z = x, y, z

    def centered(self, pad_lod=False, concat=True):
        """Mean of the two faces per axis (data_structures.py:819-833)."""
        h = 0.5
        vel = [(self.x[:, :, :, 1:] + self.x[:, :, :, :-1]) * h,
               (self.y[:, :, 1:] + self.y[:, :, :-1]) * h,
               (self.z[:, 1:] + self.z[:, :-1]) * h]
        if pad_lod:
            vel.append(self.lod_pad)
        return torch.cat(vel, dim=-1) if concat else vel

    def centered_lut_grid(self, dt=1.0):
        return self.centered() * (-dt)

    def _warp_settings(self):
        r = self.warp_renderer
        boundary = r.boundary_mode if r is not None else 'CLAMP'
        fused_ok = r is None or (r.filter_mode == 'LINEAR' and r.mip_mode == 'NONE')
        return boundary, fused_ok

    def warp(self, data, order=1, dt=1.0, clamp='NONE'):
        """Advect a centred grid (data_structures.py:870-905): semi-Lagrangian
        (order 1) or MacCormack (order 2) with the MC_SMOOTH / NEGATIVE clamps.
        Runs the fused CUDA advection; renderers with a non-LINEAR filter or
        mips fall back to the reference composition of lookup calls."""
        if _spatial(data) != self.centered_shape:
            raise ValueError('Shape mismatch')
        clamp = clamp.upper()
        if order not in (1, 2):
            raise ValueError("Unsupported warp order '{}'".format(order))
        if clamp == 'MC':
            raise NotImplementedError('MIM and MAX warp sampling have wrong gradients.')
        boundary, fused_ok = self._warp_settings()
        storage = getattr(self.warp_renderer, 'storage_dtype', None)
        if fused_ok:
            return _gops.advect(data, self.x, self.y, self.z, dt=dt, order=order,
                                clamp=clamp if clamp in ('MC_SMOOTH', 'NEGATIVE') else 'NONE',
                                boundary=boundary, storage_dtype=storage)
        return self.warp_composed(data, order, dt, clamp)

    def warp_composed(self, data, order=1, dt=1.0, clamp='NONE'):
        """The reference's composition of the warp from lookup calls and
        elementwise ops (data_structures.py:870-905)."""
        v = self.centered_lut_grid(dt)
        r = self.warp_renderer
        data_warped = r._sample_LuT(data, v, True, relative=True)
        clamp = clamp.upper()
        if order == 2:
            back = r._sample_LuT(data_warped, -v, True, relative=True)
            corr = data_warped + 0.5 * (data - back)
            if clamp in ('MC', 'MC_SMOOTH'):
                fm = r.filter_mode
                r.filter_mode = 'MIN'
                dmin = r._sample_LuT(data, v, True, relative=True)
                r.filter_mode = 'MAX'
                dmax = r._sample_LuT(data, v, True, relative=True)
                r.filter_mode = fm
                oob = torch.logical_or(corr < dmin, corr > dmax)
                corr = torch.where(oob, data_warped, corr)
            data_warped = corr
        if clamp == 'NEGATIVE':
            data_warped = torch.clamp_min(data_warped, 0)
        return data_warped

    # ---- velocity self-advection ------------------------------------------------
    def _sampled_to_shape(self, shape):
        """Each component resampled to ``shape`` with the TRANSFORM sampler
        (data_structures.py:797-817)."""
        from .transform import GridTransform
        scale = [2. / _ for _ in shape[::-1]]
        tx = GridTransform(self.x_shape, scale=scale, center=True)
        ty = GridTransform(self.y_shape, scale=scale, center=True)
        tz = GridTransform(self.z_shape, scale=scale, center=True)
        target = GridTransform(list(shape))
        r = self.scale_renderer
        return [r._sample_transform(self.x, [tx], [target]).squeeze(1) if shape != self.x_shape else self.x,
                r._sample_transform(self.y, [ty], [target]).squeeze(1) if shape != self.y_shape else self.y,
                r._sample_transform(self.z, [tz], [target]).squeeze(1) if shape != self.z_shape else self.z]

    def _sampled_to_component_shape(self, component, concat=True):
        """Other components shifted by half cells onto one component's faces
        (data_structures.py:835-862)."""
        component = component.upper()
        f, t = 0.5, -0.5
        r = self.warp_renderer
        out = [self.x if component == 'X' else
               r.resample_grid3D_offset(self.x, [[f, t, 0.0] if component == 'Y' else [f, 0.0, t]],
                                        self.y_shape if component == 'Y' else self.z_shape).squeeze(1),
               self.y if component == 'Y' else
               r.resample_grid3D_offset(self.y, [[t, f, 0.0] if component == 'X' else [0.0, f, t]],
                                        self.x_shape if component == 'X' else self.z_shape).squeeze(1),
               self.z if component == 'Z' else
               r.resample_grid3D_offset(self.z, [[t, 0.0, f] if component == 'X' else [0.0, t, f]],
                                        self.x_shape if component == 'X' else self.y_shape).squeeze(1)]
        return torch.cat(out, dim=-1) if concat else out

    def _lut_warp_vel(self, shape, dt=1.0):
        vel = self._sampled_to_shape(shape)
        return torch.cat([-v * dt for v in vel], dim=-1)

    def _warp_vel_component(self, data, lut, order=1, dt=1.0, clamp='NONE'):
        """data_structures.py:594-619."""
        if order < 1 or order > 2:
            raise ValueError("Unsupported warp order '{}'".format(order))
        r = self.warp_renderer
        warped = r._sample_LuT(data, lut, True, relative=True)
        clamp = clamp.upper()
        if order == 2:
            back = r._sample_LuT(warped, -lut, True, relative=True)
            corrected = warped + 0.5 * (data - back)
            if clamp in ('MC', 'MC_SMOOTH'):
                fm = r.filter_mode
                r.filter_mode = 'MIN'
                dmin = r._sample_LuT(data, lut, True, relative=True)
                r.filter_mode = 'MAX'
                dmax = r._sample_LuT(data, lut, True, relative=True)
                r.filter_mode = fm
                if clamp == 'MC':
                    raise NotImplementedError('MIM and MAX warp sampling have wrong gradients.')
                oob = torch.logical_or(corrected < dmin, corrected > dmax)
                corrected = torch.where(oob, warped, corrected)
            warped = corrected
        return warped

    def warped(self, vel_grid=None, order=1, dt=1.0, clamp='NONE'):
        """Self-advection (vel_grid None) or advection by another grid of each
        staggered component (data_structures.py:621-647)."""
        if vel_grid is not None and not isinstance(vel_grid, VelocityGrid):
            raise TypeError('Invalid VelocityGrid')
        out = []
        for comp, data, shape in (('X', self.x, self.x_shape), ('Y', self.y, self.y_shape), ('Z', self.z, self.z_shape)):
            if vel_grid is None:
                lut = torch.cat([-v * dt for v in self._sampled_to_component_shape(comp, concat=False)], dim=-1)
            else:
                lut = vel_grid._lut_warp_vel(shape, dt)
            out.append(self._warp_vel_component(data, lut, order=order, dt=dt, clamp=clamp))
        return tuple(out)

    def copy_warped(self, vel_grid=None, order=1, dt=1.0, clamp='NONE', **kwargs):
        x, y, z = self.warped(vel_grid, order, dt, clamp)
        return VelocityGrid(self.centered_shape, x=x, y=y, z=z, scale_renderer=self.scale_renderer,
                            warp_renderer=self.warp_renderer, device=x.device)


class State:
    """One frame: density + velocity (data_structures.py:1074-1240, subset)."""

    def __init__(self, density, velocity, frame=0, prev=None, next=None, transform=None, **kwargs):
        self.density = density
        self.velocity = velocity
        self.frame = frame
        self.prev = prev
        self.next = next
        self.transform = transform

    def density_advected(self, dt=1.0, order=1, clamp='NONE'):
        return self.density.warped(self.velocity, order=order, dt=dt, clamp=clamp)

    def velocity_advected(self, dt=1.0, order=1, clamp='NONE'):
        return self.velocity.copy_warped(order=order, dt=dt, clamp=clamp)

    def get_density_transform(self):
        return self.transform.copy_new_data(self.density.d)

    def save(self, path, suffix=None):
        """density.npz and velocity.npz (or density_<suffix>.npz, ...) in ``path``
        (data_structures.py:1213-1215); the directory is created if missing."""
        os.makedirs(path, exist_ok=True)
        self.density.save(os.path.join(path, 'density.npz' if suffix is None else 'density_' + suffix + '.npz'))
        self.velocity.save(os.path.join(path, 'velocity.npz' if suffix is None else 'velocity_' + suffix + '.npz'))

    @classmethod
    def from_file(cls, path, frame, transform=None, scale_renderer=None, warp_renderer=None, device=None,
                  density_filename='density.npz', velocity_filename='velocity.npz', **kwargs):
        """data_structures.py:1123-1128."""
        density = DensityGrid.from_file(os.path.join(path, density_filename), scale_renderer=scale_renderer,
                                        device=device)
        velocity = VelocityGrid.from_file(os.path.join(path, velocity_filename), scale_renderer=scale_renderer,
                                          warp_renderer=warp_renderer, device=device)
        return cls(density, velocity, frame, transform=transform)


class Sequence(list):
    """Frame chain (data_structures.py:1242-1322, subset)."""

    @property
    def sequence(self):
        return self

    @classmethod
    def from_file(cls, load_path, frames, transform=None, base_path=None, scale_renderer=None, warp_renderer=None,
                  device=None, density_filename='density.npz', velocity_filename='velocity.npz',
                  frame_callback=lambda idx, frame: None, **kwargs):
        """Frames from load_path/frame_{frame:06d}/ with prev/next links
        (data_structures.py:1241-1259)."""
        seq, prev = [], None
        for idx, frame in enumerate(frames):
            frame_callback(idx, frame)
            sub_dir = 'frame_{:06d}'.format(frame)
            state = State.from_file(os.path.join(load_path, sub_dir), frame, transform=transform,
                                    scale_renderer=scale_renderer, warp_renderer=warp_renderer, device=device,
                                    density_filename=density_filename, velocity_filename=velocity_filename)
            if base_path is not None:
                state.data_path = os.path.join(base_path, sub_dir)
                os.makedirs(state.data_path, exist_ok=True)
            state.prev = prev
            prev = state
            seq.append(state)
        for i in range(len(seq) - 1):
            seq[i].next = seq[i + 1]
        return cls(seq)

    def save(self, path=None, suffix=None):
        """Each frame into path/frame_{frame:06d}/ (or its data_path)
        (data_structures.py:1302-1307)."""
        for state in self:
            if path is None and hasattr(state, 'data_path'):
                state.save(state.data_path, suffix)
            else:
                state.save(os.path.join(path, 'frame_{:06d}'.format(state.frame)), suffix)

    def densities_advect_fwd(self, dt=1.0, order=1, clamp='NONE'):
        if clamp is None or clamp.upper() not in ('LOCAL', 'GLOBAL'):
            for i in range(1, len(self)):
                self[i].density.assign(self[i - 1].density_advected(order=order, dt=dt, clamp=clamp))
        elif clamp.upper() == 'LOCAL':
            for i in range(1, len(self)):
                self[i].density.assign(torch.clamp_min(self[i - 1].density_advected(order=order, dt=dt), 0))
        else:
            for i in range(1, len(self)):
                self[i].density.assign(self[i - 1].density_advected(order=order, dt=dt))
            for i in range(1, len(self)):
                self[i].density.assign(torch.clamp_min(self[i].density.d, 0))

    def velocities_advect_fwd(self, dt=1.0, order=1, clamp='NONE'):
        for i in range(1, len(self)):
            x, y, z = self[i - 1].velocity.warped(order=order, dt=dt, clamp=clamp)
            self[i].velocity.assign(x, y, z)
