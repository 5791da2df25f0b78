"""Perspective/orthographic cameras with the reference's API (phitest/render/camera.py).

The matrices and the cropping arithmetic restate the reference's Camera (MIT
licence) on purpose: the kernels consume these matrices and the tests compare
the crops with values recorded from the reference's own class
(tests/golden/camera.json)."""
import math

import numpy as np

from .transform import GridTransform, MatrixTransform


class Camera(object):
    """grid_transform: frustum grid (DHW = depth samples, height, width) placed at
    the camera; nearFar clip planes; fov horizontal in degrees, aspect = w/h
    (camera.py:24-92)."""

    def __init__(self, grid_transform, nearFar=(1, 10), topRightBottomLeft=(1, 1, -1, -1), fov=None,
                 aspect=1, perspective=True, static=None, jitter=None):
        self.transform = grid_transform
        self.jitter = jitter
        self.trbl = list(topRightBottomLeft)
        self.clip = list(nearFar)
        self.perspective = perspective
        if fov is not None:
            self.set_fov(fov, aspect)
        self.static = static
        self.scissor_pad = None

    def view_transform_inverse(self, with_jitter=True):
        if self.jitter is not None and with_jitter:
            jitter_position = np.random.uniform(-self.jitter, self.jitter, [3]).astype(np.float32)
            return GridTransform(self.transform.grid_size, translation=jitter_position, parent=self.transform)
        return self.transform

    def view_matrix_inverse(self, with_jitter=True):
        return self.view_transform_inverse(with_jitter).get_transform_matrix()

    def view_matrix(self, with_jitter=True):
        return self.view_transform_inverse(with_jitter).get_inverse_transform()

    def frustum(self):
        """[near, far, left, right, top, bottom] (camera.py:61-62)."""
        return np.asarray([self.clip[0], self.clip[1], self.trbl[3], self.trbl[1], self.trbl[0], self.trbl[2]],
                          dtype=np.float32)

    def set_fov(self, fov, aspect=1, vertical=False):
        half_h = np.tan(fov / 2. * np.pi / 180.) * self.clip[0]
        half_v = half_h / aspect
        if vertical:
            self.trbl = [half_h, half_v, -half_h, -half_v]
        else:
            self.trbl = [half_v, half_h, -half_v, -half_h]

    def projection_matrix(self):
        """OpenGL projection (camera.py:71-92)."""
        t, r, b, l = self.trbl
        n, f = self.clip
        if not self.perspective:
            m = np.asarray([[2 / (r - l), 0, 0, 0],
                            [0, 2 / (t - b), 0, 0],
                            [0, 0, -2 / (f - n), 0],
                            [-(r + l) / (r - l), -(t + b) / (t - b), -(f + n) / (f - n), 1]], dtype=np.float32)
        else:
            m = np.asarray([[2 * n / (r - l), 0, 0, 0],
                            [0, 2 * n / (t - b), 0, 0],
                            [(r + l) / (r - l), (t + b) / (t - b), -(f + n) / (f - n), -1],
                            [0, 0, -2 * f * n / (f - n), 0]], dtype=np.float32)
        return m.transpose()

    @property
    def depth_step(self):
        """View-space step between depth samples: (far - near) / D (camera.py:95-97)."""
        return (self.far - self.near) / self.transform.grid_size[0]

    @property
    def near(self):
        return self.clip[0]

    @property
    def far(self):
        return self.clip[1]

    @property
    def top(self):
        return self.trbl[0]

    @property
    def right(self):
        return self.trbl[1]

    @property
    def bottom(self):
        return self.trbl[2]

    @property
    def left(self):
        return self.trbl[3]

    @property
    def position_global(self):
        return self.transform.position_global()

    @property
    def pix_height_near(self):
        """Pixel height on the near plane (camera.py:98-101)."""
        return (self.top - self.bottom) / self.transform.grid_size[1]

    @property
    def pix_width_near(self):
        return (self.right - self.left) / self.transform.grid_size[2]

    @property
    def view_height(self):
        return self.top - self.bottom

    @property
    def view_width(self):
        return self.right - self.left

    @property
    def aspect(self):
        """view height / view width (camera.py:154-156)."""
        return self.view_height / self.view_width

    def _project_on_near(self, pos_view, near=None):
        """Intercept theorem onto the plane z = -near, in float32 as the
        reference computes it (camera.py:164-170)."""
        near = self.near if near is None else near
        p = np.asarray(pos_view, dtype=np.float32)[:3]
        return p * (near / (-p[2]))

    def _view_positions(self, coordinate_list):
        view = MatrixTransform(self.view_matrix())
        pos_view = [view.transform(p) for p in coordinate_list]
        return pos_view, np.asarray([p[2] for p in pos_view])

    def project_world_to_screenUV(self, pos_world):
        """Screen UV in [0, 1]^2 of a world position (camera.py:172-179)."""
        p = np.asarray(pos_world, dtype=np.float64)
        if p.shape[0] == 3:
            p = np.concatenate([p, [1.0]])
        pv = MatrixTransform(self.view_matrix(with_jitter=False)).transform(p)
        pn = self._project_on_near(pv)
        return (pn[:2] - np.asarray([self.left, self.bottom])) / np.asarray([self.view_width, self.view_height])

    def project_world_to_screenPIX(self, pos_world):
        return self.project_world_to_screenUV(pos_world) * np.asarray([self.transform.grid_size[2],
                                                                       self.transform.grid_size[1]])

    def copy_clipped_to_world_coords(self, coordinate_list, preserve_aspect=True, pad=0.0, clamp_to_original=True,
                                     preserve_clip=False):
        """Copy whose near/far and top/right/bottom/left are the hull of the
        given world positions (w = 1) clipped to this camera's, at the same
        resolution (a higher spatial resolution), and the scissor rectangle of
        the copy in this camera's normalised screen ((l, b), (r, t))
        (camera.py:277-354).  Used to fit the render and shadow frusta to the
        density's bounding box so that fewer rays miss the grid."""
        pos_view, z = self._view_positions(coordinate_list)
        if not preserve_clip:
            near = np.amin(-z) - pad
            far = np.amax(-z) + pad
            if clamp_to_original:
                near = np.clip(near, self.near, self.far)
                far = np.clip(far, self.near, self.far)
        else:
            near, far = self.near, self.far
        n_scale = near / self.near
        pt, pr, pb, pl = self.top * n_scale, self.right * n_scale, self.bottom * n_scale, self.left * n_scale
        xy = np.asarray([self._project_on_near(p, near) for p in pos_view])
        x, y = xy[:, 0], xy[:, 1]
        t, r, b, l = np.amax(y) + pad, np.amax(x) + pad, np.amin(y) - pad, np.amin(x) - pad
        if clamp_to_original:
            t, r, b, l = np.clip(t, pb, pt), np.clip(r, pl, pr), np.clip(b, pb, pt), np.clip(l, pl, pr)
        if preserve_aspect:
            h, v = t - b, r - l
            a_v = h / self.aspect
            if a_v < v:
                d_h_half = (v * self.aspect - h) / 2.0
                t += d_h_half
                b -= d_h_half
            else:
                d_v_half = (a_v - v) / 2.0
                r += d_v_half
                l -= d_v_half
        H, W = pt - pb, pr - pl
        scissor_rect = (((l - pl) / W, (b - pb) / H), ((r - pl) / W, (t - pb) / H))
        cam = Camera(self.transform.copy_no_data(), nearFar=[near, far], topRightBottomLeft=[t, r, b, l],
                     perspective=self.perspective, static=self.static, jitter=self.jitter)
        return cam, scissor_rect

    def copy_with_frustum_crop(self, coordinate_list, pad=0):
        """Copy cropped to the hull of the given world positions (w = 1),
        snapped outwards to this camera's sampling grid (depth steps, pixels)
        and padded by ``pad`` cells, with its frustum grid reduced to match; its
        ``scissor_pad`` ((top, bottom), (left, right), (0, 0)) pads a rendered
        crop back to this camera's image (camera.py:356-437).  The crop's grid
        height and width are its extents divided by the depth step, as the
        reference computes them (camera.py:420-427), which equals the pixel
        count where pixels and depth steps have the same size."""
        def round_up(v, base, offset):
            return math.ceil((v - offset) / base) * base + offset

        def round_down(v, base, offset):
            return math.floor((v - offset) / base) * base + offset

        pos_view, z = self._view_positions(coordinate_list)
        n, f = np.amin(-z), np.amax(-z)
        pix_depth = self.depth_step
        n = round_down(n, pix_depth, self.near)
        f = round_up(f, pix_depth, self.far)
        n = np.clip(n - pix_depth * pad, self.near, self.far)
        f = np.clip(f + pix_depth * pad, self.near, self.far)
        grid_z = int(round((f - n) / pix_depth))
        n_scale = n / self.near
        pt, pr, pb, pl = self.top * n_scale, self.right * n_scale, self.bottom * n_scale, self.left * n_scale
        xy = np.asarray([self._project_on_near(p, n) for p in pos_view])
        x, y = xy[:, 0], xy[:, 1]
        t, r, b, l = np.amax(y), np.amax(x), np.amin(y), np.amin(x)
        pix_height = self.pix_height_near * n_scale
        t = round_up(t, pix_height, pb)
        b = round_down(b, pix_height, pb)
        pix_width = self.pix_width_near * n_scale
        r = round_up(r, pix_width, pl)
        l = round_down(l, pix_width, pl)
        t = np.clip(t + pix_height * pad, pb, pt)
        b = np.clip(b - pix_height * pad, pb, pt)
        grid_y = int(round((t - b) / pix_depth))
        offset_y = int(round((b - pb) / pix_depth))
        r = np.clip(r + pix_width * pad, pl, pr)
        l = np.clip(l - pix_width * pad, pl, pr)
        grid_x = int(round((r - l) / pix_depth))
        offset_x = int(round((l - pl) / pix_depth))
        img_pad = [(offset_y, self.transform.grid_size[1] - grid_y - offset_y),
                   (offset_x, self.transform.grid_size[2] - grid_x - offset_x), (0, 0)]
        transform = self.transform.copy_no_data()
        transform.grid_size = [grid_z, grid_y, grid_x]
        cam = Camera(transform, nearFar=[n, f], topRightBottomLeft=[t, r, b, l], perspective=self.perspective,
                     static=self.static, jitter=self.jitter)
        cam.scissor_pad = img_pad
        return cam
