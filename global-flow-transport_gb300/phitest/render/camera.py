"""Perspective/orthographic cameras with the reference's API (phitest/render/camera.py)."""
import numpy as np

from .transform import GridTransform


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
