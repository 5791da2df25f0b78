"""Scene transforms with the reference's API (phitest/render/transform.py).

Matrices follow the reference convention: 4x4 float32 numpy arrays acting on
column vectors; ``get_transform_matrix`` composes parents on the left
(transform.py:122-126).  The render ops take ``matrix.transpose()`` flattened,
which the kernels read column-major.
"""
import copy

import numpy as np
from scipy.spatial.transform import Rotation


def _rotation_dcm(rotation_deg):
    r = Rotation.from_euler('xyz', rotation_deg, degrees=True)
    # scipy renamed as_dcm -> as_matrix; the reference calls as_dcm (transform.py:53)
    return r.as_matrix() if hasattr(r, 'as_matrix') else r.as_dcm()


class MatrixTransform(object):
    def __init__(self, transform_matrix=None, parent=None, grid_size=None, static=False):
        self._matrix = transform_matrix if transform_matrix is not None else self.identity_matrix()
        if parent is not None and not isinstance(parent, MatrixTransform):
            raise TypeError("parent must be a Transform object or None.")
        self.parent = parent
        self.grid_size = grid_size

    @staticmethod
    def translation_matrix(translation):
        m = np.eye(4, dtype=np.float32)
        m[:3, 3] = np.asarray(translation, dtype=np.float32)[:3]
        return m

    @staticmethod
    def rotation_matrix(rotation):
        rot = np.pad(_rotation_dcm(rotation), (0, 1), mode='constant')
        rot[-1, -1] = 1
        return rot

    @staticmethod
    def scale_matrix(scale):
        m = np.eye(4, dtype=np.float32)
        m[0, 0], m[1, 1], m[2, 2] = [np.float32(s) for s in scale[:3]]
        return m

    @staticmethod
    def identity_matrix():
        return np.eye(4, dtype=np.float32)

    def set_parent(self, parent_transform):
        if parent_transform is not None and not isinstance(parent_transform, MatrixTransform):
            raise TypeError("parent must be a Transform object or None.")
        self.parent = parent_transform

    def copy_no_data(self):
        return copy.deepcopy(self)

    def get_local_transform(self):
        return self._matrix

    def get_transform_matrix(self):
        if self.parent is not None:
            return self.parent.get_transform_matrix() @ self.get_local_transform()
        return self.get_local_transform()

    def get_inverse_transform(self):
        return np.linalg.inv(self.get_transform_matrix())

    def inverse(self):
        return MatrixTransform(self.get_inverse_transform())

    def position_global(self):
        return self.get_transform_matrix() @ np.asarray([0, 0, 0, 1])

    def forward_global(self):
        v = self.get_transform_matrix() @ np.asarray([0, 0, 1, 0])
        return v / np.linalg.norm(v)

    def up_global(self):
        v = self.get_transform_matrix() @ np.asarray([0, 1, 0, 0])
        return v / np.linalg.norm(v)

    def right_global(self):
        v = self.get_transform_matrix() @ np.asarray([1, 0, 0, 0])
        return v / np.linalg.norm(v)

    def transform(self, vector):
        return self.get_transform_matrix() @ np.asarray(vector)

    def transform_AABB(self, corner_min=(0, 0, 0), corner_max=(1, 1, 1), expand_corners=False):
        """World positions (w = 1) of an axis-aligned box's corners: min and max,
        or all 8 with expand_corners, in the order of transform.py:104-117."""
        a, b = [float(v) for v in corner_min], [float(v) for v in corner_max]
        pts = [(a[0], a[1], a[2])]
        if expand_corners:
            pts += [(b[0], a[1], a[2]), (a[0], b[1], a[2]), (a[0], a[1], b[2]), (b[0], b[1], a[2]),
                    (b[0], a[1], b[2]), (a[0], b[1], b[2])]
        pts.append((b[0], b[1], b[2]))
        return [self.transform([x, y, z, 1]) for x, y, z in pts]

    def __eq__(self, other):
        return np.array_equal(self.get_transform_matrix(), other.get_transform_matrix())


class Transform(MatrixTransform):
    def __init__(self, translation=(0, 0, 0), rotation_deg=(0, 0, 0), scale=(1, 1, 1), parent=None, static=False):
        self.translation = list(translation)
        self.rotation_deg = list(rotation_deg)
        self.scale = list(scale)
        self.parent = parent
        self.grid_size = None

    def get_local_transform(self):
        M_scale = Transform.scale_matrix(self.scale)
        M_rot = Transform.rotation_matrix(self.rotation_deg)
        M_trans = Transform.translation_matrix(self.translation)
        return M_trans @ (M_rot @ M_scale)


class GridTransform(Transform):
    """Grid placement: T * R * [norm-scale] * S * [centre] (transform.py:253-267).
    grid_size is DHW (z, y, x); object-space coordinates are xyz in [0, size]."""

    def __init__(self, grid_size, translation=(0, 0, 0), rotation_deg=(0, 0, 0), scale=(1, 1, 1),
                 center=False, normalize='NONE', parent=None, static=False):
        super().__init__(translation, rotation_deg, scale, parent)
        self.grid_size = list(grid_size)
        self.center = center
        self.normalize = normalize
        self.data = None

    @classmethod
    def from_transform(cls, transform, grid_size, center=False, normalize='NONE'):
        return cls(grid_size, transform.translation, transform.rotation_deg, transform.scale,
                   center, normalize, transform.parent)

    def set_data(self, data, format='NDHWC'):
        shape = list(data.shape)
        self.grid_size = [int(shape[format.index(_)]) for _ in 'DHW']
        self.data = data

    def get_grid_size(self):
        return np.asarray(self.grid_size)

    def get_channel(self):
        return int(self.data.shape[-1])

    def copy_no_data(self):
        gt = copy.copy(self)
        gt.data = None
        return copy.deepcopy(gt)

    def copy_new_data(self, data):
        gt = self.copy_no_data()
        gt.set_data(data)
        return gt

    def get_local_transform(self):
        size = np.flip(self.get_grid_size()).astype(np.float64)  # xyz
        M_center = Transform.translation_matrix(-size / 2.0)
        if self.normalize == 'ALL':
            M_norm_scale = Transform.scale_matrix(1.0 / size)
        elif self.normalize == 'MIN':
            M_norm_scale = Transform.scale_matrix([1.0 / np.min(size)] * 3)
        elif self.normalize == 'MAX':
            M_norm_scale = Transform.scale_matrix([1.0 / np.max(size)] * 3)
        M_scale = Transform.scale_matrix(self.scale)
        M_rot = Transform.rotation_matrix(self.rotation_deg)
        M_trans = Transform.translation_matrix(self.translation)
        M = M_scale @ M_center if self.center else M_scale
        M = M_norm_scale @ M if self.normalize != 'NONE' else M
        return M_trans @ (M_rot @ M)

    def grid_size_world(self):
        z, y, x = self.grid_size
        return np.array([np.linalg.norm(self.transform([x, 0, 0, 0])[:3]),
                         np.linalg.norm(self.transform([0, y, 0, 0])[:3]),
                         np.linalg.norm(self.transform([0, 0, z, 0])[:3])])

    def cell_size_world(self):
        return np.array([np.linalg.norm(self.transform([1, 0, 0, 0])[:3]),
                         np.linalg.norm(self.transform([0, 1, 0, 0])[:3]),
                         np.linalg.norm(self.transform([0, 0, 1, 0])[:3])])

    def __eq__(self, other):
        return (np.array_equal(self.get_transform_matrix(), other.get_transform_matrix())
                and np.array_equal(self.get_grid_size(), other.get_grid_size()))
