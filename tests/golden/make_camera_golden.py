"""Records the reference Camera's frustum crops as golden values.

Run in a container where the reference sources are present:

    python tests/golden/make_camera_golden.py /root/reference

It loads phitest/render/{vector,serialization,transform,camera}.py of the
reference directly (TensorFlow, which vector.py imports but the camera code
does not use, is replaced by an empty module, and SciPy's Rotation.as_dcm is
aliased to its current name as_matrix), builds the cameras and density
grids of the benchmark scenes with the reference's classes, and writes the
results of Camera.copy_clipped_to_world_coords and copy_with_frustum_crop
(camera.py:277-437), together with the matrices of the cameras they return,
to tests/golden/camera.json.  tests/test_host_cpu.py reproduces every case
with phitest/render/camera.py.
"""
import importlib.util
import json
import os
import sys
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))

# (grid D, H, W; camera kind; frustum resolution D, H, W; camera count; pad)
CASES = [
    ('cfg1', (64, 64, 64), 'arc', (64, 128, 128), 1, 0),
    ('cfg2', (128, 227, 128), 'arc', (192, 270, 480), 5, 0),
    ('cfg2_pad2', (128, 227, 128), 'arc', (192, 270, 480), 5, 2),
    ('cfg4', (96, 170, 96), 'hemi', (128, 0, 0), 9, 1),
    ('cfg5', (256, 455, 256), 'arc', (256, 540, 960), 5, 0),
]


def load_reference(root):
    ref = os.path.join(root, 'phitest', 'render')
    sys.modules['tensorflow'] = types.ModuleType('tensorflow')
    # the reference was written against a SciPy whose Rotation had as_dcm
    # (renamed as_matrix since)
    from scipy.spatial.transform import Rotation
    if not hasattr(Rotation, 'as_dcm'):
        Rotation.as_dcm = Rotation.as_matrix
    pkg = types.ModuleType('refrender')
    pkg.__path__ = [ref]
    sys.modules['refrender'] = pkg
    mods = {}
    for name in ('vector', 'serialization', 'transform', 'camera'):
        spec = importlib.util.spec_from_file_location('refrender.' + name, os.path.join(ref, name + '.py'))
        m = importlib.util.module_from_spec(spec)
        sys.modules['refrender.' + name] = m
        spec.loader.exec_module(m)
        mods[name] = m
    return mods


def cameras(mods, kind, res, n, seed=4000):
    """The scenes' cameras (gft.synthetic.arc_cameras / hemisphere_cameras)
    built with the reference's classes."""
    T, C = mods['transform'], mods['camera']
    radius, fov = 2.5, 30.0
    near, far = radius - 1.2, radius + 1.2
    cams = []
    if kind == 'arc':
        Dc, Hc, Wc = res
        for i in range(n):
            ang = -120.0 / 2.0 + (120.0 * i / max(n - 1, 1))
            t = T.GridTransform([Dc, Hc, Wc], translation=[0, 0, radius], parent=T.Transform(rotation_deg=[0, ang, 0]))
            cams.append(C.Camera(t, nearFar=[near, far], fov=fov, aspect=Wc / Hc))
        return cams
    rng = np.random.default_rng(seed)
    dirs = [(0.0, 0.0)]
    for _ in range(n - 1):
        u = rng.random()
        dirs.append((float(np.degrees(np.arcsin(u))), float(rng.uniform(-180.0, 180.0))))
    for k, (elev, azim) in enumerate(dirs):
        s = 256 if k == 0 else int(rng.integers(64, 257))
        t = T.GridTransform([res[0], s, s], translation=[0, 0, radius], parent=T.Transform(rotation_deg=[-elev, azim, 0]))
        cams.append(C.Camera(t, nearFar=[near, far], fov=fov, aspect=1.0))
    return cams


def _f(a):
    return np.asarray(a, dtype=np.float64).tolist()


def main(root):
    mods = load_reference(root)
    T = mods['transform']
    out = {}
    for name, shape, kind, res, n, pad in CASES:
        gt = T.GridTransform(list(shape), center=True, normalize='MIN')
        D, H, W = shape
        corners = [np.asarray(c, dtype=np.float64) for c in gt.transform_AABB([0, 0, 0], [W, H, D], True)]
        cases = []
        for cam in cameras(mods, kind, res, n):
            clipped, rect = cam.copy_clipped_to_world_coords(corners)
            crop = cam.copy_with_frustum_crop(corners, pad)
            cases.append({
                'clipped': {'clip': _f(clipped.clip), 'trbl': _f(clipped.trbl), 'scissor_rect': _f(rect),
                            'projection': _f(clipped.projection_matrix())},
                'crop': {'clip': _f(crop.clip), 'trbl': _f(crop.trbl), 'grid_size': [int(v) for v in
                                                                                   crop.transform.grid_size],
                         'scissor_pad': [[int(a), int(b)] for a, b in crop.scissor_pad],
                         'projection': _f(crop.projection_matrix())},
            })
        out[name] = {'shape': list(shape), 'kind': kind, 'res': list(res), 'n': n, 'pad': pad,
                     'corners': [_f(c) for c in corners], 'cameras': cases}
    with open(os.path.join(HERE, 'camera.json'), 'w') as f:
        json.dump(out, f, indent=0)
    print('wrote', os.path.join(HERE, 'camera.json'))


if __name__ == '__main__':
    main(sys.argv[1] if len(sys.argv) > 1 else '/root/reference')
