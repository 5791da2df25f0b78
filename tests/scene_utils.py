"""Small seeded scenes shared by the parity tests."""
import numpy as np

from gft import synthetic as syn
from phitest.render.camera import Camera
from phitest.render.transform import GridTransform, Transform


def small_grid(shape_dhw, C, seed, positive=True):
    rng = np.random.default_rng(seed)
    g = rng.random((1,) + tuple(shape_dhw) + (C,)).astype(np.float32)
    if not positive:
        g -= 0.3
    return g


def small_cameras(n, res_dhw, radius=2.0, arc=150.0, fov=40.0, tilt=12.0):
    Dc, Hc, Wc = res_dhw
    cams = []
    for i in range(n):
        ang = -arc / 2 + arc * i / max(n - 1, 1) + 7.0
        t = GridTransform([Dc, Hc, Wc], translation=[0, 0, radius],
                          parent=Transform(rotation_deg=[tilt * (1 if i % 2 else -1), ang, 0]))
        cams.append(Camera(t, nearFar=[radius - 1.0, radius + 1.0], fov=fov, aspect=Wc / Hc))
    return cams


def scene(shape_dhw, n_cams, res_dhw, **kw):
    gt = GridTransform(list(shape_dhw), center=True, normalize='MIN')
    cams = small_cameras(n_cams, res_dhw, **kw)
    M = syn.model_matrix(gt)
    V, P, F = syn.camera_params(cams)
    return gt, cams, M, V, P, F


def rel_l2(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    n = np.linalg.norm(b)
    return float(np.linalg.norm(a - b) / (n if n > 0 else 1.0))


def step_scene(step):
    """The plain-array scene of a gft.pipeline.RenderAdvectStep for the FP64
    step oracle (oracle/step.py)."""
    from oracle import step as OS
    return OS.scene_of(step)
