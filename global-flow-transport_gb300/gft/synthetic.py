"""Seeded synthetic plume scenes standing in for the ScalarFlow data.

Density: exp(gaussian_filter(U[0,1), sigma=3 voxels)) * 0.05 masked to a rising
cylinder (axis along y, radius 0.3 W, height growing with the frame).
Velocity: curl of Gaussian-smoothed noise scaled to about one voxel per step,
plus 0.5 voxel per step upwards, sampled to the staggered faces.
Cameras: perspective views on a horizontal arc around the grid; one spot light
with a shadow frustum above the front.  Seeds follow seed = config * 1000 + frame.
"""
import numpy as np
from scipy.ndimage import gaussian_filter

from phitest.render.camera import Camera
from phitest.render.transform import GridTransform, Transform


def plume_density(shape_dhw, seed, frame=0, sigma=3.0, scale=0.05):
    D, H, W = shape_dhw
    rng = np.random.default_rng(seed)
    noise = rng.random((D, H, W), dtype=np.float32)
    d = np.exp(gaussian_filter(noise, sigma, mode='wrap')) * scale
    z = (np.arange(D, dtype=np.float32) + 0.5 - D / 2.0)[:, None, None]
    x = (np.arange(W, dtype=np.float32) + 0.5 - W / 2.0)[None, None, :]
    y = np.arange(H, dtype=np.float32)[None, :, None]
    height = H * min(1.0, 0.35 + 0.04 * frame)
    mask = (np.sqrt(x * x + z * z) <= 0.3 * W) & (y < height)
    return (d * mask).astype(np.float32)[None, ..., None]


def _faces(c, axis):
    """cell-centred -> staggered faces along axis (edge values replicated)."""
    pad = [(0, 0)] * 3
    pad[axis] = (1, 1)
    p = np.pad(c, pad, mode='edge')
    lo = [slice(None)] * 3
    hi = [slice(None)] * 3
    lo[axis] = slice(0, -1)
    hi[axis] = slice(1, None)
    return 0.5 * (p[tuple(lo)] + p[tuple(hi)])


def curl_velocity(shape_dhw, seed, magnitude=1.0, upward=0.5, sigma=4.0):
    """Staggered velocity (x [D,H,W+1], y [D,H+1,W], z [D+1,H,W]), each with a
    leading batch and trailing channel dim of 1, in voxels per step."""
    D, H, W = shape_dhw
    rng = np.random.default_rng(seed)
    A = [gaussian_filter(rng.standard_normal((D, H, W)).astype(np.float32), sigma, mode='wrap') for _ in range(3)]
    # A[0..2] = (Ax, Ay, Az); array axes (z, y, x)
    dAz_dy = np.gradient(A[2], axis=1)
    dAy_dz = np.gradient(A[1], axis=0)
    dAx_dz = np.gradient(A[0], axis=0)
    dAz_dx = np.gradient(A[2], axis=2)
    dAy_dx = np.gradient(A[1], axis=2)
    dAx_dy = np.gradient(A[0], axis=1)
    vx = dAz_dy - dAy_dz
    vy = dAx_dz - dAz_dx
    vz = dAy_dx - dAx_dy
    s = magnitude / max(1e-12, float(np.max(np.sqrt(vx * vx + vy * vy + vz * vz))))
    vx, vy, vz = vx * s, vy * s + upward, vz * s
    sx = _faces(vx, 2).astype(np.float32)[None, ..., None]
    sy = _faces(vy, 1).astype(np.float32)[None, ..., None]
    sz = _faces(vz, 0).astype(np.float32)[None, ..., None]
    return sx, sy, sz


def grid_transform(shape_dhw):
    """Density grid centred at the origin, normalised so its smallest side is 1."""
    return GridTransform(list(shape_dhw), center=True, normalize='MIN')


def arc_cameras(n_views, resolution_dhw, arc_deg=120.0, radius=2.5, fov=30.0, near=None, far=None):
    """Perspective cameras on a horizontal arc of ``arc_deg`` around the origin.
    resolution = (depth samples, height, width); fov horizontal; aspect w/h."""
    Dc, Hc, Wc = resolution_dhw
    near = radius - 1.2 if near is None else near
    far = radius + 1.2 if far is None else far
    cams = []
    for i in range(n_views):
        ang = -arc_deg / 2.0 + (arc_deg * i / max(n_views - 1, 1))
        t = GridTransform([Dc, Hc, Wc], translation=[0, 0, radius], parent=Transform(rotation_deg=[0, ang, 0]))
        cams.append(Camera(t, nearFar=[near, far], fov=fov, aspect=Wc / Hc))
    return cams


def camera_params(cams):
    """(V, P, F) arrays as Renderer._get_camera_params_batch builds them (renderer.py:107-111)."""
    V = np.stack([c.view_matrix().transpose() for c in cams]).astype(np.float32)
    P = np.stack([c.projection_matrix().transpose() for c in cams]).astype(np.float32)
    F = np.stack([c.frustum() for c in cams]).astype(np.float32)
    return V, P, F


def model_matrix(gt):
    return gt.get_transform_matrix().transpose().astype(np.float32)[None]


def hemisphere_cameras(n_random, samples, sizes=(64, 256), radius=2.5, fov=30.0, seed=0, fixed_size=256):
    """One fixed camera (on the +z axis, ``fixed_size`` square) plus
    ``n_random`` cameras at seeded uniform directions on the upper hemisphere
    with square resolutions drawn uniformly from ``sizes``; all look at the
    origin.  Returns (cameras, [(samples, h, w)] per camera)."""
    rng = np.random.default_rng(seed)
    near, far = radius - 1.2, radius + 1.2
    cams, shapes = [], []
    dirs = [(0.0, 0.0)]
    for _ in range(n_random):
        u = rng.random()
        dirs.append((float(np.degrees(np.arcsin(u))), float(rng.uniform(-180.0, 180.0))))  # elevation, azimuth
    for k, (elev, azim) in enumerate(dirs):
        s = fixed_size if k == 0 else int(rng.integers(sizes[0], sizes[1] + 1))
        t = GridTransform([samples, s, s], translation=[0, 0, radius],
                          parent=Transform(rotation_deg=[-elev, azim, 0]))
        cams.append(Camera(t, nearFar=[near, far], fov=fov, aspect=1.0))
        shapes.append((samples, s, s))
    return cams, shapes


# ---- device-side generators (for long chains of large grids) ----------------
def _gauss_wrap_device(x, sigma):
    """Periodic ('wrap') Gaussian filter of a 3-D device tensor by FFT."""
    import torch
    spec = torch.fft.rfftn(x)
    out = spec
    for axis, n in enumerate(x.shape):
        f = torch.fft.fftfreq(n, device=x.device) if axis < 2 else torch.fft.rfftfreq(n, device=x.device)
        g = torch.exp(-2.0 * (torch.pi * sigma * f) ** 2)
        shape = [1, 1, 1]
        shape[axis] = g.numel()
        out = out * g.reshape(shape)
    return torch.fft.irfftn(out, s=x.shape)


def plume_density_device(shape_dhw, seed, device, frame=0, sigma=3.0, scale=0.05):
    """plume_density generated on the device ([1, D, H, W, 1] fp32): the same
    construction with the device's random generator and an FFT Gaussian."""
    import torch
    D, H, W = shape_dhw
    g = torch.Generator(device=device).manual_seed(int(seed))
    noise = torch.rand((D, H, W), generator=g, device=device)
    d = torch.exp(_gauss_wrap_device(noise, sigma)) * scale
    z = (torch.arange(D, device=device, dtype=torch.float32) + 0.5 - D / 2.0)[:, None, None]
    x = (torch.arange(W, device=device, dtype=torch.float32) + 0.5 - W / 2.0)[None, None, :]
    y = torch.arange(H, device=device, dtype=torch.float32)[None, :, None]
    height = H * min(1.0, 0.35 + 0.04 * frame)
    mask = (torch.sqrt(x * x + z * z) <= 0.3 * W) & (y < height)
    return (d * mask).float()[None, ..., None].contiguous()


def _faces_device(c, axis):
    import torch
    lo = c.narrow(axis, 0, 1)
    hi = c.narrow(axis, c.shape[axis] - 1, 1)
    p = torch.cat([lo, c, hi], dim=axis)
    n = p.shape[axis]
    return 0.5 * (p.narrow(axis, 0, n - 1) + p.narrow(axis, 1, n - 1))


def curl_velocity_device(shape_dhw, seed, device, magnitude=1.0, upward=0.5, sigma=4.0):
    """curl_velocity generated on the device: staggered components
    [1, D, H, W+1, 1], [1, D, H+1, W, 1], [1, D+1, H, W, 1] fp32."""
    import torch
    D, H, W = shape_dhw
    g = torch.Generator(device=device).manual_seed(int(seed))
    A = [_gauss_wrap_device(torch.randn((D, H, W), generator=g, device=device), sigma) for _ in range(3)]
    dAz_dy, = torch.gradient(A[2], dim=1)
    dAy_dz, = torch.gradient(A[1], dim=0)
    dAx_dz, = torch.gradient(A[0], dim=0)
    dAz_dx, = torch.gradient(A[2], dim=2)
    dAy_dx, = torch.gradient(A[1], dim=2)
    dAx_dy, = torch.gradient(A[0], dim=1)
    vx = dAz_dy - dAy_dz
    vy = dAx_dz - dAz_dx
    vz = dAy_dx - dAx_dy
    s = magnitude / max(1e-12, float(torch.sqrt(vx * vx + vy * vy + vz * vz).max()))
    vx, vy, vz = vx * s, vy * s + upward, vz * s
    return tuple(_faces_device(v, a).float()[None, ..., None].contiguous() for v, a in ((vx, 2), (vy, 1), (vz, 0)))
