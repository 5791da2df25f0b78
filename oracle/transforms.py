"""Frustum <-> object-space coordinate transforms, restated in float64.

Matrices arrive as the reference ops take them: 16 floats that the kernels read
column-major (``make_float4x4(const float*)``, vectormath.hpp:306-313;
``mat4FromArray``, transformations.hpp:37-42).  The Python callers pass
``numpy_matrix.transpose()`` (renderer.py:108-111, :243), so the flat array read
column-major is the ordinary (column-vector) matrix.  MV = V @ M
(transformations_v2.hpp:44, transformations.hpp:48).

Test infrastructure only; see the package docstring.
"""
import numpy as np


def mat_from_flat(m16):
    """Column-major 16 floats -> 4x4 float64 matrix acting on column vectors."""
    a = np.asarray(m16, dtype=np.float64).reshape(4, 4)
    return a.T.copy()


class CameraXform:
    """Per-(model, camera) constants of setTransformations/setFrustumParams
    (transformations_v2.hpp:11-55)."""

    def __init__(self, M16, V16, P16, frustum6):
        self.M = mat_from_flat(M16)
        self.V = mat_from_flat(V16)
        self.P = mat_from_flat(P16)
        self.MV = self.V @ self.M
        self.MV_inv = np.linalg.inv(self.MV)
        self.P_inv = np.linalg.inv(self.P)
        f = np.asarray(frustum6, dtype=np.float64)
        self.near, self.far = f[0], f[1]
        # c_transform.M_projection.c2.z / .c3.z  (third/fourth column, z row)
        self.p22 = self.P[2, 2]
        self.p23 = self.P[2, 3]


def _h(v3, w=1.0):
    v3 = np.asarray(v3, dtype=np.float64)
    return np.concatenate([v3, np.full(v3.shape[:-1] + (1,), w)], axis=-1)


def _apply(Mx, v4):
    return np.einsum('ij,...j->...i', Mx, v4)


def idx_to_ndc(idx, dims):
    """IDXtoNDC (transformations_v2.hpp:97-100): idx/dims*2-1, w=1."""
    return _h(np.asarray(idx, dtype=np.float64) / dims * 2.0 - 1.0)


def ndc_to_os(cam, ndc4):
    """VStoOS(NDCtoVS(ndc)) (transformations_v2.hpp:102-109)."""
    vs = _apply(cam.P_inv, ndc4)
    vs = vs / vs[..., 3:4]
    return _apply(cam.MV_inv, vs)


def idx_to_os(cam, idx, dims):
    """IDXtoOS (transformations_v2.hpp:110-112) -> (..., 3)."""
    return ndc_to_os(cam, idx_to_ndc(idx, dims))[..., :3]


def idx_to_os_lindepth(cam, idx, dims):
    """IDXtoOSlinearDepth (transformations_v2.hpp:113-123): view depth is linear
    in t = idx.z/dims.z between near and far."""
    idx = np.asarray(idx, dtype=np.float64)
    ndc = idx_to_ndc(idx, dims)
    t = idx[..., 2] / dims[2]
    z = -(cam.near + t * (cam.far - cam.near))
    ndc[..., 2] = -cam.p22 - cam.p23 / z
    return ndc_to_os(cam, ndc)[..., :3]


def os_to_ndc(cam, pos_os):
    """VStoNDC(OStoVS(p)) (transformations_v2.hpp:70-78)."""
    vs = _apply(cam.MV, _h(pos_os))
    ndc = _apply(cam.P, vs)
    return ndc / ndc[..., 3:4]


def os_to_idx(cam, pos_os, dims):
    """OStoIDX (transformations_v2.hpp:81-91)."""
    ndc = os_to_ndc(cam, pos_os)
    return (ndc[..., :3] * 0.5 + 0.5) * dims


def os_to_idx_lindepth(cam, pos_os, dims):
    """OStoIDXlinearDepth (transformations_v2.hpp:82-94)."""
    ndc = os_to_ndc(cam, pos_os)
    idx = (ndc[..., :3] * 0.5 + 0.5) * dims
    z = -cam.p23 / (ndc[..., 2] + cam.p22)
    t = -(z + cam.near) / (cam.far - cam.near)
    idx[..., 2] = t * dims[2]
    return idx


# coordinate modes of SampleGridTransform (sampling_settings.hpp:56-65 order)
LINDEPTH, LINDEPTH_REVERSE, TRANSFORM, TRANSFORM_REVERSE = 0, 1, 3, 4


def _fwd_map(cam, cm, idx, dims_in, dims_out_f):
    if cm == LINDEPTH:
        return idx_to_os_lindepth(cam, idx, dims_out_f)
    if cm == TRANSFORM:
        return idx_to_os(cam, idx, dims_out_f)
    if cm == LINDEPTH_REVERSE:
        return os_to_idx_lindepth(cam, idx, dims_in)
    if cm == TRANSFORM_REVERSE:
        return os_to_idx(cam, idx, dims_in)
    raise ValueError(cm)


def sample_positions(cam, cm, idx_coords, dims_in, dims_out, with_lod):
    """samplePos3D<CM, MIP> (sampling.hpp:58-136): position in the sampled
    grid's coordinates and, with mips, the LOD from forward differences.

    idx_coords: output cell index + 0.5 (..., 3); dims_in/dims_out (x, y, z)."""
    dims_in = np.asarray(dims_in, dtype=np.float64)
    dims_out = np.asarray(dims_out, dtype=np.float64)
    p = _fwd_map(cam, cm, idx_coords, dims_in, dims_out)
    if not with_lod:
        return np.concatenate([p, np.zeros(p.shape[:-1] + (1,))], axis=-1)
    d = []
    for a in range(3):
        e = np.zeros(3)
        e[a] = 1.0
        d.append(p - _fwd_map(cam, cm, idx_coords + e, dims_in, dims_out))
    if cm in (LINDEPTH, TRANSFORM):
        # lengths of the Jacobian rows: (d_x.x, d_y.x, d_z.x), ...
        px = np.sqrt(d[0][..., 0] ** 2 + d[1][..., 0] ** 2 + d[2][..., 0] ** 2)
        py = np.sqrt(d[0][..., 1] ** 2 + d[1][..., 1] ** 2 + d[2][..., 1] ** 2)
        pz = np.sqrt(d[0][..., 2] ** 2 + d[1][..., 2] ** 2 + d[2][..., 2] ** 2)
    else:
        # reverse modes use the lengths of the columns d_x, d_y, d_z
        px, py, pz = (np.sqrt(np.sum(di ** 2, axis=-1)) for di in d)
    dm = np.maximum(px, np.maximum(py, pz))
    with np.errstate(divide='ignore'):
        lod = np.maximum(0.0, np.log2(dm))
    return np.concatenate([p, lod[..., None]], axis=-1)


def calc_lod(cam, cm, idx_coords, dims_in, dims_out):
    """calcLoD (sampling.hpp:18-56): central differences, returns (..., 4) cell
    sizes and LOD; used by LodTransform (kComputeLoD3D, resample_grid.cu.cc:1288-1300)."""
    dims_in = np.asarray(dims_in, dtype=np.float64)
    dims_out = np.asarray(dims_out, dtype=np.float64)
    d = []
    for a in range(3):
        e = np.zeros(3)
        e[a] = 1.0
        d.append((_fwd_map(cam, cm, idx_coords - e, dims_in, dims_out) -
                  _fwd_map(cam, cm, idx_coords + e, dims_in, dims_out)) * 0.5)
    px = np.sqrt(d[0][..., 0] ** 2 + d[1][..., 0] ** 2 + d[2][..., 0] ** 2)
    py = np.sqrt(d[0][..., 1] ** 2 + d[1][..., 1] ** 2 + d[2][..., 1] ** 2)
    pz = np.sqrt(d[0][..., 2] ** 2 + d[1][..., 2] ** 2 + d[2][..., 2] ** 2)
    dm = np.maximum(px, np.maximum(py, pz))
    with np.errstate(divide='ignore'):
        lod = np.maximum(0.0, np.log2(dm))
    sizes = [np.sqrt(np.sum(di ** 2, axis=-1)) for di in d]
    return np.stack(sizes + [lod], axis=-1)
