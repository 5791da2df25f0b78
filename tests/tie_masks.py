"""Voxels where the reference's advection adjoint is discontinuous in the
lookup positions, so that an FP32 kernel and the FP64 oracle may legitimately
disagree there by O(1) relative to the voxel's gradient.

* Count ties (reference-normalised mode).  SampleGridLutGrad divides each
  voxel's scattered gradient by the number of (sample, corner) pairs that
  reached it (resample_grid.cu.cc:1231-1238).  A lookup whose position lies
  within rounding of an integer along some axis reaches corners {k-1, k} or
  {k, k+1} depending on the last bit of the position, so the counts of those
  voxels -- and every gradient normalised by them -- depend on FP32 versus
  FP64 rounding.
* Derivative jumps.  The lookup (velocity) gradient is the spatial derivative
  of the trilinear fetch at the lookup, a difference of corner values that
  changes where the lookup crosses a cell boundary.
* MC_SMOOTH flips.  The MacCormack clamp selects the corrected or the
  semi-Lagrangian value by comparing the corrected value with the min / max
  of the forward footprint (data_structures.py:890-905); where the margin is
  within rounding the two precisions select different branches, and the
  gradient of that voxel (its direct term, its back-lookup scatter and the
  forward scatter of those) takes the other route.

Both are measure-zero sets of the continuous problem; the parity tests
exclude the voxels these effects can reach (following the adjoint's
dependencies) and bound their fraction.
"""
import numpy as np

from oracle import advect as OA
from oracle import resample as R
from oracle import sampling as S


def _grid_idx(shape_dhw):
    D, H, W = shape_dhw
    z, y, x = np.meshgrid(np.arange(D, dtype=np.float64), np.arange(H, dtype=np.float64),
                          np.arange(W, dtype=np.float64), indexing='ij')
    return np.stack([x, y, z], axis=-1)


def lookup_positions(vx, vy, vz, dt=1.0, sign=1.0):
    """FP64 positions of the forward (sign +1: x - dt*v) or back (sign -1:
    x + dt*v) lookup of every voxel, (D,H,W,3) in (x, y, z)."""
    vb = OA.centered(vx, vy, vz)
    return _grid_idx(vb.shape[:3]) + sign * (-dt) * vb


def _mark(mask, x, y, z):
    D, H, W = mask.shape
    mask[np.clip(z, 0, D - 1), np.clip(y, 0, H - 1), np.clip(x, 0, W - 1)] = True


def _corners(pos):
    """The 8 trilinear corner cells (x, y, z index arrays) of every position."""
    b = np.floor(pos).astype(np.int64)
    for k in range(8):
        yield b[..., 0] + (k & 1), b[..., 1] + ((k >> 1) & 1), b[..., 2] + ((k >> 2) & 1)


def _cells_of(mask):
    """(x, y, z) index arrays of the marked cells."""
    z, y, x = np.nonzero(mask)
    return x, y, z


def _ulps(pos, n=4):
    """n float32 ulps of the position's magnitude (the rounding of a lookup
    position computed in fp32)."""
    return n * np.spacing(np.maximum(np.abs(pos), 1.0).astype(np.float32)).astype(np.float64)


def near_integer(pos):
    """Voxels whose lookup lies within rounding of an integer on some axis."""
    return np.any(np.abs(pos - np.round(pos)) < _ulps(pos), axis=-1)


def count_ties(pos):
    """Boolean map of the cells whose reference-mode count can differ between
    fp32 and fp64 positions: for a lookup within rounding of the integer k on
    axis a, cells k-1 and k+1 on that axis (whichever of them the corner set
    includes depends on the rounding), times both corners on the other axes."""
    mask = np.zeros(pos.shape[:3], dtype=bool)
    k = np.round(pos)
    near = np.abs(pos - k) < _ulps(pos)
    b = np.floor(pos).astype(np.int64)
    for a in range(3):
        sel = near[..., a]
        if not sel.any():
            continue
        p, kb, ka = pos[sel], b[sel], k[sel][:, a].astype(np.int64)
        for off in (-1, 0, 1):
            for s1 in (0, 1):
                for s2 in (0, 1):
                    c = [None, None, None]
                    c[a] = ka + off
                    o = [i for i in range(3) if i != a]
                    c[o[0]] = kb[:, o[0]] + s1
                    c[o[1]] = kb[:, o[1]] + s2
                    _mark(mask, c[0], c[1], c[2])
    return mask


def mc_flips(d, vx, vy, vz, dt, boundary, rel):
    """Voxels whose MC_SMOOTH decision is within ``rel`` (relative to the
    magnitude of the terms of the corrected value) of switching."""
    lut = np.concatenate([-dt * OA.centered(vx, vy, vz), np.zeros(d.shape[:3] + (1,))], axis=-1)[None]
    look = lambda x, l, f: R.sample_grid_lut(x[None], l, filter_mode=f, boundary=boundary,
                                             separate_camera_batch=False, relative=True)[0, 0]
    fwd = look(d, lut, S.LINEAR)
    back = look(fwd, -lut, S.LINEAR)
    corr = fwd + 0.5 * (d - back)
    mn = look(d, lut, S.MIN)
    mx = look(d, lut, S.MAX)
    # rounding of corr is relative to its terms; where they are all exactly
    # zero both precisions compute 0 and agree
    scale = np.abs(fwd) + 0.5 * np.abs(d) + 0.5 * np.abs(back)
    margin = np.minimum(np.abs(corr - mn), np.abs(corr - mx))
    return np.any((margin < rel * scale) & (scale > 0), axis=-1)


def _forward_corners_of(cells, pos_f):
    """Cells that the forward lookups of the marked cells scatter to."""
    out = np.zeros_like(cells)
    x, y, z = _cells_of(cells)
    p = pos_f[z, y, x]
    for cx, cy, cz in _corners(p):
        _mark(out, cx, cy, cz)
    return out


def advect_masks(d, vx, vy, vz, dt=1.0, order=2, clamp='MC_SMOOTH', reference=True, rel=2e-6):
    """(density_mask, velocity_voxel_mask): voxels whose density gradient, and
    voxels whose lookup gradient (hence the adjacent velocity faces), may
    differ between fp32 and fp64 for the reasons above, following the
    adjoint's dependencies: a cell whose back-lookup count or whose fwd
    adjoint changes passes the change to the corners of its forward lookup
    (density) and to its own lookup gradient (velocity); a flipped voxel
    changes its direct term, its own lookup gradient and the fwd adjoints of
    the corners of its back lookup."""
    shape = d.shape[:3]
    pos_f = lookup_positions(vx, vy, vz, dt, 1.0)
    pos_b = lookup_positions(vx, vy, vz, dt, -1.0)
    dmask = np.zeros(shape, dtype=bool)
    # the lookup gradient of a voxel is the spatial derivative of the trilinear
    # fetch at its lookup, which jumps where the lookup crosses a cell boundary
    vmask = near_integer(pos_f)
    if order == 2:
        vmask |= near_integer(pos_b)
    changed_fwd = np.zeros(shape, dtype=bool)  # cells whose fwd adjoint may change
    if reference:
        dmask |= count_ties(pos_f)
        if order == 2:
            changed_fwd |= count_ties(pos_b)
    if order == 2 and clamp == 'MC_SMOOTH':
        flips = mc_flips(d, vx, vy, vz, dt, S.CLAMP, rel)
        dmask |= flips
        vmask |= flips
        x, y, z = _cells_of(flips)
        for cx, cy, cz in _corners(pos_b[z, y, x]):
            _mark(changed_fwd, cx, cy, cz)
    vmask |= changed_fwd
    dmask |= _forward_corners_of(changed_fwd, pos_f)
    return dmask, vmask


def face_masks(vmask):
    """Velocity-face masks (x [D,H,W+1], y [D,H+1,W], z [D+1,H,W]) of the
    faces adjacent to masked voxels."""
    D, H, W = vmask.shape
    fx = np.zeros((D, H, W + 1), dtype=bool)
    fy = np.zeros((D, H + 1, W), dtype=bool)
    fz = np.zeros((D + 1, H, W), dtype=bool)
    fx[:, :, :-1] |= vmask
    fx[:, :, 1:] |= vmask
    fy[:, :-1] |= vmask
    fy[:, 1:] |= vmask
    fz[:-1] |= vmask
    fz[1:] |= vmask
    return fx, fy, fz
