"""FP64 raymarch of the rays that reach one sub-block of a large grid.

TEST INFRASTRUCTURE ONLY (imported by tests/ and the CPU leg of bench.py, as
the checker).

At full configuration sizes the FP64 oracle cannot march every ray, but a
block's density gradient depends only on the rays whose samples reach it: the
pixels inside the bounding rectangle of the block's projected corners (the
block widened by two voxels, because a sample reaches the voxels within one
cell of its position, and the rectangle by two pixels).  Marching those rays
with the other pixels' output gradient set to zero gives the block's gradient
exactly.
"""
import numpy as np

from . import raymarch as RM
from . import transforms as T


def pixel_windows(M, V, P, F, res, block, size, margin_vox=2.0, margin_px=2):
    """Per camera, the (rows, cols) slices of the pixels whose rays can reach
    the block at (z0, y0, x0) of edge ``size``."""
    z0, y0, x0 = block
    lo = np.array([x0, y0, z0], np.float64) - margin_vox
    hi = lo + size + 2 * margin_vox
    corners = np.array([[(hi if (k >> a) & 1 else lo)[a] for a in range(3)] for k in range(8)])
    D, H, W = res
    rows, cols = [], []
    for c in range(len(V)):
        cam = T.CameraXform(np.asarray(M)[0], np.asarray(V)[c], np.asarray(P)[c], np.asarray(F)[c])
        ndc = T.os_to_ndc(cam, corners)
        px = (ndc[:, 0] + 1.0) * W / 2.0 - 0.5
        py = (ndc[:, 1] + 1.0) * H / 2.0 - 0.5
        c0 = int(max(0, np.floor(px.min()) - margin_px))
        c1 = int(min(W, np.ceil(px.max()) + margin_px + 1))
        r0 = int(max(0, np.floor(py.min()) - margin_px))
        r1 = int(min(H, np.ceil(py.max()) + margin_px + 1))
        rows.append(slice(r0, max(r0, r1)))
        cols.append(slice(c0, max(c0, c1)))
    return rows, cols


def raymarch_block(x, M, V, P, F, res, dy_full, block, size, exact=False):
    """(image [1,V,H,W,C] filled in the windows, gradient [1,D,H,W,C] exact
    inside the block, rows, cols) of the BEER_LAMBERT / LINEAR / BORDER
    raymarch of x [1,D,H,W,C] with output gradient dy_full [1,V,H,W,C]."""
    rows, cols = pixel_windows(M, V, P, F, res, block, size)
    x64 = np.asarray(x, np.float64)
    y = RM.raymarch_fwd(x64, M, V, P, F, res, rows=rows, cols=cols)
    dy = np.zeros_like(y)
    for c in range(len(V)):
        dy[0, c][rows[c], cols[c]] = dy_full[0, c][rows[c], cols[c]]
    g = RM.raymarch_bwd(x64, y, dy, M, V, P, F, res, exact=exact, rows=rows, cols=cols)
    return y, g, rows, cols
