"""Blend functors and the depth reduce-blend op, restated in float64.

BlendState<T, mode> (blending.hpp:10-221).  ``acc``/``cell`` are (..., C) arrays,
C in {1, 2, 4}; the last channel is the density/opacity, the others the light.
For C == 1 every mode falls back to the generic additive template
(blending.hpp:10-21; only float2/float4 are specialised), so a one-channel
BEER_LAMBERT blend is a plain running sum.

Test infrastructure only; see the package docstring.
"""
import numpy as np

BEER_LAMBERT, BEER_LAMBERT_EXCLUSIVE, ALPHA, ALPHA_ADDITIVE, ADDITIVE = 0, 1, 2, 3, 4


def blend(mode, acc, cell):
    C = acc.shape[-1]
    if C == 1 or mode == ADDITIVE:
        return acc + cell
    L, d = acc[..., :-1], acc[..., -1]
    l, s = cell[..., :-1], cell[..., -1]
    if mode == BEER_LAMBERT:
        dn = np.maximum(d + s, 0.0)
        t = np.exp(-dn)
        return np.concatenate([L + t[..., None] * l, dn[..., None]], axis=-1)
    if mode == BEER_LAMBERT_EXCLUSIVE:
        t = np.exp(-d)
        return np.concatenate([L + t[..., None] * l, (d + s)[..., None]], axis=-1)
    if mode == ALPHA:
        t = 1.0 - d
        return np.concatenate([L + t[..., None] * l, (d + t * s)[..., None]], axis=-1)
    if mode == ALPHA_ADDITIVE:
        t = 1.0 - s
        return np.concatenate([L + t[..., None] * l, (d + s)[..., None]], axis=-1)
    raise ValueError(mode)


def blend_gradients(mode, g, cell, out, exact):
    """One back-to-front step.  ``g`` is the adjoint of the accumulator after
    this cell, ``out`` the accumulator after this cell.  Returns
    (grad of the cell, new g, accumulator before this cell).

    exact=False reproduces blendGradients of the reference literally
    (blending.hpp:29-43, :99-114, :137-152, :177-192).  exact=True differs only
    for ALPHA, where the reference's transmittance bookkeeping is not the
    adjoint of its forward blend; there the true adjoint is used."""
    C = cell.shape[-1]
    if C == 1 or mode == ADDITIVE:
        return g.copy(), g, out - cell
    gl, gd = g[..., :-1], g[..., -1]
    l, s = cell[..., :-1], cell[..., -1]
    dout = out[..., -1]
    if mode == BEER_LAMBERT:
        e = np.exp(-dout)
        dprev = np.maximum(dout - s, 0.0)
        d_dacc = gd - e * np.sum(l * gl, axis=-1)
        gcell = np.concatenate([e[..., None] * gl, d_dacc[..., None]], axis=-1)
        gnew = np.concatenate([gl, d_dacc[..., None]], axis=-1)
        return gcell, gnew, np.concatenate([out[..., :-1], dprev[..., None]], axis=-1)
    if mode == BEER_LAMBERT_EXCLUSIVE:
        dprev = np.maximum(dout - s, 0.0)
        e = np.exp(-dprev)
        d_dacc = gd - e * np.sum(l * gl, axis=-1)
        gcell = np.concatenate([e[..., None] * gl, gd[..., None]], axis=-1)
        gnew = np.concatenate([gl, d_dacc[..., None]], axis=-1)
        return gcell, gnew, np.concatenate([out[..., :-1], dprev[..., None]], axis=-1)
    if mode == ALPHA:
        if exact:
            # forward: a_i = a_{i-1} + T_{i-1} s_i, T = 1 - a ; L_i = L_{i-1} + T_{i-1} l_i
            Tprev = (1.0 - dout) / (1.0 - s)
            d_dacc = (1.0 - s) * gd - np.sum(l * gl, axis=-1)
            gcell = np.concatenate([Tprev[..., None] * gl, (Tprev * gd)[..., None]], axis=-1)
            gnew = np.concatenate([gl, d_dacc[..., None]], axis=-1)
            return gcell, gnew, np.concatenate([out[..., :-1], (1.0 - Tprev)[..., None]], axis=-1)
        wnew = (1.0 - dout) / (1.0 - s)
        t = 1.0 - wnew
        d_dacc = (1.0 - s) * gd - np.sum(l * gl, axis=-1)
        gcell = np.concatenate([t[..., None] * gl, (t * gd)[..., None]], axis=-1)
        gnew = np.concatenate([gl, d_dacc[..., None]], axis=-1)
        return gcell, gnew, np.concatenate([out[..., :-1], wnew[..., None]], axis=-1)
    if mode == ALPHA_ADDITIVE:
        t = 1.0 - s
        d_d = gd - np.sum(l * gl, axis=-1)
        gcell = np.concatenate([t[..., None] * gl, d_d[..., None]], axis=-1)
        return gcell, g, np.concatenate([out[..., :-1], (dout - s)[..., None]], axis=-1)
    raise ValueError(mode)


def reduce_grid_blend(x, mode, keep_dims):
    """ReduceGridBlend (reduce_blend.cc:23-34, kBlend reduce_blend.cu.cc:34-51).
    x: [N, D, H, W, C] -> [N, D, H, W, C] (keep_dims) or [N, H, W, C]."""
    x = np.asarray(x, dtype=np.float64)
    acc = np.zeros(x.shape[:1] + x.shape[2:])
    outs = []
    for z in range(x.shape[1]):
        acc = blend(mode, acc, x[:, z])
        if keep_dims:
            outs.append(acc)
    return np.stack(outs, axis=1) if keep_dims else acc


def reduce_grid_blend_grad(dy, y, x, mode, keep_dims, exact=False):
    """ReduceGridBlendGrad (reduce_blend.cc:37-48, kBlendGrad reduce_blend.cu.cc:53-75).
    Back to front; with keep_dims the output gradient of each depth is added and
    the stored output of each depth is used as the accumulator."""
    x = np.asarray(x, dtype=np.float64)
    dy = np.asarray(dy, dtype=np.float64)
    y = np.asarray(y, dtype=np.float64)
    gx = np.zeros_like(x)
    g = np.zeros(x.shape[:1] + x.shape[2:])
    prev = np.zeros_like(g)
    if not keep_dims:
        g = dy.copy()
        prev = y.copy()
    for z in range(x.shape[1] - 1, -1, -1):
        if keep_dims:
            g = g + dy[:, z]
            prev = y[:, z].copy()
        gc, g, prev = blend_gradients(mode, g, x[:, z], prev, exact)
        gx[:, z] = gc
    return gx
