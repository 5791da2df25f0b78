"""Tonemapping of the composited images and the image loss through it, float64.

TEST INFRASTRUCTURE ONLY (imported by tests/).

Renderer._tonemap (phitest/render/renderer.py:528-541), applied by
render_density to the background-composited images (renderer.py:632-640):

    NONE            c
    CLIP_NEGATIVE   max(c, 0)
    SATURATE        clip(c, 0, 1)
    NORMALIZE       y = c - min(c) if min(c) < 0 else c;  y / max(y) if max(y) > 0

with min / max over the whole image tensor.  The gradient follows the
framework rules the reference relies on: tf.maximum passes the gradient to
its first argument where x >= y, clip_by_value where min <= x <= max, and a
full reduce_min / reduce_max divides its gradient evenly among the elements
equal to the result.
"""
import numpy as np

MODES = ('NONE', 'CLIP_NEGATIVE', 'SATURATE', 'NORMALIZE')


def tonemap(c, mode='NONE'):
    c = np.asarray(c, dtype=np.float64)
    if mode == 'NONE':
        return c
    if mode == 'CLIP_NEGATIVE':
        return np.maximum(c, 0.0)
    if mode == 'SATURATE':
        return np.clip(c, 0.0, 1.0)
    if mode == 'NORMALIZE':
        mn = c.min()
        y = c - mn if mn < 0 else c
        mx = y.max()
        return y / mx if mx > 0 else y
    raise ValueError(mode)


def tonemap_grad(c, g, mode='NONE'):
    """d/dc of sum(g * tonemap(c))."""
    c = np.asarray(c, dtype=np.float64)
    g = np.asarray(g, dtype=np.float64)
    if mode == 'NONE':
        return g
    if mode == 'CLIP_NEGATIVE':
        return np.where(c >= 0, g, 0.0)
    if mode == 'SATURATE':
        return np.where((c >= 0) & (c <= 1), g, 0.0)
    if mode == 'NORMALIZE':
        mn = c.min()
        y = c - mn if mn < 0 else c
        mx = y.max()
        gy = g
        if mx > 0:
            z = y / mx
            gmx = -np.sum(g * z) / mx
            at_max = y == mx
            gy = g / mx + np.where(at_max, gmx / at_max.sum(), 0.0)
        gc = gy
        if mn < 0:
            at_min = c == mn
            gc = gy + np.where(at_min, -np.sum(gy) / at_min.sum(), 0.0)
        return gc
    raise ValueError(mode)


def image_loss(img, target, bkg, mode='NONE'):
    """(loss, d loss / d img) of mean((tonemap(rgb + bkg exp(-a)) - target)^2)
    for img [..., 4] (rgb + density), target [..., 3]."""
    img = np.asarray(img, dtype=np.float64)
    bkg = np.asarray(bkg, dtype=np.float64)
    e = np.exp(-img[..., 3:])
    c = img[..., :3] + bkg * e
    r = tonemap(c, mode) - np.asarray(target, dtype=np.float64)
    n = r.size
    loss = float(np.mean(r * r))
    gc = tonemap_grad(c, 2.0 * r / n, mode)
    gimg = np.empty_like(img)
    gimg[..., :3] = gc
    gimg[..., 3] = -np.sum(gc * bkg, axis=-1) * e[..., 0]
    return loss, gimg
