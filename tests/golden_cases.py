"""Loader of the golden vectors produced by the reference's own kernels
(tests/golden/make_golden.py) and the comparison rules shared by the CPU
(oracle) and GPU (libgft.so) golden tests."""
import json
import os

import numpy as np

HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), 'golden')

FWD_TOL = 1e-5
GRAD_TOL = 1e-4
STEP_FRACTION = 0.02  # share of cells allowed to differ for step-function selections


def available():
    return os.path.exists(os.path.join(HERE, 'cases.json'))


def cases(family):
    if not available():
        return []
    with open(os.path.join(HERE, 'cases.json')) as f:
        meta = json.load(f)
    return sorted(meta.get(family, {}).items())


_cache = {}


def arrays(family, case):
    if family not in _cache:
        _cache[family] = dict(np.load(os.path.join(HERE, family + '.npz')))
    d = _cache[family]
    pre = case + '/'
    return {k[len(pre):]: v for k, v in d.items() if k.startswith(pre)}


def rel_l2(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    n = np.linalg.norm(b)
    return float(np.linalg.norm(a - b) / (n if n > 0 else 1.0))


def assert_close(got, want, tol, step=False, what=''):
    got = np.asarray(got, dtype=np.float64).reshape(np.shape(want))
    want = np.asarray(want, dtype=np.float64)
    if step:
        scale = max(1e-30, float(np.max(np.abs(want))))
        bad = np.any(np.abs(got - want) > 1e-5 * scale, axis=-1)
        assert bad.mean() <= STEP_FRACTION, '%s: %.3f of cells differ' % (what, bad.mean())
        assert rel_l2(got[~bad], want[~bad]) <= tol, what
    else:
        e = rel_l2(got, want)
        assert e <= tol, '%s: rel-L2 %.3g > %.1g' % (what, e, tol)
