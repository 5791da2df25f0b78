"""Pins the FP64 oracle to the reference: every golden vector recorded from the
reference's own CUDA kernels (tests/golden/, made by make_golden.py) must be
reproduced by the oracle within the fp32 tolerances.  CPU only."""
import numpy as np
import pytest

import golden_cases as G
from oracle import blend as OB
from oracle import raymarch as RM
from oracle import resample as R
from oracle import transforms as OT

pytestmark = pytest.mark.skipif(not G.available(), reason='golden vectors not generated')

FILT = {'NEAREST': 0, 'LINEAR': 1, 'MIN': 2, 'MAX': 3}
BND = {'BORDER': 0, 'CLAMP': 1, 'WRAP': 2}
MIP = {'NONE': 0, 'NEAREST': 1, 'LINEAR': 2}
CM = {'TRANSFORM_LINDEPTH': OT.LINDEPTH, 'TRANSFORM_LINDEPTH_REVERSE': OT.LINDEPTH_REVERSE,
      'TRANSFORM': OT.TRANSFORM, 'TRANSFORM_REVERSE': OT.TRANSFORM_REVERSE}


@pytest.mark.parametrize('case,prm', G.cases('raymarch'))
def test_raymarch_golden(case, prm):
    a = G.arrays('raymarch', case)
    y = RM.raymarch_fwd(a['x'], a['M'], a['V'], a['P'], a['F'], prm['out_shape'], FILT[prm['filter']],
                        BND[prm['boundary']], getattr(OB, prm['blend']))
    G.assert_close(y, a['y'], G.FWD_TOL, step=prm['filter'] != 'LINEAR', what=case)
    if 'gx' in a:
        g = RM.raymarch_bwd(a['x'], a['y'], a['dy'], a['M'], a['V'], a['P'], a['F'], prm['out_shape'],
                            BND[prm['boundary']], getattr(OB, prm['blend']), exact=False)
        G.assert_close(g, a['gx'], G.GRAD_TOL, what=case + ' grad')


@pytest.mark.parametrize('case,prm', G.cases('blend'))
def test_blend_golden(case, prm):
    a = G.arrays('blend', case)
    mode = getattr(OB, prm['blend'])
    y = OB.reduce_grid_blend(a['x'], mode, prm['keep'])
    G.assert_close(y, a['y'], G.FWD_TOL, what=case)
    if 'gx' in a:
        g = OB.reduce_grid_blend_grad(a['dy'], a['y'], a['x'], mode, prm['keep'], exact=False)
        G.assert_close(g, a['gx'], G.GRAD_TOL, what=case + ' grad')


@pytest.mark.parametrize('case,prm', G.cases('lut'))
def test_lut_golden(case, prm):
    a = G.arrays('lut', case)
    mip = prm.get('mip', 'NONE')
    y = R.sample_grid_lut(a['x'], a['lut'], FILT[prm['filter']], BND[prm['boundary']], MIP[mip],
                          prm.get('levels', 0), prm.get('bias', 0.0), prm.get('cco', 0.0),
                          relative=prm.get('relative', True))
    G.assert_close(y, a['y'], G.FWD_TOL, step=(prm['filter'] == 'NEAREST' or mip == 'NEAREST'), what=case)
    if 'gx' in a:
        gx, gl = R.sample_grid_lut_grad(a['x'], a['dy'], a['glut_lut'], FILT[prm['filter']], BND[prm['boundary']],
                                        exact=False)
        G.assert_close(gx, a['gx'], G.GRAD_TOL, what=case + ' input grad')
        G.assert_close(gl, a['glut'], G.GRAD_TOL, what=case + ' lookup grad')


@pytest.mark.parametrize('case,prm', G.cases('transform'))
def test_transform_golden(case, prm):
    a = G.arrays('transform', case)
    if case.startswith('lod_'):
        y = R.lod_transform(prm['in_shape'], a['MV'], a['P'], a['F'], prm['out_shape'], bool(prm['inverse']))
        G.assert_close(y, a['y'], G.FWD_TOL, what=case)
    elif prm.get('grad'):
        g = R.sample_grid_transform_grad(a['x'], a['dy'], a['M'], a['V'], a['P'], a['F'], BND[prm['boundary']],
                                         CM[prm['coord']], exact=False)
        G.assert_close(g, a['gx'], G.GRAD_TOL, what=case)
    else:
        y = R.sample_grid_transform(a['x'], a['M'], a['V'], a['P'], a['F'], prm['out_shape'], FILT[prm['filter']],
                                    BND[prm['boundary']], MIP[prm['mip']], prm['levels'], prm['bias'],
                                    CM[prm['coord']])
        G.assert_close(y, a['y'], G.FWD_TOL, step=(prm['filter'] == 'NEAREST' or prm['mip'] == 'NEAREST'),
                       what=case)


def test_golden_vectors_present_and_nontrivial():
    n = sum(len(G.cases(f)) for f in ('raymarch', 'blend', 'lut', 'transform'))
    assert n >= 100
    a = G.arrays('raymarch', G.cases('raymarch')[0][0])
    assert np.abs(a['y']).sum() > 0
