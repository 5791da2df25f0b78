"""libgft.so against the golden vectors recorded from the reference's own CUDA
kernels (tests/golden/), reference gradient mode."""
import numpy as np
import pytest
import torch

import golden_cases as G

pytestmark = [pytest.mark.gpu, pytest.mark.skipif(not G.available(), reason='golden vectors not generated')]


@pytest.fixture(scope='module')
def ops():
    if not torch.cuda.is_available():
        pytest.skip('no CUDA device')
    from gft import ops as _ops
    _ops.set_grad_mode('REFERENCE')
    return _ops


def cuda(a):
    return torch.from_numpy(np.ascontiguousarray(a, dtype=np.float32)).cuda()


def np_(t):
    return t.detach().cpu().numpy()


@pytest.mark.parametrize('case,prm', G.cases('raymarch'))
def test_raymarch_golden_gpu(ops, case, prm):
    a = G.arrays('raymarch', case)
    y = ops.raymarch_grid_transform(cuda(a['x']), a['M'], a['V'], a['P'], a['F'], prm['out_shape'], prm['filter'],
                                    prm['boundary'], prm['blend'])
    G.assert_close(np_(y), a['y'], G.FWD_TOL, step=prm['filter'] != 'LINEAR', what=case)
    if 'gx' in a:
        g = ops.raymarch_grid_transform_grad(cuda(a['x']), cuda(a['y']), cuda(a['dy']), a['M'], a['V'], a['P'],
                                             a['F'], prm['out_shape'], 'LINEAR', prm['boundary'], prm['blend'])
        G.assert_close(np_(g), a['gx'], G.GRAD_TOL, what=case + ' grad')


@pytest.mark.parametrize('case,prm', G.cases('blend'))
def test_blend_golden_gpu(ops, case, prm):
    a = G.arrays('blend', case)
    y = ops.reduce_grid_blend(cuda(a['x']), prm['blend'], prm['keep'])
    G.assert_close(np_(y), a['y'], G.FWD_TOL, what=case)
    if 'gx' in a:
        g = ops.reduce_grid_blend_grad(cuda(a['dy']), cuda(a['y']), cuda(a['x']), prm['blend'], prm['keep'])
        G.assert_close(np_(g), a['gx'], G.GRAD_TOL, what=case + ' grad')


@pytest.mark.parametrize('case,prm', G.cases('lut'))
def test_lut_golden_gpu(ops, case, prm):
    a = G.arrays('lut', case)
    mip = prm.get('mip', 'NONE')
    y = ops.sample_grid_lut(cuda(a['x']), cuda(a['lut']), prm['filter'], prm['boundary'], mip, prm.get('levels', 0),
                            prm.get('bias', 0.0), cell_center_offset=prm.get('cco', 0.0),
                            relative_coords=prm.get('relative', True))
    G.assert_close(np_(y), a['y'], G.FWD_TOL, step=(prm['filter'] == 'NEAREST' or mip == 'NEAREST'), what=case)
    if 'gx' in a:
        gx, gl = ops.sample_grid_lut_grad(cuda(a['x']), cuda(a['dy']), cuda(a['glut_lut']), prm['filter'],
                                          prm['boundary'])
        G.assert_close(np_(gx), a['gx'], G.GRAD_TOL, what=case + ' input grad')
        G.assert_close(np_(gl), a['glut'], G.GRAD_TOL, what=case + ' lookup grad')


@pytest.mark.parametrize('case,prm', G.cases('transform'))
def test_transform_golden_gpu(ops, case, prm):
    a = G.arrays('transform', case)
    if case.startswith('lod_'):
        y = ops.lod_transform(prm['in_shape'], a['MV'], a['P'], a['F'], prm['out_shape'], bool(prm['inverse']))
        G.assert_close(np_(y), a['y'], G.FWD_TOL, what=case)
    elif prm.get('grad'):
        g = ops.sample_grid_transform_grad(cuda(a['x']), cuda(a['dy']), a['M'], a['V'], a['P'], a['F'], 'LINEAR',
                                           prm['boundary'], coordinate_mode=prm['coord'])
        G.assert_close(np_(g), a['gx'], G.GRAD_TOL, what=case)
    else:
        y = ops.sample_grid_transform(cuda(a['x']), a['M'], a['V'], a['P'], a['F'], prm['out_shape'], prm['filter'],
                                      prm['boundary'], prm['mip'], prm['levels'], prm['bias'], prm['coord'])
        G.assert_close(np_(y), a['y'], G.FWD_TOL, step=(prm['filter'] == 'NEAREST' or prm['mip'] == 'NEAREST'),
                       what=case)
