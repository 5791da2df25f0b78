"""gft_advect_noalloc: the advection entry point for callers that cannot give
the library device memory (it keeps its MacCormack intermediate in a static
device array instead of a workspace).

Calls it through the C ABI twice in a row, on different inputs, and compares
each result with gft_advect (workspace version) on the same inputs at the
forward tolerance of the parity tests, over batch sizes, channel counts,
storage types and both orders.  Also checks that an oversize grid is
rejected before any GPU work.  This file is collected last on purpose.
"""
import ctypes

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

FWD_TOL = 1e-5


def _rel_l2(a, b):
    a = a.double()
    b = b.double()
    n = torch.linalg.norm(b).item()
    return torch.linalg.norm(a - b).item() / (n if n > 0 else 1.0)


def _p(t):
    return ctypes.c_void_p(t.data_ptr())


@pytest.fixture(scope='module')
def lib():
    if not torch.cuda.is_available():
        pytest.skip('no CUDA device')
    from gft import _lib
    return _lib


def _inputs(seed, shape, N, C, dtype):
    D, H, W = shape
    g = torch.Generator().manual_seed(seed)
    d = torch.rand((N, D, H, W, C), generator=g).to(dtype)
    vx = torch.randn((D, H, W + 1), generator=g) * 0.8
    vy = torch.randn((D, H + 1, W), generator=g) * 0.8
    vz = torch.randn((D + 1, H, W), generator=g) * 0.8
    return [t.cuda().contiguous() for t in (d, vx, vy, vz)]


@pytest.mark.parametrize('order', [1, 2])
@pytest.mark.parametrize('dtype', [torch.float32, torch.bfloat16])
@pytest.mark.parametrize('C', [1, 4])
@pytest.mark.parametrize('N', [1, 3])
def test_noalloc_matches_workspace_advect_twice(lib, N, C, dtype, order):
    """Two calls in a row on different inputs, each equal to gft_advect on the
    same inputs; N = 3 reuses the one scratch array slice after slice on one
    stream.  The second call must not change the device's free memory."""
    L = lib.load()
    shape = (24, 30, 20)
    code = 0 if dtype == torch.float32 else 1
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    for call, seed in enumerate((101, 202)):
        d, vx, vy, vz = _inputs(seed + 7 * N + C, shape, N, C, dtype)
        dshape = lib.i64(d.shape)
        ws_bytes = L.gft_advect_workspace_size(dshape, order)
        ws = torch.empty(max(ws_bytes, 1), dtype=torch.uint8, device='cuda')
        ref = torch.empty(d.shape, dtype=torch.float32, device='cuda')
        st = L.gft_advect(_p(d), code, dshape, _p(vx), _p(vy), _p(vz), 1.25, order, 1, 1, _p(ref), _p(ws),
                          ws.numel(), stream)
        lib.check(st, 'gft_advect')
        out = torch.full(d.shape, float('nan'), dtype=torch.float32, device='cuda')
        torch.cuda.synchronize()
        free_before = torch.cuda.mem_get_info()[0]
        st = L.gft_advect_noalloc(_p(d), code, dshape, _p(vx), _p(vy), _p(vz), 1.25, order, 1, 1, _p(out), stream)
        lib.check(st, 'gft_advect_noalloc')
        torch.cuda.synchronize()
        free_after = torch.cuda.mem_get_info()[0]
        assert torch.isfinite(out).all(), 'call %d left unwritten output' % call
        assert _rel_l2(out, ref) <= FWD_TOL, 'call %d differs from gft_advect' % call
        if call == 1:  # the first call may load the module (and with it the static array)
            assert free_after == free_before, 'gft_advect_noalloc changed free device memory'


def test_noalloc_rejects_oversize(lib):
    L = lib.load()
    n = L.gft_advect_noalloc_max_elements()
    side = int(np.ceil((n + 1) ** (1.0 / 3.0))) + 1
    shape = lib.i64([1, side, side, side, 1])
    # real (small) buffers; the declared shape is rejected before any launch
    small = torch.zeros(16, dtype=torch.float32, device='cuda')
    st = L.gft_advect_noalloc(_p(small), 0, shape, _p(small), _p(small), _p(small), 1.0, 2, 1, 1, _p(small), None)
    assert st == lib.ERR_INVALID_ARGUMENT
    assert b'exceeds' in L.gft_last_error()
