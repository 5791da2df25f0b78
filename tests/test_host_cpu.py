"""CPU-only checks of the host side: the C ABI library's exports and argument
validation (no kernel launch), camera/transform matrices, the synthetic scene,
and the multi-process (replica) timing reduction over gloo."""
import ctypes
import os
import re
import socket
import subprocess
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, 'include', 'gft.h')


@pytest.fixture(scope='module')
def lib():
    from gft import _lib
    if not os.path.exists(_lib.LIB_PATH):
        sys.path.insert(0, os.path.join(ROOT, 'global-flow-transport_gb300'))
        import build
        build.build()
    return _lib


def _declared():
    text = open(HEADER).read()
    text = re.sub(r'/\*.*?\*/', '', text, flags=re.S)
    return sorted(set(re.findall(r'\b(gft_\w+)\s*\(', text)))


def test_library_exports_every_declared_symbol(lib):
    L = lib.load()
    names = _declared()
    assert len(names) >= 20
    for n in names:
        assert hasattr(L, n), n
    assert set(names) == set(lib.exported_symbols())
    assert b'sm_103a' in L.gft_version()


def _prototypes():
    """name -> (return type, [parameter declarations]) of every gft.h function."""
    text = re.sub(r'/\*.*?\*/', '', open(HEADER).read(), flags=re.S)
    protos = {}
    for m in re.finditer(r'([A-Za-z_][\w ]*?\**)\s*\b(gft_\w+)\s*\(([^;{]*?)\)\s*;', text):
        params = [p.strip() for p in m.group(3).split(',')]
        protos[m.group(2)] = (m.group(1).strip(), [] if params in ([''], ['void']) else params)
    return protos


def _kind_of_decl(decl):
    if '*' in decl or '[' in decl:
        return 'ptr'
    # size_t and unsigned long long: one 64-bit unsigned type on the LP64 hosts
    for key, kind in (('size_t', 'u64'), ('int64_t', 'i64'), ('int32_t', 'i32'), ('float', 'f32'),
                      ('unsigned long long', 'u64'), ('gft_status', 'i32')):
        if key in decl:
            return kind
    raise AssertionError('unclassified declaration: ' + decl)


def _kind_of_ctype(t):
    if t in (ctypes.c_void_p, ctypes.c_char_p) or (isinstance(t, type) and issubclass(t, ctypes._Pointer)):
        return 'ptr'
    if t in (ctypes.c_size_t, ctypes.c_ulonglong):
        return 'u64' if ctypes.sizeof(t) == 8 else 'u32'
    return {ctypes.c_int64: 'i64', ctypes.c_int32: 'i32', ctypes.c_float: 'f32'}[t]


def test_bindings_match_the_header_prototypes(lib):
    """Every ctypes signature of gft._lib has the parameter count, parameter
    kinds (pointer / f32 / i32 / i64 / u64) and return kind of its gft.h
    prototype, so a changed prototype cannot be bound with a stale layout."""
    protos = _prototypes()
    assert set(protos) == set(lib._SIGS)
    for name, (ret, params) in protos.items():
        sig_ret, sig_args = lib._SIGS[name]
        assert len(sig_args) == len(params), name
        assert [_kind_of_ctype(t) for t in sig_args] == [_kind_of_decl(p) for p in params], name
        assert _kind_of_ctype(sig_ret) == _kind_of_decl(ret), name


def test_argument_errors_without_a_gpu(lib):
    L = lib.load()
    shape3 = lib.i64([1, 8, 8, 8, 3])
    eye = np.eye(4, dtype=np.float32).reshape(-1)
    fr = np.array([1, 3, -1, 1, 1, -1], dtype=np.float32)
    p = eye.ctypes.data_as(ctypes.c_void_p)
    f = fr.ctypes.data_as(ctypes.c_void_p)
    out = lib.i32([4, 4, 4])
    # three channels: Unimplemented, as resample_grid.cc:330-331
    st = L.gft_raymarch_grid_transform(ctypes.c_void_p(1), 0, shape3, p, 1, p, p, f, 1, out, 1, 0, 0, 1,
                                       ctypes.c_void_p(1), None)
    assert st == lib.ERR_UNIMPLEMENTED
    shape4 = lib.i64([1, 8, 8, 8, 4])
    # invalid blend mode string value
    st = L.gft_raymarch_grid_transform(ctypes.c_void_p(1), 0, shape4, p, 1, p, p, f, 1, out, 1, 0, 9, 1,
                                       ctypes.c_void_p(1), None)
    assert st == lib.ERR_INVALID_ARGUMENT
    # model matrix batch mismatch
    st = L.gft_raymarch_grid_transform(ctypes.c_void_p(1), 0, shape4, p, 2, p, p, f, 1, out, 1, 0, 0, 1,
                                       ctypes.c_void_p(1), None)
    assert st == lib.ERR_INVALID_ARGUMENT and b'model matrix' in L.gft_last_error()
    # gradient needs LINEAR
    st = L.gft_raymarch_grid_transform_grad(ctypes.c_void_p(1), 0, shape4, ctypes.c_void_p(1), ctypes.c_void_p(1),
                                            p, 1, p, p, f, 1, out, 0, 0, 0, 1, 0, ctypes.c_void_p(1), None, 0, None)
    assert st == lib.ERR_INVALID_ARGUMENT
    # reference-mode gradient without workspace
    st = L.gft_raymarch_grid_transform_grad(ctypes.c_void_p(1), 0, shape4, ctypes.c_void_p(1), ctypes.c_void_p(1),
                                            p, 1, p, p, f, 1, out, 1, 0, 0, 1, 0, ctypes.c_void_p(1), None, 0, None)
    assert st == lib.ERR_WORKSPACE
    assert L.gft_raymarch_grid_transform_grad_workspace_size(shape4, 5, 1, 0) >= 8 * 8 * 8 * 5 * 4
    assert L.gft_raymarch_grid_transform_grad_workspace_size(shape4, 5, 1, 1) == 0
    # the raymarch kernels index a grid slice with 32-bit cell arithmetic
    huge = lib.i64([1, 2048, 2048, 1025, 4])
    st = L.gft_raymarch_grid_transform(ctypes.c_void_p(1), 0, huge, p, 1, p, p, f, 1, out, 1, 0, 0, 1,
                                       ctypes.c_void_p(1), None)
    assert st == lib.ERR_INVALID_ARGUMENT and b'2^32' in L.gft_last_error()
    # sample store: LINEAR only, a large enough store, a store pointer.
    # Before the pool: the pool counter, a ballot word and a pool offset per
    # warp and step, a 2x2x2 occupancy map, its empty-space distance map and
    # the distance passes' scratch (256-byte aligned parts); the full pool: one
    # 8x16-pixel tile x 4 steps x 128 lanes, plus the chunks' slack (abandoned
    # chunks hold >= 225 of 256 cells; a last chunk per warp), of 4 floats
    meta = 256 + 256 + 256 + 3 * 256
    cells = 4 * 128
    pool = -(-cells * 256 // 225) + 4 * 256
    assert L.gft_raymarch_grid_transform_samples_min_size(shape4, 1, out, 1) == meta
    assert L.gft_raymarch_grid_transform_samples_size(shape4, 1, out, 1) == meta + -(-pool * 16 // 256) * 256
    st = L.gft_raymarch_grid_transform_store(ctypes.c_void_p(1), 0, shape4, p, 1, p, p, f, 1, out, 0, 0, 0, 1,
                                             ctypes.c_void_p(1), ctypes.c_void_p(1), 1 << 20, None)
    assert st == lib.ERR_INVALID_ARGUMENT and b'LINEAR' in L.gft_last_error()
    st = L.gft_raymarch_grid_transform_store(ctypes.c_void_p(1), 0, shape4, p, 1, p, p, f, 1, out, 1, 0, 0, 1,
                                             ctypes.c_void_p(1), ctypes.c_void_p(1), meta - 256, None)
    assert st == lib.ERR_WORKSPACE
    st = L.gft_raymarch_grid_transform_grad_stored(ctypes.c_void_p(1), 0, shape4, ctypes.c_void_p(1),
                                                   ctypes.c_void_p(1), p, 1, p, p, f, 1, out, 1, 0, 0, 1, 1, None, 0,
                                                   ctypes.c_void_p(1), None, 0, None)
    assert st == lib.ERR_INVALID_ARGUMENT
    # precomputed weight sums are a reference-mode workspace: not with EXACT
    st = L.gft_raymarch_grid_transform_grad(ctypes.c_void_p(1), 0, shape4, ctypes.c_void_p(1), ctypes.c_void_p(1),
                                            p, 1, p, p, f, 1, out, 1, 0, 0, 1, 1 | 0x100, ctypes.c_void_p(1), None,
                                            0, None)
    assert st == lib.ERR_INVALID_ARGUMENT
    # the weight pass validates like the gradient: workspace, boundary, cameras
    st = L.gft_raymarch_grid_transform_grad_weights(shape4, p, 1, p, p, f, 1, out, 0, 1, None, 0, None)
    assert st == lib.ERR_WORKSPACE
    st = L.gft_raymarch_grid_transform_grad_weights(shape4, p, 1, p, p, f, 1, out, 5, 1, ctypes.c_void_p(1),
                                                    1 << 20, None)
    assert st == lib.ERR_INVALID_ARGUMENT
    st = L.gft_raymarch_grid_transform_grad_weights(shape4, p, 2, p, p, f, 1, out, 0, 1, ctypes.c_void_p(1),
                                                    1 << 20, None)
    assert st == lib.ERR_INVALID_ARGUMENT
    # SampleGridTransform: cell centre offset must be 0.5 for transform modes
    st = L.gft_sample_grid_transform(ctypes.c_void_p(1), 0, shape4, p, 1, p, p, f, 1, out, 1, 0, 0, 0, 0.0, 0,
                                     0.25, 1, ctypes.c_void_p(1), None, 0, None)
    assert st == lib.ERR_INVALID_ARGUMENT
    # mips without levels
    st = L.gft_sample_grid_transform(ctypes.c_void_p(1), 0, shape4, p, 1, p, p, f, 1, out, 1, 0, 2, 0, 0.0, 0,
                                     0.5, 1, ctypes.c_void_p(1), None, 0, None)
    assert st == lib.ERR_INVALID_ARGUMENT
    # blend gradient does not accept ALPHA_ADDITIVE (reduce_blend.cc:41)
    st = L.gft_reduce_grid_blend_grad(ctypes.c_void_p(1), ctypes.c_void_p(1), ctypes.c_void_p(1), shape4, 3, 0, 0,
                                      ctypes.c_void_p(1), None)
    assert st == lib.ERR_INVALID_ARGUMENT
    # advection order
    st = L.gft_advect(ctypes.c_void_p(1), 0, lib.i64([1, 8, 8, 8, 1]), ctypes.c_void_p(1), ctypes.c_void_p(1),
                      ctypes.c_void_p(1), 1.0, 3, 0, 1, ctypes.c_void_p(1), None, 0, None)
    assert st == lib.ERR_INVALID_ARGUMENT
    # the forward's intermediate is reused only for MacCormack on one batch slice
    one = ctypes.c_void_p(1)
    for shape, order in (([1, 8, 8, 8, 1], 1), ([2, 8, 8, 8, 1], 2)):
        st = L.gft_advect_grad(one, lib.i64(shape), one, one, one, 1.0, order, 0, 1, 1 | 0x200, one, one, one, one,
                               one, one, 1 << 30, None)
        assert st == lib.ERR_INVALID_ARGUMENT and b'FORWARD_READY' in L.gft_last_error()


def test_misaligned_pointers_are_rejected(lib):
    """Device pointers off their channel vector's alignment (C x element bytes,
    16 for the float4 images) and workspaces or sample stores off 16 bytes are
    argument / workspace errors, found before any launch (no GPU needed)."""
    L = lib.load()
    eye = np.eye(4, dtype=np.float32).reshape(-1)
    fr = np.array([1, 3, -1, 1, 1, -1], dtype=np.float32)
    bkg = np.zeros(3, dtype=np.float32)
    p = eye.ctypes.data_as(ctypes.c_void_p)
    f = fr.ctypes.data_as(ctypes.c_void_p)
    out = lib.i32([4, 4, 4])
    shape4 = lib.i64([1, 8, 8, 8, 4])
    al = ctypes.c_void_p(1 << 20)  # aligned fake device addresses, never dereferenced
    off4 = ctypes.c_void_p((1 << 20) + 4)
    off2 = ctypes.c_void_p((1 << 20) + 2)
    # a four-channel fp32 input, then an output, 4 bytes off a 16-byte boundary
    st = L.gft_raymarch_grid_transform(off4, 0, shape4, p, 1, p, p, f, 1, out, 1, 0, 0, 1, al, None)
    assert st == lib.ERR_INVALID_ARGUMENT and b'aligned' in L.gft_last_error()
    st = L.gft_raymarch_grid_transform(al, 0, shape4, p, 1, p, p, f, 1, out, 1, 0, 0, 1, off4, None)
    assert st == lib.ERR_INVALID_ARGUMENT and b'aligned' in L.gft_last_error()
    # a sample store and a gradient workspace 4 bytes off 16
    st = L.gft_raymarch_grid_transform_store(al, 0, shape4, p, 1, p, p, f, 1, out, 1, 0, 0, 1, al, off4, 1 << 20,
                                             None)
    assert st == lib.ERR_WORKSPACE and b'16-byte' in L.gft_last_error()
    st = L.gft_raymarch_grid_transform_grad(al, 0, shape4, al, al, p, 1, p, p, f, 1, out, 1, 0, 0, 1, 0, al, off4,
                                            1 << 20, None)
    assert st == lib.ERR_WORKSPACE and b'16-byte' in L.gft_last_error()
    st = L.gft_raymarch_grid_transform_grad_weights(shape4, p, 1, p, p, f, 1, out, 0, 1, off4, 1 << 20, None)
    assert st == lib.ERR_WORKSPACE
    # a two-channel bf16 density needs 4 bytes, a two-channel fp32 output 8
    shape2 = lib.i64([1, 8, 8, 8, 2])
    st = L.gft_advect(off2, 1, shape2, al, al, al, 1.0, 1, 0, 1, al, None, 0, None)
    assert st == lib.ERR_INVALID_ARGUMENT and b'aligned' in L.gft_last_error()
    st = L.gft_advect(al, 0, shape2, al, al, al, 1.0, 1, 0, 1, off4, None, 0, None)
    assert st == lib.ERR_INVALID_ARGUMENT and b'aligned' in L.gft_last_error()
    st = L.gft_advect_noalloc(off2, 1, shape2, al, al, al, 1.0, 1, 0, 1, al, None)
    assert st == lib.ERR_INVALID_ARGUMENT and b'aligned' in L.gft_last_error()
    # the image loss reads RGB + density pixels as float4
    st = L.gft_image_loss(off4, al, bkg.ctypes.data_as(ctypes.c_void_p), 16, al, al, 1 << 20, None)
    assert st == lib.ERR_INVALID_ARGUMENT and b'aligned' in L.gft_last_error()


def test_tonemap_and_deterministic_arguments(lib):
    """Argument checks of the tonemapped image loss and the deterministic
    advection workspace, rejected before any launch."""
    L = lib.load()
    buf = np.zeros(4096, np.float32)
    al = buf.ctypes.data + (-buf.ctypes.data) % 256
    bkg = np.zeros(3, np.float32).ctypes.data_as(ctypes.c_void_p)
    st = L.gft_image_loss_tonemap(al, al, bkg, 16, 4, al, al, 1 << 20, None)
    assert st == lib.ERR_INVALID_ARGUMENT and b'tonemap' in L.gft_last_error()
    st = L.gft_image_loss_tonemap_grad(al, al, bkg, 16, 3, al, al, None, 0, None)
    assert st == lib.ERR_WORKSPACE
    assert L.gft_image_loss_workspace_size(16) >= 4 * (4 + 5)
    shape = lib.i64([1, 16, 20, 12, 1])
    base = L.gft_advect_grad_workspace_size(shape, 2)
    assert L.gft_advect_grad_workspace_size_mode(shape, 2, 0) == base
    assert L.gft_advect_grad_workspace_size_mode(shape, 2, 0x400) > base
    assert L.gft_advect_grad_workspace_size_mode(shape, 2, 0x400 | 1) >= 16 * 20 * 12 * (6 * 4 + 3 * 4 + 2 * 4)


def test_projected_gradient_and_factored_light_arguments(lib):
    """The projected raymarch adjoint takes 4-channel bricked inputs; the
    composition's projection is (scale rgb, 0, scale ambient x3, scale);
    checks happen before any launch."""
    L = lib.load()
    eye = np.eye(4, dtype=np.float32).reshape(-1)
    fr = np.array([1, 3, -1, 1, 1, -1], dtype=np.float32)
    p = eye.ctypes.data_as(ctypes.c_void_p)
    f = fr.ctypes.data_as(ctypes.c_void_p)
    out = lib.i32([4, 4, 4])
    proj = np.zeros(8, np.float32)
    pj = proj.ctypes.data_as(ctypes.c_void_p)
    one = ctypes.c_void_p(1)
    brick = 0x10

    def grad(shape, code, mode, projection):
        return L.gft_raymarch_grid_transform_grad_projected(one, code, lib.i64(shape), one, one, p, 1, p, p, f, 1,
                                                            out, 1, 0, 0, 1, mode, None, 0, projection, one, None,
                                                            0, None)
    assert grad([1, 8, 8, 8, 4], brick, 1, None) == lib.ERR_INVALID_ARGUMENT
    assert b'projection' in L.gft_last_error()
    assert grad([1, 8, 8, 8, 2], brick, 1, pj) == lib.ERR_INVALID_ARGUMENT
    assert b'4 channels' in L.gft_last_error()
    assert grad([1, 8, 8, 8, 4], 0, 1, pj) == lib.ERR_INVALID_ARGUMENT
    assert b'brick' in L.gft_last_error()
    # deterministic projected gradient: accepted (here it stops at the missing workspace)
    assert grad([1, 8, 8, 8, 4], brick, 0x400 | 1, pj) == lib.ERR_WORKSPACE
    # per-camera sums: projected GFT_GRAD_REFERENCE without GFT_GRAD_WEIGHTS_READY only
    assert grad([1, 8, 8, 8, 4], brick, 0x800 | 1, pj) == lib.ERR_INVALID_ARGUMENT
    assert b'CAMERA_SUMS' in L.gft_last_error()
    assert grad([1, 8, 8, 8, 4], brick, 0x800 | 0x100, pj) == lib.ERR_INVALID_ARGUMENT
    assert L.gft_raymarch_grid_transform_grad(one, brick, lib.i64([1, 8, 8, 8, 4]), one, one, p, 1, p, p, f, 1, out,
                                              1, 0, 0, 1, 0x800, one, None, 0, None) == lib.ERR_INVALID_ARGUMENT
    assert L.gft_light_compose_factored_grad_cameras(one, one, one, lib.i64([1, 4, 4, 4, 1]), 0, one, one, one,
                                                     one, None) == lib.ERR_INVALID_ARGUMENT
    rgb = np.array([0.5, 2.0, -1.0], np.float32)
    assert L.gft_light_compose_projection(rgb.ctypes.data_as(ctypes.c_void_p), 0.25, 4.0, pj) == lib.OK
    assert proj.tolist() == [2.0, 8.0, -4.0, 0.0, 1.0, 1.0, 1.0, 4.0]
    assert L.gft_light_compose_projection(None, 0.25, 4.0, pj) == lib.ERR_INVALID_ARGUMENT
    shape = lib.i64([1, 4, 4, 4, 1])
    assert L.gft_light_compose_factored(one, one, one, None, shape, 0.5, 1.0, brick, one, None) == \
        lib.ERR_INVALID_ARGUMENT
    assert L.gft_light_compose_factored_grad(one, one, one, shape, 7, one, one, one, None) == \
        lib.ERR_INVALID_ARGUMENT


def test_workspace_sizes(lib):
    L = lib.load()
    s = lib.i64([2, 16, 20, 12, 2])
    # mips: levels 1..3 for both batch slices, 256 B aligned; then per slice
    # two occupancy maps of 2x3x2 8^3-voxel blocks (256 B aligned each)
    n = L.gft_sample_grid_transform_workspace_size(s, 2, 3)
    lv = [(16 >> m) * (20 >> m) * (12 >> m) * 2 for m in (1, 2, 3)]
    mips = 2 * 4 * sum((v + 63) // 64 * 64 for v in lv)
    assert n == (mips + 255) // 256 * 256 + 2 * 2 * 256
    assert L.gft_sample_grid_transform_workspace_size(s, 0, 3) == 0
    assert L.gft_advect_workspace_size(s, 1) == 0 and L.gft_advect_workspace_size(s, 2) >= 16 * 20 * 12 * 2 * 4


def test_camera_matrices_follow_the_reference_conventions():
    from phitest.render.camera import Camera
    from phitest.render.transform import GridTransform, Transform
    cam = Camera(GridTransform([16, 9, 11], translation=[0, 0, 2], parent=Transform(rotation_deg=[0, 30, 0])),
                 nearFar=[1.0, 3.0], fov=40, aspect=11 / 9)
    P = cam.projection_matrix()
    n, f = 1.0, 3.0
    assert np.isclose(P[2, 2], -(f + n) / (f - n)) and np.isclose(P[2, 3], -2 * f * n / (f - n))
    assert np.isclose(P[3, 2], -1.0)
    # camera sits at R_y(30) (0,0,2) and looks at the origin along its -z
    pos = cam.transform.position_global()[:3]
    assert np.allclose(pos, [2 * np.sin(np.radians(30)), 0, 2 * np.cos(np.radians(30))], atol=1e-6)
    vs = cam.view_matrix() @ np.array([0, 0, 0, 1.0])
    assert np.allclose(vs[:2], 0, atol=1e-6) and np.isclose(vs[2], -2.0)
    assert np.allclose(cam.frustum(), [1, 3, cam.left, cam.right, cam.top, cam.bottom])
    assert np.isclose(cam.depth_step, 2.0 / 16)
    gt = GridTransform([8, 10, 6], center=True, normalize='MIN')
    c = gt.get_transform_matrix() @ np.array([3, 5, 4, 1.0])
    assert np.allclose(c[:3], 0, atol=1e-6)


def test_synthetic_scene_is_seeded():
    from gft import synthetic as syn
    a = syn.plume_density((16, 20, 12), 5)
    b = syn.plume_density((16, 20, 12), 5)
    assert np.array_equal(a, b) and a.shape == (1, 16, 20, 12, 1) and a.max() > 0
    vx, vy, vz = syn.curl_velocity((16, 20, 12), 6)
    assert vx.shape == (1, 16, 20, 13, 1) and vy.shape == (1, 16, 21, 12, 1) and vz.shape == (1, 17, 20, 12, 1)
    assert abs(float(np.mean(vy)) - 0.5) < 0.2


_WORKER = r'''
import os, sys
sys.path[:0] = [%r, %r]
import torch.distributed as dist
import bench
dist.init_process_group('gloo', rank=int(os.environ['RANK']), world_size=2)
v = bench.max_over_ranks(1.5 + int(os.environ['RANK']), 'cpu')
print('RESULT', v)
dist.destroy_process_group()
'''


def _free_port():
    s = socket.socket()
    s.bind(('127.0.0.1', 0))
    p = s.getsockname()[1]
    s.close()
    return p


def test_replica_timing_reduction_gloo_two_ranks(tmp_path):
    script = tmp_path / 'w.py'
    script.write_text(_WORKER % (ROOT, os.path.join(ROOT, 'global-flow-transport_gb300')))
    port = _free_port()
    procs = []
    for r in range(2):
        env = dict(os.environ, RANK=str(r), WORLD_SIZE='2', MASTER_ADDR='127.0.0.1', MASTER_PORT=str(port),
                   LOCAL_RANK=str(r))
        procs.append(subprocess.Popen([sys.executable, str(script)], env=env, stdout=subprocess.PIPE,
                                      stderr=subprocess.STDOUT, text=True))
    outs = [p.communicate(timeout=120)[0] for p in procs]
    for p, o in zip(procs, outs):
        assert p.returncode == 0, o
        assert 'RESULT 2.5' in o, o


def test_brick_layout_conversion():
    """to_bricks / from_bricks follow the documented GFT_LAYOUT_BRICK cell order."""
    import torch
    from gft import ops
    D, H, W, C = 5, 4, 7, 2
    x = torch.arange(D * H * W * C, dtype=torch.float32).reshape(1, D, H, W, C)
    xb = ops.to_bricks(x)
    assert xb.shape == (1, ops.brick_cells((D, H, W)), C)

    def cell(xx, yy, zz):
        b = ((zz >> 1) * ((H + 1) // 2) + (yy >> 1)) * ((W + 1) // 2) + (xx >> 1)
        return b * 8 + ((zz & 1) << 2 | (yy & 1) << 1 | (xx & 1))
    for zz in range(D):
        for yy in range(H):
            for xx in range(W):
                assert torch.equal(xb[0, cell(xx, yy, zz)], x[0, zz, yy, xx])
    assert torch.equal(ops.from_bricks(xb, (D, H, W)), x)


def _golden_cameras(kind, res, n, seed=4000):
    from gft import synthetic as syn
    if kind == 'arc':
        return syn.arc_cameras(n, tuple(res), radius=2.5, fov=30.0)
    cams, _ = syn.hemisphere_cameras(n - 1, res[0], seed=seed)
    return cams


def test_camera_crops_match_the_reference_golden_values():
    """Camera.copy_clipped_to_world_coords and copy_with_frustum_crop against
    the values recorded from the reference's own Camera class
    (tests/golden/make_camera_golden.py) for the benchmark scenes: the
    density grid's 8 world corners, every camera of cfg1, cfg2 (pad 0 and 2),
    cfg4's hemisphere views and cfg5."""
    import json
    from phitest.render.transform import GridTransform
    path = os.path.join(ROOT, 'tests', 'golden', 'camera.json')
    with open(path) as f:
        golden = json.load(f)
    for name, g in golden.items():
        D, H, W = g['shape']
        gt = GridTransform([D, H, W], center=True, normalize='MIN')
        corners = gt.transform_AABB([0, 0, 0], [W, H, D], True)
        np.testing.assert_allclose(np.asarray(corners), np.asarray(g['corners']), rtol=1e-6, atol=1e-7)
        cams = _golden_cameras(g['kind'], g['res'], g['n'])
        assert len(cams) == len(g['cameras'])
        for cam, want in zip(cams, g['cameras']):
            clipped, rect = cam.copy_clipped_to_world_coords(corners)
            w = want['clipped']
            np.testing.assert_allclose(clipped.clip, w['clip'], rtol=1e-6, err_msg=name)
            np.testing.assert_allclose(clipped.trbl, w['trbl'], rtol=1e-6, atol=1e-7, err_msg=name)
            np.testing.assert_allclose(np.asarray(rect), np.asarray(w['scissor_rect']), rtol=1e-6, atol=1e-7)
            np.testing.assert_allclose(clipped.projection_matrix(), np.asarray(w['projection']), rtol=1e-6,
                                       atol=1e-7)
            crop = cam.copy_with_frustum_crop(corners, g['pad'])
            w = want['crop']
            assert [int(v) for v in crop.transform.grid_size] == w['grid_size'], name
            assert [[int(a), int(b)] for a, b in crop.scissor_pad] == w['scissor_pad'], name
            np.testing.assert_allclose(crop.clip, w['clip'], rtol=1e-6, err_msg=name)
            np.testing.assert_allclose(crop.trbl, w['trbl'], rtol=1e-6, atol=1e-7, err_msg=name)
            np.testing.assert_allclose(crop.projection_matrix(), np.asarray(w['projection']), rtol=1e-6, atol=1e-7)


def test_state_npz_round_trip_and_reference_keys(tmp_path):
    """DensityGrid / VelocityGrid / State / Sequence .npz files: the keys and
    layout of the reference's files (data_structures.py:332-353, :680-681,
    :1213-1215, :1302-1307), a lossless round trip, and the legacy velocity
    file without 'centered_shape'."""
    import torch
    from phitest.render.data_structures import DensityGrid, Sequence, State, VelocityGrid
    rng = np.random.default_rng(0)
    shape = [5, 6, 4]
    d = torch.from_numpy(rng.random([1] + shape + [1]).astype(np.float32))
    hull = torch.from_numpy((rng.random([1] + shape + [1]) > 0.5).astype(np.float32))
    inflow = torch.from_numpy(rng.random([1, 2, 3, 2, 1]).astype(np.float32))
    dg = DensityGrid(shape, d=d, hull=hull, inflow=inflow, inflow_offset=[1, 2, 1], device='cpu')
    dg.save(str(tmp_path / 'density.npz'))
    with np.load(str(tmp_path / 'density.npz')) as f:
        assert set(f.files) == {'arr_0', 'hull', 'inflow', 'inflow_offset'}
        assert f['arr_0'].shape == (1, 5, 6, 4, 1) and f['inflow_offset'].tolist() == [1, 2, 1]
    dl = DensityGrid.from_file(str(tmp_path / 'density.npz'), device='cpu')
    assert dl.shape == shape and torch.equal(dl.d, d) and torch.equal(dl.hull, hull)
    assert torch.equal(dl.inflow, inflow) and dl.inflow_offset == [1, 2, 1]
    vg = VelocityGrid(shape, std=0.3, device='cpu')
    vg.save(str(tmp_path / 'velocity.npz'))
    with np.load(str(tmp_path / 'velocity.npz')) as f:
        assert set(f.files) == {'centered_shape', 'vel_x', 'vel_y', 'vel_z'}
        assert f['vel_x'].shape == (1, 5, 6, 5, 1) and f['vel_y'].shape == (1, 5, 7, 4, 1)
    vl = VelocityGrid.from_file(str(tmp_path / 'velocity.npz'), device='cpu')
    assert vl.centered_shape == shape and all(torch.equal(a, b) for a, b in zip((vl.x, vl.y, vl.z),
                                                                                (vg.x, vg.y, vg.z)))
    np.savez_compressed(str(tmp_path / 'legacy.npz'), vel_x=vg.x.numpy(), vel_y=vg.y.numpy(), vel_z=vg.z.numpy())
    assert VelocityGrid.from_file(str(tmp_path / 'legacy.npz'), device='cpu').centered_shape == shape
    assert DensityGrid.from_file(str(tmp_path / 'missing.npz'), device='cpu') is None
    # a sequence of three frames: frame_{:06d}/density.npz, velocity.npz
    states = [State(DensityGrid(shape, d=d * (i + 1), device='cpu'), VelocityGrid(shape, std=0.1 * (i + 1),
                                                                                  device='cpu'), frame=10 + i)
              for i in range(3)]
    Sequence(states).save(str(tmp_path / 'seq'))
    assert sorted(os.listdir(str(tmp_path / 'seq'))) == ['frame_000010', 'frame_000011', 'frame_000012']
    seq = Sequence.from_file(str(tmp_path / 'seq'), [10, 11, 12], device='cpu')
    assert [s.frame for s in seq] == [10, 11, 12] and seq[0].next is seq[1] and seq[2].prev is seq[1]
    for a, b in zip(seq, states):
        assert torch.equal(a.density.d, b.density.d) and torch.equal(a.velocity.z, b.velocity.z)
    states[0].save(str(tmp_path / 'one'), suffix='it5')
    assert sorted(os.listdir(str(tmp_path / 'one'))) == ['density_it5.npz', 'velocity_it5.npz']


def test_launch_knobs_validate_and_round_trip(lib):
    """gft_set_knob / gft_get_knob (no launch): every documented value is
    accepted and read back, anything else is rejected and leaves the knob."""
    from gft import autotune as at
    before = at.knobs()
    try:
        for name, (_, cands, default) in at.KNOBS.items():
            for v in cands:
                at.set_knob(name, v)
                assert at.get_knob(name) == v
            at.set_knob(name, default)
            with pytest.raises(ValueError):
                at.set_knob(name, -3)
            assert at.get_knob(name) == default
        L = lib.load()
        assert L.gft_set_knob(99, 1) == 1 and b"unknown knob" in L.gft_last_error()
    finally:
        at.apply(before)
