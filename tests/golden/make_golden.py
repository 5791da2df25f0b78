"""Generates the golden vectors in tests/golden/ by running the REFERENCE's own
CUDA kernels (phitest/render/cuda/src/*.cu.cc, built unchanged by
oracle/ref/build_ref.py into oracle/_ref/libref_*.so) on seeded small inputs.

Run on a machine with a GPU after building the reference libraries:

    python oracle/ref/build_ref.py && python tests/golden/make_golden.py

Writes tests/golden/<family>.npz (inputs and reference outputs, keyed
"<case>/<array>") and tests/golden/cases.json (the attributes of each case).
tests/test_oracle_golden.py checks the FP64 oracle against these vectors on
the CPU; tests/test_gpu_golden.py checks libgft.so against them on the GPU.
Inputs stay where the reference kernels are valid: the WRAP lookup cases keep
every sample position above -dims (the reference's positive modulo leaves the
grid for negative multiples of the size), and MIN/MAX raymarch cases use CLAMP (the
reference returns +-FLOAT_MAX outside a BORDER domain); the resample-gradient
and raymarch cases use BORDER and CLAMP only.
"""
import ctypes
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
for p in (ROOT, os.path.join(ROOT, 'global-flow-transport_gb300'), os.path.dirname(HERE)):
    if p not in sys.path:
        sys.path.insert(0, p)

import torch  # noqa: E402

from scene_utils import scene, small_grid  # noqa: E402

REF = os.path.join(ROOT, 'oracle', '_ref')

BLENDS = {'BEER_LAMBERT': 0, 'ALPHA': 2, 'ALPHA_ADDITIVE': 3, 'ADDITIVE': 4}
FILTERS = {'NEAREST': 0, 'LINEAR': 1, 'MIN': 2, 'MAX': 3}
BOUNDS = {'BORDER': 0, 'CLAMP': 1, 'WRAP': 2}
MIPS = {'NONE': 0, 'NEAREST': 1, 'LINEAR': 2}
CMS = {'TRANSFORM_LINDEPTH': 0, 'TRANSFORM_LINDEPTH_REVERSE': 1, 'TRANSFORM': 3, 'TRANSFORM_REVERSE': 4}

GRID = (8, 10, 9)
RES = (11, 7, 9)


def i64(v):
    return (ctypes.c_longlong * len(v))(*[int(x) for x in v])


def p(t):
    return ctypes.c_void_p(t.data_ptr())


def hp(a):
    return np.ascontiguousarray(a, dtype=np.float32).ctypes.data_as(ctypes.c_void_p)


_KEEP = []


def dev(a):
    """Device copy that stays alive until the process ends (the pointers handed
    to the C functions must not be recycled by the allocator mid-call)."""
    t = torch.from_numpy(np.ascontiguousarray(a, dtype=np.float32)).cuda()
    _KEEP.append(t)
    return t


def zeros(shape, dtype=torch.float32):
    t = torch.zeros(tuple(int(s) for s in shape), dtype=dtype, device='cuda')
    _KEEP.append(t)
    return t


def mip_atlas_bytes(shape, C, levels):
    """setupMipAtlas's size (resample_grid.cc:201-220) with generous slack."""
    n = ((levels + 1) * 8 + 127) // 128 * 128 + 128
    for m in range(1, levels + 1):
        e = (shape[0] >> m) * (shape[1] >> m) * (shape[2] >> m)
        if e <= 0:
            break
        n += (e * 4 * C + 127) // 128 * 128
    return 2 * n + 4096


class Store:
    def __init__(self):
        self.arrays = {}
        self.cases = {}

    def add(self, family, case, params, **arrays):
        self.cases.setdefault(family, {})[case] = params
        d = self.arrays.setdefault(family, {})
        for k, v in arrays.items():
            d['%s/%s' % (case, k)] = np.asarray(v, dtype=np.float32)

    def save(self):
        for fam, d in self.arrays.items():
            np.savez_compressed(os.path.join(HERE, fam + '.npz'), **d)
        with open(os.path.join(HERE, 'cases.json'), 'w') as f:
            json.dump(self.cases, f, indent=1, sort_keys=True)


def check(rc, what):
    if rc != 0:
        raise RuntimeError('%s returned %d' % (what, rc))


def gen_raymarch(lib, st):
    _, _, M, V, P, F = scene(GRID, 2, RES)
    D, H, W = RES
    combos = [(C, b, bd, 'LINEAR') for C in (1, 2, 4) for b in BLENDS for bd in ('BORDER', 'CLAMP')]
    combos += [(4, 'ADDITIVE', 'CLAMP', f) for f in ('NEAREST', 'MIN', 'MAX')]
    for k, (C, blend, bd, filt) in enumerate(combos):
        x = small_grid(GRID, C, 100 + k) * 0.4
        out_shape6 = [1, 2, D, H, W, C]
        xd = dev(x)
        y = zeros([1, 2, H, W, C])
        check(lib.ref_raymarch_fwd(p(xd), i64(x.shape), hp(M), hp(V), hp(P), hp(F), 2, FILTERS[filt], BOUNDS[bd],
                                   BLENDS[blend], 1, p(y), i64(out_shape6)), 'ref_raymarch_fwd')
        arrays = dict(x=x, y=y.cpu().numpy())
        if filt == 'LINEAR' and C in (1, 4) and bd != 'WRAP':
            rng = np.random.default_rng(200 + k)
            dy = rng.standard_normal((1, 2, H, W, C)).astype(np.float32)
            gx = zeros(x.shape)
            buf = zeros([np.prod(GRID) * C])
            cnt = zeros([np.prod(GRID)])
            check(lib.ref_raymarch_bwd(p(xd), p(gx), p(buf), p(cnt), i64(x.shape), hp(M), hp(V), hp(P), hp(F), 2,
                                       1, BOUNDS[bd], BLENDS[blend], 1, p(y), p(dev(dy)), i64(out_shape6)),
                  'ref_raymarch_bwd')
            arrays.update(dy=dy, gx=gx.cpu().numpy())
        st.add('raymarch', 'rm_%d_%s_%s_%s' % (C, blend, bd, filt),
               dict(C=C, blend=blend, boundary=bd, filter=filt, out_shape=list(RES)), M=M, V=V, P=P, F=F, **arrays)


def gen_blend(lib, st):
    for C in (1, 2, 4):
        for blend in BLENDS:
            for keep in (False, True):
                rng = np.random.default_rng(300 + C * 10 + BLENDS[blend] * 2 + keep)
                x = (rng.random((1, 9, 5, 4, C)) * 0.3).astype(np.float32)
                N, D, H, W, _ = x.shape
                oshape = [N, D if keep else 1, H, W, C]
                y = zeros(oshape)
                check(lib.ref_blend_fwd(p(dev(x)), i64(x.shape), BLENDS[blend], int(keep), p(y), i64(oshape)),
                      'ref_blend_fwd')
                arrays = dict(x=x, y=y.cpu().numpy().reshape([N, D, H, W, C] if keep else [N, H, W, C]))
                if blend != 'ALPHA_ADDITIVE':
                    dy = rng.standard_normal(oshape).astype(np.float32)
                    gx = zeros(x.shape)
                    check(lib.ref_blend_bwd(p(dev(x)), p(gx), i64(x.shape), BLENDS[blend], int(keep), p(y),
                                            p(dev(dy)), i64(oshape)), 'ref_blend_bwd')
                    arrays.update(dy=dy.reshape(arrays['y'].shape), gx=gx.cpu().numpy())
                st.add('blend', 'bl_%d_%s_%d' % (C, blend, keep), dict(C=C, blend=blend, keep=keep), **arrays)


def gen_lut(lib, st):
    k = 0
    for C in (1, 4):
        for filt in FILTERS:
            for bd in BOUNDS:
                k += 1
                rng = np.random.default_rng(400 + k)
                x = small_grid(GRID, C, 410 + k)
                # offsets clipped to +-3.5 cells: every WRAP position stays above -dims
                lut = np.concatenate([np.clip(rng.standard_normal((2, 6, 7, 5, 3)) * 1.8, -3.5, 3.5),
                                      np.zeros((2, 6, 7, 5, 1))], -1).astype(np.float32)
                oshape = [1, 2, 6, 7, 5, C]
                y = zeros(oshape)
                atlas = zeros([16], torch.uint8)
                check(lib.ref_sample_lut(p(dev(x)), i64(x.shape), 2, p(dev(lut)), p(atlas), FILTERS[filt], BOUNDS[bd],
                                         0, 0, ctypes.c_float(0.0), ctypes.c_float(0.0), 1, 1, 0, p(y), i64(oshape)),
                      'ref_sample_lut')
                arrays = dict(x=x, lut=lut, y=y.cpu().numpy())
                if filt in ('LINEAR', 'NEAREST'):
                    glut_lut = np.concatenate([np.clip(rng.standard_normal((2,) + GRID + (3,)) * 1.5, -3.5, 3.5),
                                               np.zeros((2,) + GRID + (1,))], -1).astype(np.float32)
                    dy = rng.standard_normal((1, 2) + GRID + (C,)).astype(np.float32)
                    gx = zeros(x.shape)
                    gl = zeros(glut_lut.shape)
                    cnt = zeros([np.prod(GRID)], torch.int32)
                    check(lib.ref_sample_lut_grad(p(dev(x)), i64(x.shape), 2, p(dev(glut_lut)), FILTERS[filt],
                                                  BOUNDS[bd], ctypes.c_float(0.0), 1, 1, 0, p(dev(dy)),
                                                  i64(dy.shape), p(gx), p(gl), p(cnt)), 'ref_sample_lut_grad')
                    arrays.update(glut_lut=glut_lut, dy=dy, gx=gx.cpu().numpy(), glut=gl.cpu().numpy())
                st.add('lut', 'lut_%d_%s_%s' % (C, filt, bd), dict(C=C, filter=filt, boundary=bd), **arrays)
    # mipmapped lookups with absolute coordinates
    for mip in ('NEAREST', 'LINEAR'):
        for bd in ('BORDER', 'CLAMP'):
            k += 1
            rng = np.random.default_rng(450 + k)
            x = small_grid((16, 18, 14), 2, 460 + k)
            lut = np.concatenate([rng.random((1, 7, 6, 5, 3)) * [14, 18, 16], rng.random((1, 7, 6, 5, 1)) * 3.5],
                                 -1).astype(np.float32)
            oshape = [1, 1, 7, 6, 5, 2]
            y = zeros(oshape)
            atlas = zeros([mip_atlas_bytes((16, 18, 14), 2, 3)], torch.uint8)
            check(lib.ref_sample_lut(p(dev(x)), i64(x.shape), 1, p(dev(lut)), p(atlas), 1, BOUNDS[bd], MIPS[mip], 3,
                                     ctypes.c_float(0.25), ctypes.c_float(0.5), 1, 0, 0, p(y), i64(oshape)),
                  'ref_sample_lut mip')
            st.add('lut', 'lutmip_%s_%s' % (mip, bd), dict(C=2, filter='LINEAR', boundary=bd, mip=mip, levels=3,
                                                           bias=0.25, cco=0.5, relative=False),
                   x=x, lut=lut, y=y.cpu().numpy())


def gen_transform(lib, st):
    shape, res = GRID, RES
    _, _, M, V, P, F = scene(shape, 2, res)
    k = 0
    for cm in CMS:
        rev = cm.endswith('REVERSE')
        in_shape, out_shape = (res, shape) if rev else (shape, res)
        for filt in ('NEAREST', 'LINEAR'):
            for bd in ('BORDER', 'CLAMP'):
                for mip in ('NONE', 'LINEAR', 'NEAREST'):
                    k += 1
                    x = small_grid(in_shape, 2, 500 + k)
                    oshape = [1, 2] + list(out_shape) + [2]
                    y = zeros(oshape)
                    levels = 2 if mip != 'NONE' else 0
                    atlas = zeros([mip_atlas_bytes(in_shape, 2, max(levels, 1))], torch.uint8)
                    check(lib.ref_sample_transform(p(dev(x)), i64(x.shape), hp(M), hp(V), hp(P), hp(F), 2, p(atlas),
                                                   CMS[cm], FILTERS[filt], BOUNDS[bd], MIPS[mip], levels,
                                                   ctypes.c_float(0.3), 1, p(y), i64(oshape)), 'ref_sample_transform')
                    st.add('transform', 'st_%s_%s_%s_%s' % (cm, filt, bd, mip),
                           dict(coord=cm, filter=filt, boundary=bd, mip=mip, levels=levels, bias=0.3,
                                out_shape=list(out_shape)), x=x, y=y.cpu().numpy(), M=M, V=V, P=P, F=F)
        for bd in ('BORDER', 'CLAMP'):  # WRAP scatter is covered by the lookup cases
            k += 1
            rng = np.random.default_rng(600 + k)
            x = small_grid(in_shape, 4, 610 + k)
            dy = rng.standard_normal((1, 2) + tuple(out_shape) + (4,)).astype(np.float32)
            gx = zeros(x.shape)
            cnt = zeros([np.prod(in_shape)], torch.int32)
            check(lib.ref_sample_transform_grad(p(dev(x)), i64(x.shape), hp(M), hp(V), hp(P), hp(F), 2, CMS[cm], 1,
                                                BOUNDS[bd], 1, p(dev(dy)), i64(dy.shape), p(gx), p(cnt)),
                  'ref_sample_transform_grad')
            st.add('transform', 'stg_%s_%s' % (cm, bd), dict(coord=cm, boundary=bd, grad=True),
                   x=x, dy=dy, gx=gx.cpu().numpy(), M=M, V=V, P=P, F=F)
    # LodTransform
    MV = np.stack([M[0] @ V[i] for i in range(2)]).astype(np.float32)
    for inv in (0, 1):
        ins, outs = (shape, res) if not inv else (res, shape)
        out = zeros((2,) + tuple(outs) + (4,))
        check(lib.ref_lod_transform(i64((2,) + tuple(ins) + (4,)), hp(MV), hp(P), hp(F), inv, p(out),
                                    i64((2,) + tuple(outs) + (4,))), 'ref_lod_transform')
        st.add('transform', 'lod_%d' % inv, dict(inverse=inv, in_shape=list(ins), out_shape=list(outs)),
               MV=MV, P=P, F=F, y=out.cpu().numpy())


def main():
    libs = {n: ctypes.CDLL(os.path.join(REF, 'libref_%s.so' % n)) for n in ('raymarch', 'resample', 'blend')}
    st = Store()
    gen_raymarch(libs['raymarch'], st)
    gen_blend(libs['blend'], st)
    gen_lut(libs['resample'], st)
    gen_transform(libs['resample'], st)
    st.save()
    n = sum(len(v) for v in st.cases.values())
    print('wrote %d golden cases to %s' % (n, HERE))


if __name__ == '__main__':
    main()
