"""Times the plain per-op render + advect step composed from the REFERENCE's own
CUDA kernels (oracle/_ref/libref_*.so, built by oracle/ref/build_ref.py from
the unchanged reference sources) beside this repository's batched step.

ORACLE / MEASUREMENT INFRASTRUCTURE ONLY: a measurement of the reference, not
part of the product.

The plain step of gft.pipeline (RenderAdvectStep(mode='plain'): one raymarch
call per camera, advection as four SampleGridLut calls plus elementwise ops,
the shadow pass as SampleGridTransform + ReduceGridBlend with the
inverse-resampling gradient, tensor-op glue, no CUDA graph, FP32) is run with
its four kernel ops -- SampleGridLut(+Grad), SampleGridTransform,
ReduceGridBlend(+Grad), RaymarchGridTransform(+Grad) -- served by the
reference's launchers (which synchronise the device after every call, as in
the reference) instead of this repository's.  That is the reference's
per-op structure on its own kernels, the composition glue being the same
tensor ops.  Both steps are timed with CUDA events over whole steps.

    python oracle/ref/build_ref.py && python oracle/ref/time_ref_step.py --config cfg2
"""
import argparse
import ctypes
import json
import os
import sys
import time

import numpy as np
import torch

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path[:0] = [ROOT, os.path.join(ROOT, 'global-flow-transport_gb300')]
REF = os.path.join(ROOT, 'oracle', '_ref')

FILTER = {'NEAREST': 0, 'LINEAR': 1, 'MIN': 2, 'MAX': 3}
BOUNDARY = {'BORDER': 0, 'CLAMP': 1, 'WRAP': 2}
MIP = {'NONE': 0, 'NEAREST': 1, 'LINEAR': 2}
COORD = {'TRANSFORM_LINDEPTH': 0, 'TRANSFORM_LINDEPTH_REVERSE': 1}


def i64(v):
    return (ctypes.c_longlong * len(v))(*[int(x) for x in v])


def p(t):
    return ctypes.c_void_p(t.data_ptr())


def hp(a):
    a = np.ascontiguousarray(a, dtype=np.float32)
    hp.keep.append(a)  # alive until the synchronous call returns
    return a.ctypes.data_as(ctypes.c_void_p)


hp.keep = []


def check(rc, what):
    if rc != 0:
        raise RuntimeError('%s returned %d' % (what, rc))


def mip_atlas_bytes(shape, C, levels):
    """setupMipAtlas's size (resample_grid.cc:201-220) with generous slack."""
    n = ((levels + 1) * 8 + 127) // 128 * 128 + 128
    for m in range(1, levels + 1):
        e = (shape[0] >> m) * (shape[1] >> m) * (shape[2] >> m)
        if e <= 0:
            break
        n += (e * 4 * C + 127) // 128 * 128
    return 2 * n + 4096


def reference_ops(libs):
    """Replacements of the four kernel ops of gft.ops, served by the
    reference's launchers (FP32, the arguments the plain step passes)."""
    rm, rs, bl = libs['raymarch'], libs['resample'], libs['blend']

    class Lut(torch.autograd.Function):
        @staticmethod
        def forward(ctx, x, lut, filt, boundary):
            x = x.contiguous()
            lut = lut.contiguous()
            N, D, H, W, C = x.shape
            out = torch.empty((N, 1, D, H, W, C), device=x.device)
            atlas = torch.empty(16, dtype=torch.uint8, device=x.device)
            check(rs.ref_sample_lut(p(x), i64(x.shape), 1, p(lut), p(atlas), filt, boundary, 0, 0,
                                    ctypes.c_float(0.0), ctypes.c_float(0.0), 1, 1, 0, p(out), i64(out.shape)),
                  'ref_sample_lut')
            ctx.save_for_backward(x, lut)
            ctx.k = (filt, boundary)
            return out

        @staticmethod
        def backward(ctx, g):
            x, lut = ctx.saved_tensors
            filt, boundary = ctx.k
            g = g.contiguous()
            gx = torch.empty_like(x)
            gl = torch.empty_like(lut)
            cnt = torch.empty(x[0].numel() // x.shape[-1], dtype=torch.int32, device=x.device)
            check(rs.ref_sample_lut_grad(p(x), i64(x.shape), 1, p(lut), filt, boundary, ctypes.c_float(0.0), 1, 1, 0,
                                         p(g), i64(g.shape), p(gx), p(gl), p(cnt)), 'ref_sample_lut_grad')
            return gx, gl, None, None

    class Blend(torch.autograd.Function):
        @staticmethod
        def forward(ctx, x):
            x = x.contiguous()
            out = torch.empty_like(x)
            check(bl.ref_blend_fwd(p(x), i64(x.shape), 0, 1, p(out), i64(out.shape)), 'ref_blend_fwd')
            ctx.save_for_backward(x, out)
            return out

        @staticmethod
        def backward(ctx, g):
            x, out = ctx.saved_tensors
            gx = torch.empty_like(x)
            g = g.contiguous()
            check(bl.ref_blend_bwd(p(x), p(gx), i64(x.shape), 0, 1, p(out), p(g), i64(out.shape)), 'ref_blend_bwd')
            return gx

    class Raymarch(torch.autograd.Function):
        @staticmethod
        def forward(ctx, x, M, V, P, F, res):
            x = x.contiguous()
            nv = len(V)
            D, H, W = res
            out6 = [x.shape[0], nv, D, H, W, x.shape[-1]]
            y = torch.empty((x.shape[0], nv, H, W, x.shape[-1]), device=x.device)
            check(rm.ref_raymarch_fwd(p(x), i64(x.shape), hp(M), hp(V), hp(P), hp(F), nv, 1, 0, 0, 1, p(y), i64(out6)),
                  'ref_raymarch_fwd')
            ctx.save_for_backward(x, y)
            ctx.k = (M, V, P, F, out6)
            return y

        @staticmethod
        def backward(ctx, g):
            x, y = ctx.saved_tensors
            M, V, P, F, out6 = ctx.k
            gx = torch.empty_like(x)
            buf = torch.empty(x.numel(), device=x.device)
            cnt = torch.empty(x.numel() // x.shape[-1], device=x.device)
            g = g.contiguous()
            check(rm.ref_raymarch_bwd(p(x), p(gx), p(buf), p(cnt), i64(x.shape), hp(M), hp(V), hp(P), hp(F), len(V),
                                      1, 0, 0, 1, p(y), p(g), i64(out6)), 'ref_raymarch_bwd')
            return gx, None, None, None, None, None

    def sample_grid_lut(input, lookup, interpolation='LINEAR', boundary='BORDER', separate_camera_batch=True,
                        relative_coords=True, **kw):
        assert not separate_camera_batch and relative_coords
        return Lut.apply(input, lookup, FILTER[interpolation], BOUNDARY[boundary])

    def sample_grid_transform(input, matrix_m, matrix_v, matrix_p, frustum_params, output_shape,
                              interpolation='LINEAR', boundary='BORDER', mipmapping='NONE', num_mipmaps=0,
                              mip_bias=0.0, coordinate_mode='TRANSFORM_LINDEPTH', separate_camera_batch=True, **kw):
        x = input.detach().contiguous()
        nv = len(matrix_v)
        Do, Ho, Wo = [int(v) for v in output_shape]
        N = x.shape[0]
        out = torch.empty((N, nv, Do, Ho, Wo, x.shape[-1]), device=x.device)
        atlas = torch.empty(mip_atlas_bytes(tuple(x.shape[1:4]), x.shape[-1], num_mipmaps), dtype=torch.uint8,
                            device=x.device)
        check(rs.ref_sample_transform(p(x), i64(x.shape), hp(np.asarray(matrix_m)[:N]), hp(matrix_v), hp(matrix_p),
                                      hp(frustum_params), nv, p(atlas), COORD[coordinate_mode], FILTER[interpolation],
                                      BOUNDARY[boundary], MIP[mipmapping], int(num_mipmaps), ctypes.c_float(mip_bias),
                                      1, p(out), i64(out.shape)), 'ref_sample_transform')
        return out

    def reduce_grid_blend(input, blending_mode='BEER_LAMBERT', keep_dims=False):
        assert blending_mode == 'BEER_LAMBERT' and keep_dims
        return Blend.apply(input)

    def raymarch_grid_transform(input, matrix_m, matrix_v, matrix_p, frustum_params, output_shape, *a, **kw):
        return Raymarch.apply(input, matrix_m, matrix_v, matrix_p, frustum_params, tuple(int(v) for v in output_shape))

    return dict(sample_grid_lut=sample_grid_lut, sample_grid_transform=sample_grid_transform,
                reduce_grid_blend=reduce_grid_blend, raymarch_grid_transform=raymarch_grid_transform)


def timed_steps(fn, steps, warmup):
    for _ in range(warmup):
        fn()
    torch.cuda.synchronize()
    ts = []
    for _ in range(steps):
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        a.record()
        fn()
        b.record()
        torch.cuda.synchronize()
        ts.append(a.elapsed_time(b))
        hp.keep.clear()
    return float(np.median(ts))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument('--config', default='cfg2')
    ap.add_argument('--steps', type=int, default=5)
    ap.add_argument('--out', default=None)
    args = ap.parse_args()
    from oracle.ref import build_ref
    from gft import autotune, ops
    from gft.pipeline import RenderAdvectStep
    build_ref.build(quiet=True)
    libs = {n: ctypes.CDLL(os.path.join(REF, 'libref_%s.so' % n)) for n in ('raymarch', 'resample', 'blend')}
    dev = torch.device('cuda', 0)
    ops.set_grad_mode('REFERENCE')
    res = {'config': args.config}

    # this repository's batched step (BF16 and FP32 storage), tuned and captured
    plain = RenderAdvectStep(args.config, dev, mode='plain')
    inputs = plain.make_inputs()
    for name, dt in (('batched_bf16', torch.bfloat16), ('batched_f32', None)):
        with autotune.knob_settings(autotune.knobs()):
            st = RenderAdvectStep(args.config, dev, storage_dtype=dt, mode='batched', autotune=True)
            st.setup_static(inputs)
            st.capture(warmup=3)
            res[name + '_ms'] = timed_steps(st.replay, max(args.steps, 10), 3)
            res[name + '_loss'] = float(st.g_loss)
        del st
        torch.cuda.empty_cache()
    # the plain per-op step on this repository's kernels
    plain.setup_static(inputs)
    res['plain_ours_ms'] = timed_steps(plain.run_static, args.steps, 2)
    res['plain_ours_loss'] = float(plain.run_static()[0])
    # the same plain step on the reference's kernels
    saved = {k: getattr(ops, k) for k in ('sample_grid_lut', 'sample_grid_transform', 'reduce_grid_blend',
                                          'raymarch_grid_transform')}
    try:
        for k, f in reference_ops(libs).items():
            setattr(ops, k, f)
        t0 = time.perf_counter()
        res['plain_reference_kernels_ms'] = timed_steps(plain.run_static, args.steps, 2)
        loss, grads = plain.run_static()
        torch.cuda.synchronize()
        res['plain_reference_kernels_loss'] = float(loss)
        res['plain_reference_wall_s'] = time.perf_counter() - t0
    finally:
        for k, f in saved.items():
            setattr(ops, k, f)
    res['speedup_batched_bf16_vs_plain_reference_kernels'] = res['plain_reference_kernels_ms'] / res['batched_bf16_ms']
    res['speedup_batched_bf16_vs_plain_ours'] = res['plain_ours_ms'] / res['batched_bf16_ms']
    s = json.dumps(res)
    print(s)
    if args.out:
        with open(args.out, 'w') as f:
            f.write(s + '\n')


if __name__ == '__main__':
    main()
