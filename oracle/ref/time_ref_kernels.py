"""Times the reference's own CUDA kernels (oracle/_ref/libref_*.so, built by
oracle/ref/build_ref.py from the unchanged reference sources) beside this
repository's kernels, op by op, on the 5-view 128x227x128 render + advect
workload (images 270x480, 192 samples, shadow frustum 256x196x196, 3 mips).

ORACLE / TEST INFRASTRUCTURE ONLY: a measurement of the reference, not part of
the product.  The reference launchers synchronise the device after every op,
so both sides are timed as host wall time around synchronised calls (median
of ``--reps``), with the L2 flushed (a 258 MB write) before each call.

    python oracle/ref/build_ref.py && python oracle/ref/time_ref_kernels.py
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


def i64(v):
    return (ctypes.c_longlong * len(v))(*[int(x) for x in v])


def p(t):
    return ctypes.c_void_p(t.data_ptr())


def hp(a):
    return np.ascontiguousarray(a, dtype=np.float32).ctypes.data_as(ctypes.c_void_p)


def mip_atlas_bytes(shape, C, levels):
    """setupMipAtlas's size (resample_grid.cc:201-220) with generous slack."""
    n = ((levels + 1) * 8 + 127) // 128 * 128 + 128
    for m in range(1, levels + 1):
        e = (shape[0] >> m) * (shape[1] >> m) * (shape[2] >> m)
        if e <= 0:
            break
        n += (e * 4 * C + 127) // 128 * 128
    return 2 * n + 4096


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument('--reps', type=int, default=7)
    ap.add_argument('--out', default=None, help='write the JSON result here too')
    args = ap.parse_args()
    from gft import ops
    from gft.pipeline import RenderAdvectStep
    libs = {n: ctypes.CDLL(os.path.join(REF, 'libref_%s.so' % n)) for n in ('raymarch', 'resample', 'blend')}
    dev = torch.device('cuda', 0)
    step = RenderAdvectStep('cfg2', dev, mode='batched')
    inp = step.make_inputs()
    step.setup_static(inp)
    flush = torch.empty(258 * 2 ** 20 // 4, device=dev)

    def timed(fn):
        fn()
        torch.cuda.synchronize()
        ts = []
        for i in range(args.reps):
            flush.fill_(float(i))
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            fn()
            torch.cuda.synchronize()
            ts.append((time.perf_counter() - t0) * 1e3)
        return float(np.median(ts))

    def check(rc, what):
        if rc != 0:
            raise RuntimeError('%s returned %d' % (what, rc))

    with torch.no_grad():
        d = step.advect(step.s_d, step.s_vx, step.s_vy, step.s_vz).contiguous()
        light = d * (step.shadow(d) * step.falloff_col + step.ambient)
        data = (torch.cat([light, d], dim=-1) * step.depth_step).contiguous()
    D, H, W = step.res
    nv = len(step.V)
    C = 4
    res = {}
    rm, rs, bl = libs['raymarch'], libs['resample'], libs['blend']

    # raymarch forward: one fused launch per camera in the reference launcher
    out6 = [1, nv, D, H, W, C]
    y_ref = torch.empty((1, nv, H, W, C), device=dev)
    f_ref = lambda: check(rm.ref_raymarch_fwd(p(data), i64(data.shape), hp(step.M), hp(step.V), hp(step.P),
                                              hp(step.F), nv, 1, 0, 0, 1, p(y_ref), i64(out6)), 'ref_raymarch_fwd')
    f_our = lambda: ops._raymarch_fwd(data, step.M, step.V, step.P, step.F, step.res, 1, 0, 0, True)
    res['raymarch_fwd'] = (timed(f_ref), timed(f_our))
    y = f_our()
    torch.manual_seed(0)
    dy = torch.randn_like(y) * 1e-3
    # raymarch gradient, reference normalisation (per-camera weight sums)
    g_ref = torch.empty_like(data)
    buf = torch.empty(data.numel(), device=dev)
    cnt = torch.empty(data.numel() // C, device=dev)
    b_ref = lambda: check(rm.ref_raymarch_bwd(p(data), p(g_ref), p(buf), p(cnt), i64(data.shape), hp(step.M),
                                              hp(step.V), hp(step.P), hp(step.F), nv, 1, 0, 0, 1, p(y), p(dy),
                                              i64(out6)), 'ref_raymarch_bwd')
    b_our = lambda: ops._raymarch_bwd(data, y, dy, step.M, step.V, step.P, step.F, step.res, 1, 0, 0, True,
                                      ops.GRAD['REFERENCE'])
    res['raymarch_bwd'] = (timed(b_ref), timed(b_our))
    b_ref()
    g_our = b_our()
    torch.cuda.synchronize()
    res['raymarch_bwd_relL2'] = float((g_our - g_ref).double().norm() / g_ref.double().norm())
    # Conditioning: this repository's own gradient when the model matrix moves
    # by one float ulp (relative 2^-23), against the unperturbed one.
    M1 = (np.asarray(step.M, dtype=np.float64) * (1.0 + 2.0 ** -23)).astype(np.float32)
    g_pert = ops._raymarch_bwd(data, y, dy, M1, step.V, step.P, step.F, step.res, 1, 0, 0, True,
                               ops.GRAD['REFERENCE'])
    torch.cuda.synchronize()
    res['raymarch_bwd_one_ulp_matrix_relL2'] = float((g_pert - g_our).double().norm() / g_our.double().norm())
    # The same comparison with the adjoint that training feeds: the gradient of
    # the L2 image loss against the target renders (spatially smooth, unlike
    # the i.i.d. noise above, to which the scatter is most sensitive).
    from gft import fused
    yl = y.detach().clone().requires_grad_(True)
    fused.image_loss(yl[0], step.s_t, step.bkg_host).backward()
    dy_loss = yl.grad.contiguous()
    check(rm.ref_raymarch_bwd(p(data), p(g_ref), p(buf), p(cnt), i64(data.shape), hp(step.M), hp(step.V),
                              hp(step.P), hp(step.F), nv, 1, 0, 0, 1, p(y), p(dy_loss), i64(out6)), 'ref_raymarch_bwd')
    g_our = ops._raymarch_bwd(data, y, dy_loss, step.M, step.V, step.P, step.F, step.res, 1, 0, 0, True,
                              ops.GRAD['REFERENCE'])
    torch.cuda.synchronize()
    res['raymarch_bwd_loss_grad_relL2'] = float((g_our - g_ref).double().norm() / g_ref.double().norm())
    res['raymarch_fwd_relL2'] = float((f_our() - (f_ref() or y_ref)).double().norm() / y_ref.double().norm())

    # shadow pass: volume -> light frustum (LINDEPTH, LINEAR, BORDER, 3 mip levels)
    r = step.rs
    ds = (d * step.shadow_step).contiguous()
    sres = step.shadow_res
    levels = r.num_mips
    atlas = torch.empty(mip_atlas_bytes(step.shape, 1, levels), dtype=torch.uint8, device=dev)
    sh_ref = torch.empty((1, 1) + tuple(sres) + (1,), device=dev)
    s_ref = lambda: check(rs.ref_sample_transform(p(ds), i64(ds.shape), hp(step.M), hp(step.Vs), hp(step.Ps),
                                                  hp(step.Fs), 1, p(atlas), 0, 1, 0, 2, levels,
                                                  ctypes.c_float(r.mip_bias), 1, p(sh_ref),
                                                  i64([1, 1] + list(sres) + [1])), 'ref_sample_transform')
    s_our = lambda: ops.sample_grid_transform(ds, step.M, step.Vs, step.Ps, step.Fs, sres, 'LINEAR', 'BORDER',
                                              'LINEAR', levels, r.mip_bias, 'TRANSFORM_LINDEPTH')
    res['shadow_sample'] = (timed(s_ref), timed(s_our))
    s_ref()
    sh_our = s_our()
    torch.cuda.synchronize()
    res['shadow_sample_relL2'] = float((sh_our - sh_ref).double().norm() / sh_ref.double().norm())
    # depth blend of the shadow frustum
    sh = sh_our[0].contiguous()
    bo_ref = torch.empty_like(sh)
    l_ref = lambda: check(bl.ref_blend_fwd(p(sh), i64(sh.shape), 0, 1, p(bo_ref), i64(sh.shape)), 'ref_blend_fwd')
    l_our = lambda: ops.reduce_grid_blend(sh, 'BEER_LAMBERT', keep_dims=True)
    res['shadow_blend'] = (timed(l_ref), timed(l_our))
    # back projection: light frustum -> volume (LINDEPTH_REVERSE, mips)
    tr = torch.exp(-sh).contiguous()
    atlas2 = torch.empty(mip_atlas_bytes(tuple(sres), 1, levels), dtype=torch.uint8, device=dev)
    bp_ref_out = torch.empty((1, 1) + tuple(step.shape) + (1,), device=dev)
    p_ref = lambda: check(rs.ref_sample_transform(p(tr), i64(tr.shape), hp(step.M), hp(step.Vs), hp(step.Ps),
                                                  hp(step.Fs), 1, p(atlas2), 1, 1, 0, 2, levels,
                                                  ctypes.c_float(r.mip_bias), 1, p(bp_ref_out),
                                                  i64([1, 1] + list(step.shape) + [1])), 'ref_sample_transform rev')
    p_our = lambda: ops.sample_grid_transform(tr, step.M, step.Vs, step.Ps, step.Fs, step.shape, 'LINEAR', 'BORDER',
                                              'LINEAR', levels, r.mip_bias, 'TRANSFORM_LINDEPTH_REVERSE')
    res['shadow_backproject'] = (timed(p_ref), timed(p_our))

    # advection: the reference's MacCormack = 4 SampleGridLut calls (forward,
    # back, MIN, MAX; data_structures.py:870-905) plus tensor glue, against the
    # fused two-kernel advection here.
    from gft.pipeline import centered_lut
    lut = centered_lut(step.s_vx.detach(), step.s_vy.detach(), step.s_vz.detach(), 1.0).contiguous()
    d0 = step.s_d.detach().contiguous()
    shp6 = [1, 1] + list(step.shape) + [1]
    a_out = [torch.empty((1, 1) + tuple(step.shape) + (1,), device=dev) for _ in range(4)]
    atl = torch.empty(16, dtype=torch.uint8, device=dev)
    neg_lut = (-lut).contiguous()

    def adv_ref():
        for k, (src, lu, filt) in enumerate(((d0, lut, 1), (a_out[0][0], neg_lut, 1), (d0, lut, 2), (d0, lut, 3))):
            check(rs.ref_sample_lut(p(src), i64(src.shape), 1, p(lu), p(atl), filt, 1, 0, 0, ctypes.c_float(0.0),
                                    ctypes.c_float(0.0), 1, 1, 0, p(a_out[k]), i64(shp6)), 'ref_sample_lut')

    a_our = lambda: ops._advect_fwd(d0, step.s_vx.detach(), step.s_vy.detach(), step.s_vz.detach(), 1.0, 2, 1, 1)
    res['advect_fwd'] = (timed(adv_ref), timed(a_our))
    # advection adjoint: the reference's two SampleGridLutGrad calls against the fused adjoint
    gl_x = torch.empty_like(d0)
    gl_l = torch.empty_like(lut)
    gl_c = torch.empty(d0.numel(), dtype=torch.int32, device=dev)
    dyv = torch.ones((1, 1) + tuple(step.shape) + (1,), device=dev)

    def adv_bwd_ref():
        for src, lu in ((d0, lut), (a_out[0][0], neg_lut)):
            check(rs.ref_sample_lut_grad(p(src), i64(src.shape), 1, p(lu), 1, 1, ctypes.c_float(0.0), 1, 1, 0,
                                         p(dyv), i64(shp6), p(gl_x), p(gl_l), p(gl_c)), 'ref_sample_lut_grad')

    a_bwd_our = lambda: ops._advect_bwd(d0, step.s_vx.detach(), step.s_vy.detach(), step.s_vz.detach(),
                                        dyv[0], 1.0, 2, 1, 1, ops.GRAD['REFERENCE'])
    res['advect_bwd'] = (timed(adv_bwd_ref), timed(a_bwd_our))
    # as the step runs it: the adjoint reads the semi-Lagrangian grid the
    # forward left in the shared workspace (GFT_GRAD_FORWARD_READY)
    ws_adv = ops._advect_grad_workspace(d0.shape, 2, dev)
    ops._advect_fwd(d0, step.s_vx.detach(), step.s_vy.detach(), step.s_vz.detach(), 1.0, 2, 1, 1, ws=ws_adv)
    a_bwd_ready = lambda: ops._advect_bwd(d0, step.s_vx.detach(), step.s_vy.detach(), step.s_vz.detach(),
                                          dyv[0], 1.0, 2, 1, 1, ops.GRAD['REFERENCE'] | ops.FORWARD_READY, ws=ws_adv)
    res['advect_bwd_forward_ready'] = timed(a_bwd_ready)

    ops_rows = [k for k, v in res.items() if isinstance(v, tuple)]

    tot_ref = sum(res[k][0] for k in ops_rows)
    tot_our = sum(res[k][1] for k in ops_rows)
    out = {'workload': '5 views 480x270x192, density 128x227x128, shadow 256x196x196, 3 mips',
           'timing': 'host wall ms, median of %d, synchronised, L2 flushed' % args.reps,
           'ops': {k: {'reference_ms': res[k][0], 'ours_ms': res[k][1], 'speedup': res[k][0] / res[k][1]}
                   for k in ops_rows},
           'sum_reference_ms': tot_ref, 'sum_ours_ms': tot_our,
           'raymarch_fwd_relL2_vs_reference': res['raymarch_fwd_relL2'],
           'raymarch_bwd_relL2_vs_reference': res['raymarch_bwd_relL2'],
           'raymarch_bwd_relL2_vs_reference_image_loss_adjoint': res['raymarch_bwd_loss_grad_relL2'],
           'raymarch_bwd_relL2_own_one_ulp_matrix_change': res['raymarch_bwd_one_ulp_matrix_relL2'],
           'shadow_sample_relL2_vs_reference': res['shadow_sample_relL2'],
           'advect_bwd_ours_forward_ready_ms': res['advect_bwd_forward_ready']}
    s = json.dumps(out)
    print(s)
    if args.out:
        with open(args.out, 'w') as f:
            f.write(s + '\n')


if __name__ == '__main__':
    main()
