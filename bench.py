"""Benchmark: fwd+bwd render + advect iterations per second on one GB300.

Workload (default ``cfg2``, the multi-view frame configuration): plume density
128x227x128 advected one MacCormack step (MC_SMOOTH, CLAMP) by a staggered
curl-noise velocity field, spot light with a 256x196x196 shadow frustum (3 mip
levels, inverse-resampling gradients), 5 perspective views of 480x270 with 192
depth samples, fused Beer-Lambert raymarch, L2 image loss against seeded target
renders; one step = forward + backward to the previous density and all three
velocity components.  Synthetic seeded data stand in for ScalarFlow.

Arms:
  default            this repo: batched kernels, whole step in one CUDA graph
  --impl reference   the FP64 NumPy port of the reference ops on the host cores
                     (the reference's ops are CUDA-only TensorFlow kernels)

One JSON line on stdout (rank 0).
"""
import argparse
import json
import os
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, 'global-flow-transport_gb300')
for _p in (ROOT, PKG):
    if _p not in sys.path:
        sys.path.insert(0, _p)

METRIC = 'fwd+bwd render+advect iters/s'
L2_BYTES = 129 * 1024 * 1024


def _peaks():
    try:
        with open(os.path.join(ROOT, 'MEASURED_PEAKS.json')) as f:
            p = json.load(f)
        return float(p['hbm_gbs']), 'measured'
    except Exception:
        return 6800.0, 'fallback'


class ClockSampler:
    """nvidia-smi clocks/throttle sampling (every 50 ms) around the timed
    region.  A reader thread stamps each sample on arrival; the summary keeps
    the samples inside [start, stop] of the region (mark()/__exit__), widened
    to the nearest three samples when the region is shorter than that."""
    Q = ('index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,'
         'clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,'
         'clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap')

    def __init__(self, gpu_index, out_path=None):
        self.idx = gpu_index
        self.out_path = out_path
        self.proc = None
        self.samples = []  # (arrival time, line)
        self.t0 = self.t1 = None

    def _read(self):
        for line in self.proc.stdout:
            if line.strip():
                self.samples.append((time.perf_counter(), line.strip()))

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(['nvidia-smi', '-i', str(self.idx), '--query-gpu=' + self.Q,
                                          '--format=csv,noheader,nounits', '-lms', '50'],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
            t_end = time.perf_counter() + 3.0
            while not self.samples and time.perf_counter() < t_end:  # sampler running before the region
                time.sleep(0.01)
        except Exception:
            self.proc = None
        return self

    def mark(self):
        self.t0 = time.perf_counter()

    def __exit__(self, *a):
        self.t1 = time.perf_counter()
        if self.proc is not None:
            time.sleep(0.06)  # one more sample after the region
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
            self.thread.join(timeout=2)
        t0 = self.t0 if self.t0 is not None else self.t1
        inside = [l for t, l in self.samples if t0 <= t <= self.t1 + 0.055]
        if len(inside) < 3 and self.samples:
            mid = 0.5 * (t0 + self.t1)
            inside = [l for _, l in sorted(self.samples, key=lambda s: abs(s[0] - mid))[:3]]
        self.lines = inside
        if self.out_path:
            with open(self.out_path, 'w') as f:
                f.write('\n'.join(l for _, l in self.samples) + '\n')

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ['hw_slowdown', 'hw_thermal_slowdown', 'sw_thermal_slowdown', 'sw_power_cap']
        for l in getattr(self, 'lines', []):
            f = [x.strip() for x in l.split(',')]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower() == 'active':
                    reasons.add(n)
        sm.sort()
        return {'sm_mhz': sm[len(sm) // 2] if sm else None, 'sm_max_mhz': mx, 'reasons': sorted(reasons),
                'samples': len(sm)}


def max_over_ranks(value, device):
    """Max of a per-rank scalar over the process group (the slowest replica
    defines the step time), followed by a barrier."""
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    dist.barrier()
    return float(t.item())


def _ddp():
    ws = int(os.environ.get('WORLD_SIZE', '1'))
    rank = int(os.environ.get('RANK', '0'))
    local = int(os.environ.get('LOCAL_RANK', '0'))
    return ws, rank, local


def bench_ours(args):
    import numpy as np
    import torch
    from gft import _lib, ops
    from gft.pipeline import RenderAdvectStep

    ws, rank, local = _ddp()
    torch.cuda.set_device(local)
    dev = torch.device('cuda', local)
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group('nccl', device_id=dev)
    lib = _lib.load()
    storage = torch.bfloat16 if args.storage == 'bf16' else None
    ops.set_grad_mode(args.grad_mode)

    step = RenderAdvectStep(args.config, dev, storage_dtype=storage, mode='batched')
    inputs = step.make_inputs(frame=rank)
    step.setup_static(inputs)
    n0 = lib.gft_launch_count()
    step.capture(warmup=args.warmup)
    launches_per_step = (lib.gft_launch_count() - n0) // (args.warmup + 1)
    flush = torch.empty(2 * L2_BYTES // 4, dtype=torch.float32, device=dev)

    def timed(fn, k, flush_l2=True):
        evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(k)]
        for i in range(k):
            if flush_l2:
                flush.fill_(float(i))
            evs[i][0].record()
            fn()
            evs[i][1].record()
        torch.cuda.synchronize()
        return [a.elapsed_time(b) for a, b in evs]

    # ---- timed region: graph replays, L2 flushed between steps -------------
    for _ in range(args.warmup):
        step.replay()
    torch.cuda.synchronize()
    if ws > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    with ClockSampler(local, args.save_clocks) as cs:
        cs.mark()
        t_wall0 = time.perf_counter()
        times = timed(step.replay, args.steps)
        t_wall = time.perf_counter() - t_wall0
    ms = float(np.mean(times))
    if ws > 1:
        ms = max_over_ranks(ms, dev)
    loss_val = float(step.g_loss.item())

    result = {}
    if rank == 0 and not args.quick:
        result = extras(args, step, dev, timed, storage, inputs, ms)
    clocks = cs.summary()
    if rank != 0:
        if ws > 1:
            torch.distributed.destroy_process_group()
        return
    value = ws * 1000.0 / ms
    line = {
        'metric': METRIC, 'value': value, 'unit': 'iters/s', 'n_gpus': ws, 'steps': args.steps,
        'warmup': args.warmup, 'ms_per_step': ms, 'higher_is_better': True, 'scaling': 'weak',
        'vs_baseline': None, 'dtype': 'f32' if storage is None else 'bf16-storage/f32',
        'data': 'synthetic (seeded plume + curl-noise velocity; ScalarFlow absent)',
        'config': {'workload': '%s: density %s, MacCormack advect, spot-light shadow %s (%d mips), %d views %dx%d x%d '
                               'samples, L2 image loss, fwd+bwd' % (args.config, 'x'.join(map(str, step.shape)),
                                                                   'x'.join(map(str, step.shadow_res)), step.rs.num_mips,
                                                                   len(step.cams), step.res[1], step.res[2],
                                                                   step.res[0]),
                   'grad_mode': args.grad_mode, 'cuda_graph': True,
                   'l2': 'flushed between timed steps (write of 258 MB)', 'parallelism': 'replicas' if ws > 1 else 'single'},
        'gpu_launches': int(launches_per_step * args.steps),
        'launches_per_step': int(launches_per_step),
        'loss': loss_val,
        'wall_s_timed': t_wall,
        'clocks': clocks,
    }
    line.update(result)
    print(json.dumps(line), flush=True)
    if ws > 1:
        torch.distributed.destroy_process_group()


def extras(args, step, dev, timed, storage, inputs, ms):
    """e2e through the public API, the plain per-op path, per-kernel roofline
    and the CPU baseline."""
    import numpy as np
    import torch
    from gft import ops
    from gft.pipeline import RenderAdvectStep
    out = {}
    # ---- e2e: pinned host inputs -> device, graph step, loss -> host ----------
    # Through the public streaming API (gft.pipeline.StreamedSteps): every
    # step copies its own inputs (two frames' inputs alternate) from pinned
    # host memory and reads its loss back; the copy of step i+1's inputs
    # overlaps step i.  e2e_serial: one step at a time, the host waiting for
    # each loss before it copies the next inputs.
    from gft.pipeline import StreamedSteps
    hosts = [StreamedSteps.host_inputs(inputs), StreamedSteps.host_inputs(step.make_inputs(frame=1))]
    h2d = StreamedSteps.h2d_bytes(hosts[0])
    streamed = StreamedSteps(step, inputs, warmup=args.warmup)
    k = min(max(6, args.steps // 2), 60)
    streamed.run([hosts[i % 2] for i in range(4)])
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    losses = streamed.run([hosts[i % 2] for i in range(k)])
    e2e_ms = (time.perf_counter() - t0) * 1000.0 / k
    out['e2e'] = {'value': 1000.0 / e2e_ms, 'unit': 'iters/s', 'h2d_bytes_per_step': int(h2d),
                  'd2h_bytes_per_step': 4, 'ms_per_step': e2e_ms, 'steps': k,
                  'what': 'StreamedSteps: per-step H2D of pinned inputs overlapping the previous step, loss read '
                          'back one step later', 'loss_last': losses[-1]}

    def serial_step(host):
        return streamed.run([host])[0]

    for i in range(2):
        serial_step(hosts[i % 2])
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for i in range(k):
        serial_step(hosts[i % 2])
    ser_ms = (time.perf_counter() - t0) * 1000.0 / k
    out['e2e_serial'] = {'value': 1000.0 / ser_ms, 'unit': 'iters/s', 'ms_per_step': ser_ms,
                         'what': 'one step at a time: copy inputs, replay, read the loss, wait'}
    del streamed

    # ---- plain: per-camera launches, composed advection, no graph -----------
    plain = RenderAdvectStep(args.config, dev, storage_dtype=None, mode='plain')
    plain.setup_static(inputs)
    for _ in range(2):
        plain.run_static()
    torch.cuda.synchronize()
    pt = timed(plain.run_static, min(max(3, args.steps // 3), 30))
    out['plain'] = {'value': 1000.0 / float(np.mean(pt)), 'unit': 'iters/s', 'ms_per_step': float(np.mean(pt)),
                    'what': 'same step, one raymarch launch per camera, advection from 4 SampleGridLut calls + '
                            'elementwise ops, no CUDA graph'}
    out['batched_vs_plain'] = out['plain']['ms_per_step'] / ms
    del plain

    # ---- per-kernel timing of the dominant ops (roofline) -------------------
    out.update(kernel_roofline(step, dev, timed))
    out['static_cameras'] = static_cameras(args, dev, timed, storage, inputs)
    out['uneven_views'] = uneven_views(dev, timed)
    out['transport_chain'] = transport_chain(step, dev, timed)

    # ---- CPU baseline ------------------------------------------------------------
    if not args.no_cpu:
        try:
            from oracle import cpu_step
            out['cpu_baseline'] = cpu_step.time_step(step, inputs, budget_s=args.cpu_budget, workers=1)
        except Exception as e:  # the baseline is reported, not required
            out['cpu_baseline'] = {'error': repr(e)}
    return out


def static_cameras(args, dev, timed, storage, inputs):
    """The same graph step with ops.set_raymarch_weight_cache(True): for a
    fixed camera rig the reference-normalised gradient's weight sums depend on
    the geometry alone, so they are computed once and reused instead of in
    every step (opt-in; the headline number recomputes them every step)."""
    import numpy as np
    from gft import ops
    from gft.pipeline import RenderAdvectStep
    if args.grad_mode != 'REFERENCE':
        return None
    ops.set_raymarch_weight_cache(True)
    try:
        st = RenderAdvectStep(args.config, dev, storage_dtype=storage, mode='batched')
        st.setup_static(inputs)
        st.capture(warmup=args.warmup)
        for _ in range(3):
            st.replay()
        t = timed(st.replay, min(max(10, args.steps // 2), 100))
        return {'ms_per_step': float(np.mean(t)), 'value': 1000.0 / float(np.mean(t)), 'unit': 'iters/s',
                'what': 'cached raymarch weight sums (fixed cameras), otherwise the timed step'}
    finally:
        ops.set_raymarch_weight_cache(False)


def transport_chain(step, dev, timed, frames=16, every=4):
    """The global-transport chain on the step's workload: an initial density
    and 15 seeded staggered velocity fields, MacCormack advection through 16
    frames, every frame rendered by the 5 views and compared with its target,
    gradients to the initial density and all velocities, the adjoint
    recomputing each 4-frame segment from its stored first density
    (gft.chain.TransportChain).  One CUDA graph per iteration when capture
    succeeds, else eager."""
    import numpy as np
    import torch
    from gft import synthetic as syn
    from gft.chain import TransportChain
    shape = step.shape
    d0 = torch.from_numpy(syn.plume_density(shape, 3000)).to(dev).requires_grad_(True)
    vels = []
    for t in range(frames - 1):
        vx, vy, vz = syn.curl_velocity(shape, 3100 + t)
        vels.append(tuple(torch.from_numpy(v).to(dev).requires_grad_(True) for v in (vx, vy, vz)))
    with torch.no_grad():
        targets = [step.render(torch.from_numpy(syn.plume_density(shape, 3200 + t, t)).to(dev))[..., :3].contiguous()
                   for t in range(frames)]
    chain = TransportChain(step, frames=frames, checkpoint_every=every)
    params = [d0] + [v for tr in vels for v in tr]

    def it():
        loss = chain.loss(d0, vels, targets)
        return loss, torch.autograd.grad(loss, params)

    graph, why = None, None
    try:
        side = torch.cuda.Stream(dev)
        side.wait_stream(torch.cuda.current_stream(dev))
        with torch.cuda.stream(side):
            for _ in range(2):
                it()
        torch.cuda.current_stream(dev).wait_stream(side)
        torch.cuda.synchronize(dev)
        graph = torch.cuda.CUDAGraph()
        with torch.cuda.graph(graph):
            out = it()
        run = graph.replay
    except Exception as e:
        graph, why = None, repr(e)[:200]
        torch.cuda.synchronize(dev)
        run = it
    run()
    ms = float(np.median(timed(run, 5, flush_l2=False)))
    return {'workload': '%d frames, density %s, 5 views, MacCormack chain, fwd+bwd to the initial density and all '
                        'velocities, checkpoint every %d frames' % (frames, 'x'.join(map(str, shape)), every),
            'ms_per_iteration': ms, 'iters_per_s': 1000.0 / ms, 'cuda_graph': graph is not None,
            'frames_per_s': frames * 1000.0 / ms, **({'capture_error': why} if why else {})}


def uneven_views(dev, timed):
    """One frame of the uneven-view batch workload: density 96x170x96 (C = 4
    light + density), one fixed 256x256 view plus 8 seeded upper-hemisphere
    views of 64-256 pixels square, 128 samples, reference-normalised gradient.
    Raymarch forward + adjoint of all 9 views in one launch each
    (raymarch_grid_transform_multi) against one launch per view (the
    reference's structure: one call per image size)."""
    import numpy as np
    import torch
    from gft import ops
    from gft import synthetic as syn
    from phitest.render.transform import GridTransform
    shape = (96, 170, 96)
    gt = GridTransform(list(shape), center=True, normalize='MIN')
    M = syn.model_matrix(gt)
    cams, shapes = syn.hemisphere_cameras(8, 128, seed=4000)
    V, P, F = syn.camera_params(cams)
    d = torch.from_numpy(syn.plume_density(shape, 4000)).to(dev)
    x = (torch.cat([d * 0.7, d * 0.5, d * 0.3, d], -1) * 0.02).contiguous()
    ref = ops.GRAD['REFERENCE']
    y = ops._raymarch_multi_fwd(x, M, V, P, F, [list(s) for s in shapes], 1, 0, 0)
    torch.manual_seed(0)
    dy = torch.randn_like(y) * 1e-3
    sl = [list(s) for s in shapes]

    def multi():
        yy = ops._raymarch_multi_fwd(x, M, V, P, F, sl, 1, 0, 0)
        ops._raymarch_multi_bwd(x, yy, dy, M, V, P, F, sl, 1, 0, 0, ref)

    offs = np.cumsum([0] + [h * w for _, h, w in shapes])
    dys = [dy[:, offs[c]:offs[c + 1]].reshape(1, 1, shapes[c][1], shapes[c][2], 4).contiguous()
           for c in range(len(shapes))]

    def per_view():
        for c, s in enumerate(shapes):
            yc = ops._raymarch_fwd(x, M, V[c:c + 1], P[c:c + 1], F[c:c + 1], s, 1, 0, 0, True)
            ops._raymarch_bwd(x, yc, dys[c], M, V[c:c + 1], P[c:c + 1], F[c:c + 1], s, 1, 0, 0, True, ref)

    for _ in range(2):
        multi(), per_view()
    tm = float(np.median(timed(multi, 7)))
    tp = float(np.median(timed(per_view, 7)))
    return {'workload': 'density 96x170x96, views 256^2 + 8 x (64-256)^2 upper hemisphere, 128 samples, '
                        'raymarch fwd + reference-normalised adjoint',
            'sizes': [s[1] for s in shapes], 'one_launch_ms': tm, 'per_view_ms': tp, 'speedup': tp / tm}


SCATTER_PROFILE = os.path.join(ROOT, 'profiles', 'raymarch_scatter_cfg2.md')


def _profiled_traffic():
    """DRAM bytes per launch of the raymarch adjoint scatter pass from the
    committed ncu summary (its ``dram_bytes_per_launch:`` line), else None."""
    try:
        with open(SCATTER_PROFILE) as f:
            for line in f:
                if line.strip().startswith('dram_bytes_per_launch:'):
                    return int(line.split(':', 1)[1].strip().split()[0])
    except (OSError, ValueError):
        pass
    return None


def _clipped_samples(step):
    """Ray samples inside the raymarch's clipped step ranges at this workload
    (the kernels' BORDER slab test, in float64): the samples the forward
    stores and the adjoint reads back."""
    import numpy as np
    D, H, W = step.res
    gz, gy, gx = step.shape
    m = np.asarray(step.M, np.float64)[0].T
    ys, xs = np.meshgrid(np.arange(H) + 0.5, np.arange(W) + 0.5, indexing='ij')
    zmax = max(D - 1, 1)
    hi = np.array([gx, gy, gz], np.float64) + 0.55
    total = 0
    for c in range(len(step.cams)):
        inv = np.linalg.inv(np.asarray(step.V, np.float64)[c].T @ m) @ np.linalg.inv(np.asarray(step.P, np.float64)[c].T)

        def os_at(zi):
            ndc = np.stack([xs / W * 2 - 1, ys / H * 2 - 1, np.full_like(xs, zi / D * 2 - 1), np.ones_like(xs)], -1)
            h = ndc @ inv.T
            return h[..., :3] / h[..., 3:4]
        near = os_at(0.5)
        st = (os_at(zmax + 0.5) - near) / zmax
        with np.errstate(divide='ignore', invalid='ignore'):
            a, b = (-1.05 - near) / st, (hi - near) / st
        t0 = np.maximum(0.0, np.max(np.minimum(a, b), -1))
        t1 = np.minimum(D - 1.0, np.min(np.maximum(a, b), -1))
        i0, i1 = np.maximum(0, np.floor(t0) - 1), np.minimum(D - 1, np.ceil(t1) + 1)
        total += int(np.sum(np.where(t0 <= t1, i1 - i0 + 1, 0)))
    return total


def kernel_roofline(step, dev, timed):
    """Times the render kernels alone with CUDA events on their stream (L2
    flushed before each launch) and converts the algorithmic bytes per launch
    into GB/s against the measured HBM peak.  The dominant kernel is the
    raymarch adjoint's scatter pass (k_raymarch_scatter, one launch for the 5
    views) as the step runs it: reading the samples the forward stored, with
    its per-camera weight sums precomputed (GFT_GRAD_WEIGHTS_READY: a gradient
    memset plus the scatter launch)."""
    import numpy as np
    import torch
    from gft import ops
    peak, src = _peaks()
    with torch.no_grad():
        d = step.advect(step.s_d, step.s_vx, step.s_vy, step.s_vz)
        light = d * (step.shadow(d) * step.falloff_col + step.ambient)
        # the raymarch input in the brick layout the step uses
        data = ops.to_bricks((torch.cat([light, d], dim=-1) * step.depth_step).contiguous())
    grid = step.shape
    D, H, W = step.res
    V = len(step.cams)
    mode = ops.get_grad_mode()
    shape5 = (data.shape[0],) + tuple(grid) + (data.shape[-1],)
    smp = ops._samples_buffer(shape5, V, step.res, True, dev)
    fwd = lambda: ops._raymarch_fwd(data, step.M, step.V, step.P, step.F, step.res, 1, 0, 0, True, grid=grid,
                                    samples=smp)
    y = fwd()
    torch.manual_seed(0)
    dy = torch.randn_like(y) * 1e-3
    bwd = lambda m: ops._raymarch_bwd(data, y, dy, step.M, step.V, step.P, step.F, step.res, 1, 0, 0, True,
                                      ops.GRAD[m], grid=grid, samples=smp)
    weights = lambda: ops._raymarch_weights(shape5, data.device, step.M, step.V, step.P, step.F, step.res, 0, True)
    ws = weights()
    scatter = lambda: ops._raymarch_bwd(data, y, dy, step.M, step.V, step.P, step.F, step.res, 1, 0, 0, True,
                                        ops.GRAD['REFERENCE'], weights=ws, grid=grid, samples=smp)
    resample = lambda: ops._raymarch_bwd(data, y, dy, step.M, step.V, step.P, step.F, step.res, 1, 0, 0, True,
                                         ops.GRAD['REFERENCE'], weights=ws, grid=grid)
    for _ in range(2):
        fwd(), bwd('REFERENCE'), bwd('EXACT'), weights(), scatter(), resample()
    tf = float(np.median(timed(fwd, 7)))
    tb_ref = float(np.median(timed(lambda: bwd('REFERENCE'), 7)))
    tb_ex = float(np.median(timed(lambda: bwd('EXACT'), 7)))
    tw = float(np.median(timed(weights, 7)))
    ts = float(np.median(timed(scatter, 7)))
    tr = float(np.median(timed(resample, 7)))
    nvox = int(np.prod(step.shape))
    s, C = 4, 4
    pix = V * H * W
    samples = pix * D
    # bytes of the sample store written / read: the samples the forward stored
    # (inside the clipped ranges and outside empty occupancy blocks)
    n_stored = ops.stored_sample_count(smp, shape5, V, step.res)
    stored = n_stored * C * 4
    bytes_fwd = nvox * C * s + pix * C * 4 + stored
    # scatter pass: stored samples read, image + adjoint read, per-camera
    # reciprocal weights read, gradient read-modify-write
    bytes_scatter = stored + 2 * pix * C * 4 + V * nvox * 4 + 2 * nvox * C * 4
    bytes_resample = nvox * C * s + 2 * pix * C * 4 + V * nvox * 4 + 2 * nvox * C * 4
    bytes_exact = stored + 2 * pix * C * 4 + 2 * nvox * C * 4
    bytes_weights = 2 * V * nvox * 4
    kern = {
        'raymarch_fwd': {'ms': tf, 'alg_bytes': bytes_fwd, 'GBps': bytes_fwd / tf / 1e6,
                         'samples_per_s': samples / tf * 1e3},
        'raymarch_bwd_scatter': {'ms': ts, 'alg_bytes': bytes_scatter, 'GBps': bytes_scatter / ts / 1e6,
                                 'samples_per_s': samples / ts * 1e3,
                                 'what': 'reference normalisation, weights ready, stored samples'},
        'raymarch_bwd_scatter_resampling': {'ms': tr, 'alg_bytes': bytes_resample, 'GBps': bytes_resample / tr / 1e6,
                                            'what': 'the same pass re-sampling the grid (no sample store)'},
        'raymarch_samples_stored_bytes': stored,
        'raymarch_samples_in_clipped_ranges': _clipped_samples(step),
        'raymarch_samples_stored': n_stored,
        'raymarch_bwd_weights': {'ms': tw, 'alg_bytes': bytes_weights, 'GBps': bytes_weights / tw / 1e6,
                                 'samples_per_s': samples / tw * 1e3},
        'raymarch_bwd_reference': {'ms': tb_ref, 'what': 'whole op: weights + inversion + scatter'},
        'raymarch_bwd_exact': {'ms': tb_ex, 'alg_bytes': bytes_exact, 'GBps': bytes_exact / tb_ex / 1e6,
                               'samples_per_s': samples / tb_ex * 1e3},
        'grad_mode': mode,
    }
    traffic = _profiled_traffic()
    return {'roofline': {'kernel': 'k_raymarch_scatter (raymarch adjoint scatter pass, 5 views)', 'bound': 'hbm',
                         'achieved': kern['raymarch_bwd_scatter']['GBps'], 'peak': peak, 'unit': 'GB/s',
                         'frac': kern['raymarch_bwd_scatter']['GBps'] / peak, 'peak_source': src,
                         'traffic': traffic, 'alg_bytes': bytes_scatter,
                         'traffic_source': 'ncu dram__bytes_read.sum + dram__bytes_write.sum, one launch, '
                                           'profiles/raymarch_scatter_cfg2.md' if traffic else None,
                         'note': 'algorithmic bytes = compulsory unique traffic (the stored samples the pass '
                                 'reads, image and adjoint, reciprocal weights, gradient read-modify-write); the '
                                 'pass is bound by the L1/L2 path of its merged trilinear gradient reductions and '
                                 'by latency, not by HBM'},
            'kernels': kern}


def kernel_only(args):
    """Runs one op of the cfg workload ``args.repeat`` times without a graph
    (for ncu captures of a single kernel)."""
    import torch
    from gft import ops
    from gft.pipeline import RenderAdvectStep
    dev = torch.device('cuda', 0)
    ops.set_grad_mode(args.grad_mode)
    step = RenderAdvectStep(args.config, dev, mode='batched')
    inputs = step.make_inputs()
    step.setup_static(inputs)
    with torch.no_grad():
        d = step.advect(step.s_d, step.s_vx, step.s_vy, step.s_vz)
        light = d * (step.shadow(d) * step.falloff_col + step.ambient)
        data = ops.to_bricks((torch.cat([light, d], dim=-1) * step.depth_step).contiguous())
        grid = step.shape
        smp = ops._samples_buffer((1,) + tuple(grid) + (4,), len(step.cams), step.res, True, dev)
        y = ops._raymarch_fwd(data, step.M, step.V, step.P, step.F, step.res, 1, 0, 0, True, grid=grid, samples=smp)
        dy = torch.randn_like(y) * 1e-3
    gm = ops.GRAD[ops.get_grad_mode()]
    fns = {
        'raymarch_fwd': lambda: ops._raymarch_fwd(data, step.M, step.V, step.P, step.F, step.res, 1, 0, 0, True,
                                                  grid=grid, samples=smp),
        'raymarch_bwd': lambda: ops._raymarch_bwd(data, y, dy, step.M, step.V, step.P, step.F, step.res, 1, 0, 0,
                                                  True, gm, grid=grid, samples=smp),
        'advect_fwd': lambda: ops._advect_fwd(step.s_d.detach(), step.s_vx.detach(), step.s_vy.detach(),
                                              step.s_vz.detach(), 1.0, 2, 1, 1),
        'advect_bwd': lambda: ops._advect_bwd(step.s_d.detach(), step.s_vx.detach(), step.s_vy.detach(),
                                              step.s_vz.detach(), torch.ones_like(d), 1.0, 2, 1, 1, gm),
        'shadow_fwd': lambda: step.shadow(d),
        'raymarch_weights': lambda: ops._raymarch_weights((1,) + tuple(grid) + (4,), data.device, step.M, step.V,
                                                          step.P, step.F, step.res, 0, True),
    }
    if args.kernel_only == 'raymarch_scatter':
        ws = ops._raymarch_weights((1,) + tuple(grid) + (4,), data.device, step.M, step.V, step.P, step.F, step.res,
                                   0, True)
        fns['raymarch_scatter'] = lambda: ops._raymarch_bwd(data, y, dy, step.M, step.V, step.P, step.F, step.res, 1,
                                                            0, 0, True, ops.GRAD['REFERENCE'], weights=ws,
                                                            grid=grid, samples=smp)
    fn = fns[args.kernel_only]
    for _ in range(args.repeat):
        fn()
    torch.cuda.synchronize()
    print(json.dumps({'kernel_only': args.kernel_only, 'repeat': args.repeat, 'ok': True}))


def bench_reference(args):
    """The reference's own implementation of the path is CUDA-only TensorFlow
    ops; its CPU stand-in is the FP64 NumPy port in oracle/, timed on a bounded
    sample of the same workload with all host cores."""
    ws, rank, _ = _ddp()
    if rank != 0:
        return
    from oracle import cpu_step
    workers = os.cpu_count() or 1
    res = cpu_step.time_step(None, None, budget_s=args.cpu_budget, workers=workers, config=args.config)
    v = res['value']
    line = {'impl': 'reference', 'metric': METRIC, 'value': v, 'unit': 'iters/s', 'n_gpus': ws, 'steps': args.steps,
            'warmup': args.warmup, 'ms_per_step': 1000.0 / v if v else None, 'higher_is_better': True,
            'scaling': 'weak', 'vs_baseline': None, 'dtype': 'f64', 'data': 'synthetic',
            'config': {'workload': args.config + ' (same step as the GPU arm)'},
            'cpu_baseline': res,
            'e2e': {'value': v, 'unit': 'iters/s', 'h2d_bytes_per_step': 0, 'd2h_bytes_per_step': 0}}
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument('--gpus', type=int, default=1)
    ap.add_argument('--steps', type=int, default=200)
    ap.add_argument('--warmup', type=int, default=3)
    ap.add_argument('--impl', default='ours', choices=['ours', 'reference'])
    ap.add_argument('--config', default='cfg2')
    ap.add_argument('--storage', default='f32', choices=['f32', 'bf16'])
    ap.add_argument('--grad-mode', default='REFERENCE', choices=['REFERENCE', 'EXACT'])
    ap.add_argument('--quick', action='store_true', help='only the timed graph replays')
    ap.add_argument('--no-cpu', action='store_true')
    ap.add_argument('--cpu-budget', type=float, default=20.0)
    ap.add_argument('--save-clocks', default=None, metavar='CSV', help='write every clock sample to this file')
    ap.add_argument('--kernel-only', default=None,
                    choices=['raymarch_fwd', 'raymarch_bwd', 'raymarch_weights', 'raymarch_scatter', 'advect_fwd',
                             'advect_bwd', 'shadow_fwd'],
                    help='run one op of the workload --repeat times (profiling)')
    ap.add_argument('--repeat', type=int, default=3)
    args = ap.parse_args()
    args.warmup = max(3, args.warmup)
    if args.kernel_only:
        kernel_only(args)
    elif args.impl == 'reference':
        bench_reference(args)
    else:
        bench_ours(args)


if __name__ == '__main__':
    main()
