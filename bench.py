"""Benchmark: fwd+bwd render + advect iterations per second on one GB300.

Workload (default ``cfg5``, the largest configuration, with BF16 storage and
FP32 arithmetic): plume density 256x455x256 advected one MacCormack step
(MC_SMOOTH, CLAMP) by a staggered curl-noise velocity field, spot light with a
256x196x196 shadow frustum (4 mip levels, inverse-resampling gradients), 5
perspective portrait views of 540x960 (width x height) with 256 depth samples, fused Beer-Lambert
raymarch, L2 image loss against seeded target renders; one step = forward +
backward to the previous density and all three velocity components, replayed
from one CUDA graph.  Synthetic seeded data stand in for ScalarFlow.

Arms:
  default            this repo: batched kernels, whole step in one CUDA graph
  --impl reference   the reference's path on the host cores: its ops are
                     CUDA-only TensorFlow kernels, so its CPU stand-in is the
                     FP64 NumPy port in oracle/, run as whole iterations on all
                     cores (oracle/cpu_step.py FullStep)

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
DEFAULT_CONFIG = 'cfg5'
DEFAULT_STORAGE = 'bf16'


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




# ---------------------------------------------------------------- workload
def _storage_dtype(name):
    import torch
    return torch.bfloat16 if name == 'bf16' else None


def workload_config(config, storage, grad_mode):
    """The ``config`` object both arms print: the workload they run."""
    from gft.pipeline import CONFIGS
    c = CONFIGS[config]
    D, H, W = c['grid']
    Hi, Wi = c['image']  # rows, columns (the pipeline's order)
    return {'workload': '%s: density %dx%dx%d (raymarch input in %s storage, fp32 arithmetic), MacCormack advect '
                        '(MC_SMOOTH, CLAMP), '
                        'spot-light shadow %s (%d mips), %d views %dx%d (width x height) x%d samples, L2 image loss, '
                        'fwd+bwd'
                        % (config, D, H, W, storage, 'x'.join(map(str, c['shadow'])), c['mips'], c['views'], Wi, Hi,
                           c['samples']),
            'config': config, 'storage': storage, 'grad_mode': grad_mode,
            'l2': 'inputs larger than L2 (129 MB); the GPU arm also flushes L2 between timed steps'}


def alg_bytes(step, storage_bytes):
    """Compulsory unique bytes of one iteration by the per-op formulas of the
    path (s = bytes per stored grid element; the grids the shadow pass
    resamples, the velocities and every gradient are fp32):
      mips          sum over the 4 pyramids (two resampled grids, two resampled
                    gradients) of sum_m (N_m + N_m+1) * 4
      render fwd    N*4*s + P*4*4                 (P = views * H * W pixels)
      render bwd    N*4*s + 2*P*4*4 + 2*N*4*4
      shadow        2 * (N*4 + 2*S*4 + S*4 + N*4) (forward and its inverse-
                    resampling gradient; S frustum cells)
      advect fwd    N*s + F*4 + N*4               (F velocity faces)
      advect bwd    (2*N + 2*F)*4 + N*s
    Returns (total, per-part dict)."""
    import numpy as np
    D, H, W = step.shape
    N = D * H * W
    Dc, Hi, Wi = step.res
    P = len(step.cams) * Hi * Wi
    Ds, Hs, Ws = step.shadow_res
    S = Ds * Hs * Ws
    F = (W + 1) * H * D + W * (H + 1) * D + W * H * (D + 1)
    s = storage_bytes

    def pyramid(dims, L):
        tot, d = 0, tuple(dims)
        for _ in range(L):
            nxt = tuple(max(1, x // 2) for x in d)
            tot += (int(np.prod(d)) + int(np.prod(nxt))) * 4
            d = nxt
        return tot
    L = step.rs.num_mips
    parts = {
        'mips': 2 * pyramid((D, H, W), L) + 2 * pyramid((Ds, Hs, Ws), L),
        'render_fwd': N * 4 * s + P * 16,
        'render_bwd': N * 4 * s + 2 * P * 16 + 2 * N * 16,
        'shadow': 2 * (N * 4 + 2 * S * 4 + S * 4 + N * 4),
        'advect_fwd': N * s + F * 4 + N * 4,
        'advect_bwd': (2 * N + 2 * F) * 4 + N * s,
    }
    return sum(parts.values()), parts


# DRAM bytes (dram__bytes_read.sum + dram__bytes_write.sum) of one launch of
# the dominant kernel, from one ncu capture of
#   python bench.py --kernel-only raymarch_scatter_projected --config <c> --storage <s>
# (summaries in profiles/raymarch_scatter_<c>.md): cfg5 BF16, the projected
# MODE 1 launch, 2.17 GB read + 1.10 GB written.
SCATTER_TRAFFIC = {('cfg5', 'bf16'): 3.27e9}


# ------------------------------------------------------------------ our arm
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
    storage = _storage_dtype(args.storage)
    ops.set_grad_mode(args.grad_mode)

    step = RenderAdvectStep(args.config, dev, storage_dtype=storage, mode='batched')
    inputs = step.make_inputs(frame=rank)
    step.setup_static(inputs)
    tune_log = {}
    if args.knobs:
        # fixed launch-configuration knobs (e.g. for a profiler run of the tuned step)
        from gft import autotune
        autotune.apply({k: int(v) for k, v in (kv.split('=') for kv in args.knobs.split(','))})
        step.knobs = autotune.knobs()
    elif not args.no_autotune:
        # launch-configuration knobs timed on this workload before the capture
        from gft import autotune
        statics = (step.s_d, step.s_vx, step.s_vy, step.s_vz, step.s_t)
        step.knobs = autotune.tune(lambda: step.step(*statics), key=autotune.step_key(step), log=tune_log)
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
    total_bytes, parts = alg_bytes(step, 2 if storage is not None else 4)
    peak, src = _peaks()
    line = {
        'metric': METRIC, 'value': value, 'unit': 'iters/s', 'n_gpus': ws, 'steps': args.steps,
        'warmup': args.warmup, 'ms_per_step': ms, 'higher_is_better': True, 'scaling': 'weak',
        'vs_baseline': None, 'dtype': 'bf16-storage/f32' if storage is not None else 'f32',
        'data': 'synthetic (seeded plume + curl-noise velocity; ScalarFlow absent)',
        'config': workload_config(args.config, args.storage, args.grad_mode),
        'cuda_graph': True, 'parallelism': 'replicas' if ws > 1 else 'single',
        'gpu_launches': int(launches_per_step * args.steps),
        'launches_per_step': int(launches_per_step),
        'loss': loss_val,
        'wall_s_timed': t_wall,
        'clocks': clocks,
        'autotune': {'knobs': step.knobs, 'candidates_ms': tune_log} if step.knobs else None,
        'step_roofline': {'alg_bytes': total_bytes, 'parts': parts, 'achieved_GBps': total_bytes / ms / 1e6,
                          'peak': peak, 'frac': total_bytes / ms / 1e6 / peak, 'unit': 'GB/s',
                          'what': 'whole iteration: compulsory bytes by the per-op formulas / step time'},
    }
    line.update(result)
    print(json.dumps(line), flush=True)
    if ws > 1:
        torch.distributed.destroy_process_group()


def _load_inputs(step, inputs):
    """Copies make_inputs() arrays into a captured step's static inputs."""
    import torch
    with torch.no_grad():
        for dst, key, lead in ((step.s_d, 'd_prev', False), (step.s_vx, 'vx', True), (step.s_vy, 'vy', True),
                               (step.s_vz, 'vz', True), (step.s_t, 'target', False)):
            a = torch.from_numpy(inputs[key])
            dst.copy_(a[None] if lead else a)


def _grads_of(step, inputs):
    import torch
    _load_inputs(step, inputs)
    loss, grads = step.replay()
    torch.cuda.synchronize()
    return float(loss.detach()), [g.detach().float().clone() for g in grads]


def _rel(a, b):
    import torch
    n = float(torch.linalg.norm(b.double()))
    return float(torch.linalg.norm((a - b).double())) / (n if n > 0 else 1.0)


def extras(args, step, dev, timed, storage, inputs, ms):
    """e2e through the public API, the FP32 step beside the headline, the
    plain per-op FP32 path, the accuracy of BF16 storage, per-kernel
    roofline, the other workloads and the CPU baseline."""
    import numpy as np
    import torch
    from gft.pipeline import RenderAdvectStep, StreamedSteps
    out = {}
    # ---- e2e: pinned host inputs -> device, graph step, loss -> host ----------
    # Through the public streaming API (gft.pipeline.StreamedSteps): every
    # step copies its own inputs (two frames' inputs alternate) from pinned
    # host memory and reads its loss back; the copy of step i+1's inputs
    # overlaps step i.  e2e_serial: one step at a time, the host waiting for
    # each loss before it copies the next inputs.
    hosts = [StreamedSteps.host_inputs(inputs), StreamedSteps.host_inputs(step.make_inputs(frame=1))]
    h2d = StreamedSteps.h2d_bytes(hosts[0])
    streamed = StreamedSteps(step, inputs, warmup=args.warmup)
    # wall-clock over k steps per trial; three trials, the median one reported
    # (a host hiccup inside one short trial would otherwise set the figure)
    k = min(max(10, args.steps), 60)
    trials = 3
    streamed.run([hosts[i % 2] for i in range(4)])
    trial_ms = []
    for _ in range(trials):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        losses = streamed.run([hosts[i % 2] for i in range(k)])
        trial_ms.append((time.perf_counter() - t0) * 1000.0 / k)
    e2e_ms = float(np.median(trial_ms))
    out['e2e'] = {'value': 1000.0 / e2e_ms, 'unit': 'iters/s', 'h2d_bytes_per_step': int(h2d),
                  'd2h_bytes_per_step': 4, 'ms_per_step': e2e_ms, 'steps': k, 'trials_ms_per_step': trial_ms,
                  'what': 'StreamedSteps: per-step H2D of pinned inputs overlapping the previous step, loss read '
                          'back one step later; median of %d trials of %d steps' % (trials, k),
                  'loss_last': losses[-1]}

    def serial_step(host):
        return streamed.run([host])[0]

    for i in range(2):
        serial_step(hosts[i % 2])
    ser_trials = []
    for _ in range(trials):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for i in range(k):
            serial_step(hosts[i % 2])
        ser_trials.append((time.perf_counter() - t0) * 1000.0 / k)
    ser_ms = float(np.median(ser_trials))
    out['e2e_serial'] = {'value': 1000.0 / ser_ms, 'unit': 'iters/s', 'ms_per_step': ser_ms,
                         'trials_ms_per_step': ser_trials,
                         'what': 'one step at a time: copy inputs, replay, read the loss, wait; median of %d '
                                 'trials of %d steps' % (trials, k)}
    del streamed
    torch.cuda.empty_cache()

    # ---- the same batched graph step with FP32 storage ------------------------
    f32 = step
    if storage is not None:
        f32 = RenderAdvectStep(args.config, dev, storage_dtype=None, mode='batched')
        f32.setup_static(inputs)
        f32.capture(warmup=args.warmup)
        for _ in range(3):
            f32.replay()
        t = timed(f32.replay, min(max(5, args.steps), 50))
        out['batched_f32'] = {'value': 1000.0 / float(np.mean(t)), 'unit': 'iters/s',
                              'ms_per_step': float(np.mean(t)),
                              'what': 'the headline step with FP32 storage'}
        # accuracy of BF16 storage against the FP32 step on the same inputs
        # (the FP32 path is held to the FP64 oracle by the -m gpu tests)
        lb, gb = _grads_of(step, inputs)
        lf, gf = _grads_of(f32, inputs)
        out['bf16_accuracy'] = {'loss_rel': abs(lb - lf) / abs(lf),
                                'grad_rel_l2': dict(zip(('density', 'vel_x', 'vel_y', 'vel_z'),
                                                        [_rel(a, b) for a, b in zip(gb, gf)])),
                                'against': 'FP32 storage, same inputs (FP32 is within 1e-4 of FP64: '
                                           'tests/test_gpu_configs.py)'}
    ms_f32 = out.get('batched_f32', {}).get('ms_per_step', ms)

    # ---- plain: per-camera launches, composed advection, no graph, FP32 ------
    plain = RenderAdvectStep(args.config, dev, storage_dtype=None, mode='plain')
    plain.setup_static(inputs)
    for _ in range(2):
        plain.run_static()
    torch.cuda.synchronize()
    pt = timed(plain.run_static, min(max(3, args.steps // 3), 20))
    out['plain'] = {'value': 1000.0 / float(np.mean(pt)), 'unit': 'iters/s', 'ms_per_step': float(np.mean(pt)),
                    'what': 'FP32 storage, one raymarch launch per camera, advection from 4 SampleGridLut calls + '
                            'elementwise ops, tensor-op glue, no CUDA graph'}
    out['batched_vs_plain'] = out['plain']['ms_per_step'] / ms
    out['batched_f32_vs_plain'] = out['plain']['ms_per_step'] / ms_f32
    del plain
    torch.cuda.empty_cache()

    # ---- per-kernel timing of the dominant ops (roofline) -------------------
    out.update(kernel_roofline(step, dev, timed, storage))
    if f32 is not step:
        del f32
        torch.cuda.empty_cache()
    out['fp64_check'] = fp64_check(args, dev, timed, storage, inputs, ms)
    out['static_cameras'] = static_cameras(args, dev, timed, storage, inputs)
    out['cfg4'] = uneven_batch(dev, timed, storage)
    out['cfg2'] = other_config('cfg2', args, dev, timed)
    out['transport_chain'] = transport_chain('cfg2', dev, timed, frames=16, every=4)
    if not args.no_chain5:
        out['transport_chain_cfg5'] = transport_chain(args.config, dev, timed, frames=args.chain_frames, every=8,
                                                      storage=storage, iters=2)

    # ---- CPU baseline ------------------------------------------------------------
    if not args.no_cpu:
        try:
            from oracle import cpu_step
            out['cpu_baseline'] = cpu_step.time_step(budget_s=args.cpu_budget, workers=1, config=args.config)
        except Exception as e:  # the baseline is reported, not required
            out['cpu_baseline'] = {'error': repr(e)}
        out['fp64_subblock'] = fp64_subblock(step, dev, storage)
    return out


def fp64_subblock(step, dev, storage, size=32):
    """The headline step's raymarch (its own input: the light composition of
    the advected density, stored as the step stores it) against the FP64
    oracle on a size^3 block inside the plume: rel-L2 of the images over the
    pixels whose rays reach the block and of the density gradient inside it,
    for the adjoint of the step's image loss.  The oracle marches the
    unrounded FP32 input, so BF16 storage rounding is part of the error.
    (The oracle here is the checker, run on the host.)"""
    import numpy as np
    import torch
    from gft import fused, ops
    from oracle import subblock as SB
    t0 = time.perf_counter()
    with torch.no_grad():
        d = step.advect(step.s_d, step.s_vx, step.s_vy, step.s_vz)
        light = d * (step.shadow(d) * step.falloff_col + step.ambient)
        data = (torch.cat([light, d], dim=-1) * step.depth_step).contiguous()
    x = data.clone().requires_grad_(True)
    y = ops.raymarch_grid_transform(x, step.M, step.V, step.P, step.F, step.res, storage_dtype=storage)
    yl = y.detach().clone().requires_grad_(True)
    fused.image_loss(yl[0], step.s_t, step.bkg_host).backward()
    dy = yl.grad.contiguous()
    (gx,) = torch.autograd.grad(y, x, dy)
    D, H, W = step.shape
    block = (D // 2 - size // 2, max(0, int(0.2 * H) - size // 2), W // 2 - size // 2)
    x64 = data.double().cpu().numpy()
    y_ref, g_ref, rows, cols = SB.raymarch_block(x64, step.M, step.V, step.P, step.F, step.res,
                                                 dy.double().cpu().numpy(), block, size)
    yg = y.detach().double().cpu().numpy()
    gg = gx.detach().double().cpu().numpy()

    def rel(a, b):
        return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))

    img = max(rel(yg[0, c][rows[c], cols[c]], y_ref[0, c][rows[c], cols[c]]) for c in range(len(step.V)))
    box = (0, slice(block[0], block[0] + size), slice(block[1], block[1] + size), slice(block[2], block[2] + size))
    return {'image_rel_l2_max_over_views': img, 'density_grad_rel_l2': rel(gg[box], g_ref[box]),
            'block': {'zyx': list(block), 'size': size}, 'storage': 'bf16' if storage is not None else 'f32',
            'grad_mode': ops.get_grad_mode(), 'seconds': time.perf_counter() - t0,
            'what': 'raymarch of the step vs the FP64 oracle on the rays reaching a block in the plume; '
                    'adjoint of the step\'s image loss'}


def other_config(config, args, dev, timed):
    """The headline's graph step on another configuration, FP32 and BF16."""
    import numpy as np
    import torch
    from gft.pipeline import RenderAdvectStep
    res = {}
    inputs = None
    from gft import autotune
    for name, dt in (('f32', None), ('bf16', torch.bfloat16)):
        # this workload's own launch configuration; the headline's is restored after
        with autotune.knob_settings(autotune.knobs()):
            st = RenderAdvectStep(config, dev, storage_dtype=dt, mode='batched', autotune=not args.no_autotune)
            inputs = inputs or st.make_inputs()
            st.setup_static(inputs)
            st.capture(warmup=3)
            for _ in range(3):
                st.replay()
            t = timed(st.replay, 30)
        res[name] = {'ms_per_step': float(np.mean(t)), 'value': 1000.0 / float(np.mean(t)), 'unit': 'iters/s',
                     'knobs': st.knobs, 'candidates_ms': st.tune_log or None}
        del st
        torch.cuda.empty_cache()
    res['workload'] = workload_config(config, 'f32|bf16', args.grad_mode)['workload']
    return res


def fp64_check(args, dev, timed, storage, inputs, ms):
    """The headline step with the FP64 check step inside its graph
    (RenderAdvectStep(fp64_check=True)): the largest deviations of the FP32
    shadow transmittance (every 7th light-frustum column) and of the raymarch's
    accumulated density (every 257th ray) from their double-precision
    recomputation on the GPU, and the time the check adds to a step."""
    import numpy as np
    import torch
    from gft.pipeline import RenderAdvectStep
    try:
        st = RenderAdvectStep(args.config, dev, storage_dtype=storage, mode='batched', fp64_check=True)
        st.setup_static(inputs)
        st.capture(warmup=3)
        for _ in range(3):
            st.replay()
        t = float(np.mean(timed(st.replay, 10)))
        res = st.fp64_errors()
        res.update({'ms_per_step_with_check': t, 'check_ms': t - ms})
        del st
        torch.cuda.empty_cache()
        return res
    except Exception as e:  # reported, not required
        torch.cuda.empty_cache()
        return {'error': repr(e)[:300]}


def static_cameras(args, dev, timed, storage, inputs):
    """The same graph step with ops.set_raymarch_weight_cache(True): for a
    fixed camera rig the reference-normalised gradient's weight sums depend on
    the geometry alone, so they are computed once and reused instead of in
    every step (opt-in; the headline number recomputes them every step)."""
    import numpy as np
    import torch
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
        torch.cuda.empty_cache()


def transport_chain(config, dev, timed, frames=16, every=4, storage=None, iters=5):
    """The global-transport chain on a configuration's workload: an initial
    density and frames-1 seeded staggered velocity fields, MacCormack advection
    through all frames, every frame rendered by the views and compared with
    its target, gradients to the initial density and all velocities, the
    adjoint recomputing each segment of ``every`` frames from its stored first
    density (gft.chain.TransportChain).  One CUDA graph per iteration when
    capture succeeds, else eager.  Reports the peak device memory."""
    import numpy as np
    import torch
    from gft import synthetic as syn
    from gft.chain import TransportChain
    from gft.pipeline import RenderAdvectStep
    try:
        step = RenderAdvectStep(config, dev, storage_dtype=storage, mode='batched')
        shape = step.shape
        torch.cuda.empty_cache()
        torch.cuda.reset_peak_memory_stats(dev)
        base = torch.cuda.memory_allocated(dev)
        d0 = torch.from_numpy(syn.plume_density(shape, 3000)).to(dev).requires_grad_(True)
        vels = []
        for t in range(frames - 1):
            vx, vy, vz = syn.curl_velocity_device(shape, 3100 + t, dev)
            vels.append(tuple(v.requires_grad_(True) for v in (vx, vy, vz)))
        with torch.no_grad():
            targets = [step.render(syn.plume_density_device(shape, 3200 + t, dev, t))[..., :3].contiguous()
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
        ms = float(np.median(timed(run, iters, flush_l2=False)))
        peak = torch.cuda.max_memory_allocated(dev) - base
        res = {'workload': '%d frames, density %s (%s storage), %d views, MacCormack chain, fwd+bwd to the initial '
                           'density and all velocities, checkpoint every %d frames'
                           % (frames, 'x'.join(map(str, shape)), 'bf16' if storage is not None else 'f32',
                              len(step.cams), every),
               'ms_per_iteration': ms, 'iters_per_s': 1000.0 / ms, 'cuda_graph': graph is not None,
               'frames_per_s': frames * 1000.0 / ms, 'peak_hbm_bytes': int(peak),
               **({'capture_error': why} if why else {})}
        del graph, chain, vels, targets, d0, params
        torch.cuda.empty_cache()
        return res
    except Exception as e:  # reported, not required
        torch.cuda.empty_cache()
        return {'error': repr(e)[:300]}


def uneven_batch(dev, timed, storage=None, frames=64, views=8):
    """cfg4: 64 frames of 96x170x96 density, each rendered by 1 fixed view
    (256^2) + 8 seeded upper-hemisphere views of 64-256 px square (cameras
    narrowed to the grid's bounding box), 128 samples, Beer-Lambert + spot
    light with shadow, L2 image loss; all 576 renders and their adjoints plus
    the batched shadow pass in one CUDA graph (gft.pipeline.UnevenBatchStep).
    Beside it, the raymarch alone (forward + reference-normalised adjoint) of
    the 576 views: views bound to their frame in launches of 16
    (raymarch_grid_transform_views) against one call per view (the reference's
    structure: one call per camera image size)."""
    import numpy as np
    import torch
    from gft import ops
    from gft.pipeline import UnevenBatchStep
    try:
        st = UnevenBatchStep(frames=frames, views=views, device=dev, storage_dtype=storage)
        inputs = st.make_inputs(seed=4000)
        st.setup_static(inputs)
        torch.cuda.reset_peak_memory_stats(dev)
        from gft import autotune
        tune_log = {}
        with autotune.knob_settings(autotune.knobs()):  # this workload's own knobs, the headline's restored after
            st.capture(warmup=3, autotune=True, tune_log=tune_log)
            for _ in range(2):
                st.replay()
            t = float(np.median(timed(st.replay, 5)))
        nviews = len(st.shapes)
        res = {'workload': '%d frames x (1 + %d) views of 64-256 px, density %s, %d samples, shadow + BEER_LAMBERT, '
                           'fwd+bwd to every frame density, one CUDA graph' % (frames, views,
                                                                               'x'.join(map(str, st.shape)),
                                                                               st.shapes[0][0]),
               'ms_per_iteration': t, 'iters_per_s': 1000.0 / t, 'renders_per_s': nviews * 1000.0 / t,
               'views': nviews, 'pixels': st.pixels, 'peak_hbm_bytes': int(torch.cuda.max_memory_allocated(dev)),
               'autotune': {'knobs': getattr(st, 'knobs', None), 'candidates_ms': tune_log}}
        # raymarch alone: one views op vs one call per view
        with torch.no_grad():
            x = (torch.from_numpy(inputs['d']).to(dev).repeat(1, 1, 1, 1, 4) * 0.02).contiguous()
        cb, shapes = st.camera_batch, st.shapes
        ref = ops.GRAD['REFERENCE']
        y = ops._raymarch_views_fwd(x, st.M, st.V, st.P, st.F, cb, shapes, 1, 0, 0)
        dy = torch.randn_like(y) * 1e-3

        def views_op():
            yy = ops._raymarch_views_fwd(x, st.M, st.V, st.P, st.F, cb, shapes, 1, 0, 0)
            ops._raymarch_views_bwd(x, yy, dy, st.M, st.V, st.P, st.F, cb, shapes, 1, 0, 0, ref)

        offs = np.cumsum([0] + [h * w for _, h, w in shapes])
        dys = [dy[offs[c]:offs[c + 1]].reshape(1, 1, shapes[c][1], shapes[c][2], 4).contiguous()
               for c in range(len(shapes))]

        def per_view():
            for c, s in enumerate(shapes):
                b = cb[c]
                xb = x[b:b + 1]
                yc = ops._raymarch_fwd(xb, st.M[b:b + 1], st.V[c:c + 1], st.P[c:c + 1], st.F[c:c + 1], s, 1, 0, 0,
                                       True)
                ops._raymarch_bwd(xb, yc, dys[c], st.M[b:b + 1], st.V[c:c + 1], st.P[c:c + 1], st.F[c:c + 1], s, 1,
                                  0, 0, True, ref)

        views_op(), per_view()
        tv = float(np.median(timed(views_op, 3)))
        tp = float(np.median(timed(per_view, 3)))
        res['raymarch_only'] = {'views_op_ms': tv, 'per_view_calls_ms': tp, 'speedup': tp / tv}
        del st, x, y, dy, dys
        torch.cuda.empty_cache()
        return res
    except Exception as e:  # reported, not required
        torch.cuda.empty_cache()
        return {'error': repr(e)[:300]}


def kernel_roofline(step, dev, timed, storage=None):
    """Times the render kernels alone with CUDA events on their stream (L2
    flushed before each launch).  The dominant kernel is the raymarch
    adjoint's scatter pass (k_raymarch_scatter, one launch for all views) as
    the step runs it: reading the samples the forward stored, with its
    per-camera weight sums precomputed (GFT_GRAD_WEIGHTS_READY: a gradient
    memset plus the scatter launch), accumulating the two projections of the
    4-channel gradient that the light composition's adjoint reads.
    ``alg_bytes`` is the render-backward formula (N*4*s + 2*P*4*4 + 2*N*4*4:
    the grid read once, image and adjoint, 4-channel gradient
    read-modify-write); ``impl_bytes`` is what this implementation moves (the
    stored samples it reads instead of re-gathering, image and adjoint, the
    per-camera reciprocal weight sums, the 2-channel gradient
    read-modify-write).  The 4-channel scatter is timed beside it."""
    import numpy as np
    import torch
    from gft import fused, ops
    peak, src = _peaks()
    with torch.no_grad():
        d = step.advect(step.s_d, step.s_vx, step.s_vy, step.s_vz)
        light = d * (step.shadow(d) * step.falloff_col + step.ambient)
        # the raymarch input in the brick layout the step uses
        data = ops.to_bricks((torch.cat([light, d], dim=-1) * step.depth_step).contiguous())
        if storage is not None:
            data = data.to(storage)
        del d, light
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
    proj = fused.compose_projection(step.light[1], step.ambient, step.depth_step)
    scatter = lambda: ops._raymarch_bwd(data, y, dy, step.M, step.V, step.P, step.F, step.res, 1, 0, 0, True,
                                        ops.GRAD['REFERENCE'], weights=ws, grid=grid, samples=smp, projection=proj)
    scatter4 = lambda: ops._raymarch_bwd(data, y, dy, step.M, step.V, step.P, step.F, step.res, 1, 0, 0, True,
                                         ops.GRAD['REFERENCE'], weights=ws, grid=grid, samples=smp)
    for _ in range(2):
        fwd(), bwd('REFERENCE'), bwd('EXACT'), weights(), scatter(), scatter4()
    tf = float(np.median(timed(fwd, 7)))
    tb_ref = float(np.median(timed(lambda: bwd('REFERENCE'), 7)))
    tb_ex = float(np.median(timed(lambda: bwd('EXACT'), 7)))
    tw = float(np.median(timed(weights, 7)))
    ts = float(np.median(timed(scatter, 7)))
    ts4 = float(np.median(timed(scatter4, 7)))
    nvox = int(np.prod(step.shape))
    s = 2 if storage is not None else 4
    C = 4
    pix = V * H * W
    samples = pix * D
    n_stored = ops.stored_sample_count(smp, shape5, V, step.res)
    stored = n_stored * C * 4
    alg_fwd = nvox * C * s + pix * C * 4
    alg_bwd = nvox * C * s + 2 * pix * C * 4 + 2 * nvox * C * 4
    impl_scatter = stored + 2 * pix * C * 4 + V * nvox * 4 + 2 * nvox * 2 * 4
    impl_scatter4 = stored + 2 * pix * C * 4 + V * nvox * 4 + 2 * nvox * C * 4
    kern = {
        'raymarch_fwd': {'ms': tf, 'alg_bytes': alg_fwd, 'GBps': alg_fwd / tf / 1e6,
                         'impl_bytes': alg_fwd + stored, 'samples_per_s': samples / tf * 1e3},
        'raymarch_bwd_scatter': {'ms': ts, 'alg_bytes': alg_bwd, 'GBps': alg_bwd / ts / 1e6,
                                 'impl_bytes': impl_scatter, 'samples_per_s': samples / ts * 1e3,
                                 'what': 'reference normalisation, weights ready, stored samples, gradient '
                                         'projected onto the light composition\'s two sums (as the step)'},
        'raymarch_bwd_scatter_4ch': {'ms': ts4, 'alg_bytes': alg_bwd, 'GBps': alg_bwd / ts4 / 1e6,
                                     'impl_bytes': impl_scatter4, 'samples_per_s': samples / ts4 * 1e3,
                                     'what': 'the same pass accumulating the 4-channel gradient'},
        'raymarch_samples_stored': n_stored,
        'raymarch_samples_stored_bytes': stored,
        'raymarch_bwd_weights': {'ms': tw, 'impl_bytes': 2 * V * nvox * 4, 'samples_per_s': samples / tw * 1e3,
                                 'what': 'geometry-only pass of the reference normalisation (per-camera weight sums)'},
        'raymarch_bwd_reference': {'ms': tb_ref, 'alg_bytes': alg_bwd, 'GBps': alg_bwd / tb_ref / 1e6,
                                   'what': 'whole op: weights + inversion + scatter'},
        'raymarch_bwd_exact': {'ms': tb_ex, 'alg_bytes': alg_bwd, 'GBps': alg_bwd / tb_ex / 1e6},
        'grad_mode': mode,
    }
    traffic = SCATTER_TRAFFIC.get((step.config_name, 'bf16' if storage is not None else 'f32'))
    del smp, ws, data, y, dy
    torch.cuda.empty_cache()
    return {'roofline': {'kernel': 'k_raymarch_scatter (raymarch adjoint scatter pass, %d views)' % V,
                         'bound': 'hbm', 'achieved': kern['raymarch_bwd_scatter']['GBps'], 'peak': peak,
                         'unit': 'GB/s', 'frac': kern['raymarch_bwd_scatter']['GBps'] / peak, 'peak_source': src,
                         'traffic': traffic, 'alg_bytes': alg_bwd, 'impl_bytes': impl_scatter,
                         'traffic_source': ('ncu dram__bytes_read.sum + dram__bytes_write.sum, one launch'
                                            if traffic else None),
                         'note': 'alg_bytes = the render-backward formula; the pass is bound by the L1/L2 path of '
                                 'its merged trilinear gradient reductions and by latency, not by HBM; it '
                                 'accumulates two projected channels (impl_bytes), as the step does'},
            'kernels': kern}


def kernel_only(args):
    """Runs one op of the workload ``args.repeat`` times without a graph
    (for ncu captures of a single kernel)."""
    import torch
    from gft import ops
    from gft.pipeline import RenderAdvectStep
    dev = torch.device('cuda', 0)
    ops.set_grad_mode(args.grad_mode)
    storage = _storage_dtype(args.storage)
    step = RenderAdvectStep(args.config, dev, mode='batched', storage_dtype=storage)
    inputs = step.make_inputs()
    step.setup_static(inputs)
    with torch.no_grad():
        d = step.advect(step.s_d, step.s_vx, step.s_vy, step.s_vz)
        light = d * (step.shadow(d) * step.falloff_col + step.ambient)
        data = ops.to_bricks((torch.cat([light, d], dim=-1) * step.depth_step).contiguous())
        if storage is not None:
            data = data.to(storage)
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
    if args.kernel_only in ('raymarch_scatter', 'raymarch_scatter_projected'):
        from gft import fused
        ws = ops._raymarch_weights((1,) + tuple(grid) + (4,), data.device, step.M, step.V, step.P, step.F, step.res,
                                   0, True)
        proj = (fused.compose_projection(step.light[1], step.ambient, step.depth_step)
                if args.kernel_only == 'raymarch_scatter_projected' else None)
        fns[args.kernel_only] = lambda: ops._raymarch_bwd(data, y, dy, step.M, step.V, step.P, step.F, step.res, 1,
                                                          0, 0, True, ops.GRAD['REFERENCE'], weights=ws,
                                                          grid=grid, samples=smp, projection=proj)
    fn = fns[args.kernel_only]
    for _ in range(args.repeat):
        fn()
    torch.cuda.synchronize()
    print(json.dumps({'kernel_only': args.kernel_only, 'repeat': args.repeat, 'ok': True}))


# ------------------------------------------------------------ reference arm
def bench_reference(args):
    """The reference's own implementation of the path is CUDA-only
    TensorFlow ops; its CPU stand-in is the FP64 NumPy port in oracle/, run
    as whole iterations of the same workload on all host cores
    (oracle/cpu_step.py FullStep).  A whole iteration of the default workload
    takes on the order of a minute, so the arm runs as many as fit in
    ``--ref-budget`` seconds (at least one) and reports the steps it ran."""
    ws, rank, _ = _ddp()
    if rank != 0:
        return
    from oracle import cpu_step
    workers = os.cpu_count() or 1
    t0 = time.perf_counter()
    res = cpu_step.time_full_steps(args.config, workers=workers, budget_s=args.ref_budget, max_steps=args.steps)
    wall = time.perf_counter() - t0
    times = res['seconds_per_step']
    sec = sum(times) / len(times)
    v = 1.0 / sec
    line = {'impl': 'reference', 'metric': METRIC, 'value': v, 'unit': 'iters/s', 'n_gpus': ws,
            'steps': len(times), 'warmup': 0, 'steps_requested': args.steps, 'warmup_requested': args.warmup,
            'ms_per_step': 1000.0 * sec, 'higher_is_better': True, 'scaling': 'weak', 'vs_baseline': None,
            'dtype': 'f64', 'data': 'synthetic (seeded plume + curl-noise velocity; ScalarFlow absent)',
            'config': workload_config(args.config, args.storage, args.grad_mode),
            'cpu_baseline': {'value': v, 'unit': 'iters/s', 'cores': res['workers'], 'kind': 'port',
                             'sample': 'whole iterations (every voxel, ray and frustum cell), FP64 NumPy port of '
                                       'the reference ops, %d spawned workers sharing memory; per-stage seconds '
                                       'per step: %s' % (res['workers'], json.dumps(
                                           {k: round(x, 2) for k, x in res['stages_s'].items()})),
                             'seconds_per_step': times},
            'e2e': {'value': v, 'unit': 'iters/s', 'h2d_bytes_per_step': 0, 'd2h_bytes_per_step': 0},
            'wall_s': wall, 'loss': res['loss'][-1]}
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument('--gpus', type=int, default=1)
    ap.add_argument('--steps', type=int, default=20)
    ap.add_argument('--warmup', type=int, default=3)
    ap.add_argument('--impl', default='ours', choices=['ours', 'reference'])
    ap.add_argument('--config', default=DEFAULT_CONFIG)
    ap.add_argument('--storage', default=DEFAULT_STORAGE, choices=['f32', 'bf16'])
    ap.add_argument('--grad-mode', default='REFERENCE', choices=['REFERENCE', 'EXACT'])
    ap.add_argument('--quick', action='store_true', help='only the timed graph replays')
    ap.add_argument('--no-cpu', action='store_true')
    ap.add_argument('--no-chain5', action='store_true', help='skip the long transport chain on the headline grid')
    ap.add_argument('--no-autotune', action='store_true', help='default launch configuration (no tuning)')
    ap.add_argument('--knobs', default=None, metavar='NAME=V,...',
                    help='fixed launch-configuration knobs instead of tuning (gft.autotune.KNOBS names)')
    ap.add_argument('--chain-frames', type=int, default=120)
    ap.add_argument('--cpu-budget', type=float, default=20.0)
    ap.add_argument('--ref-budget', type=float, default=240.0,
                    help='reference arm: seconds of whole FP64 iterations to run (at least one)')
    ap.add_argument('--save-clocks', default=None, metavar='CSV', help='write every clock sample to this file')
    ap.add_argument('--kernel-only', default=None,
                    choices=['raymarch_fwd', 'raymarch_bwd', 'raymarch_weights', 'raymarch_scatter',
                             'raymarch_scatter_projected', 'advect_fwd', 'advect_bwd', 'shadow_fwd'],
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
