"""bench.py's reference arm runs on the host cores alone (whole iterations of
the FP64 oracle port of the step): one JSON line with the metric, unit, value
and config of the GPU arm's workload, the number of whole steps it ran, its
cpu_baseline record and an end-to-end record without transfers."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_arm_prints_one_json_line():
    out = subprocess.run([sys.executable, 'bench.py', '--impl', 'reference', '--config', 'cfg1', '--ref-budget', '1',
                          '--steps', '2', '--warmup', '3'], cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert out.returncode == 0, out.stderr[-2000:]
    lines = [l for l in out.stdout.splitlines() if l.strip()]
    assert len(lines) == 1
    line = json.loads(lines[0])
    assert line['impl'] == 'reference'
    assert line['metric'] == 'fwd+bwd render+advect iters/s' and line['unit'] == 'iters/s'
    assert line['value'] > 0 and line['higher_is_better'] is True and line['n_gpus'] == 1
    sys.path.insert(0, ROOT)
    import bench
    assert line['config'] == bench.workload_config('cfg1', bench.DEFAULT_STORAGE, 'REFERENCE')
    assert 1 <= line['steps'] <= 2 and len(line['cpu_baseline']['seconds_per_step']) == line['steps']
    assert abs(line['ms_per_step'] - 1000.0 * sum(line['cpu_baseline']['seconds_per_step']) / line['steps']) < 1e-6
    assert line['wall_s'] >= line['steps'] * line['ms_per_step'] / 1000.0
    cb = line['cpu_baseline']
    assert cb['kind'] == 'port' and cb['cores'] >= 1 and cb['sample'] and cb['value'] == line['value']
    assert line['e2e'] == {'value': line['value'], 'unit': 'iters/s', 'h2d_bytes_per_step': 0,
                           'd2h_bytes_per_step': 0}


def test_reference_arm_other_ranks_exit_without_work():
    """Under torchrun with N > 1 only rank 0 times and prints; rank 1 exits 0
    and prints nothing."""
    env = dict(os.environ, RANK='1', LOCAL_RANK='1', WORLD_SIZE='2')
    out = subprocess.run([sys.executable, 'bench.py', '--impl', 'reference', '--gpus', '2', '--cpu-budget', '1',
                          '--steps', '1', '--warmup', '3'], cwd=ROOT, env=env, capture_output=True, text=True,
                         timeout=300)
    assert out.returncode == 0, out.stderr[-2000:]
    assert out.stdout.strip() == ''
