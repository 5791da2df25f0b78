"""Builds libgft.so (the CUDA kernels + C ABI) for sm_103a with nvcc.

Translation units compile in parallel into ``_build/`` and link into
``gft/libgft.so`` next to the Python bindings.  Rebuilds only what changed.

    python build.py [--force] [--jobs N]
"""
import argparse
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, 'csrc')
OBJ = os.path.join(HERE, '_build')
OUT = os.path.join(HERE, 'gft', 'libgft.so')
INCLUDE = os.path.join(os.path.dirname(HERE), 'include')

ARCH = ['-gencode', 'arch=compute_103a,code=sm_103a']
CFLAGS = ['-O3', '-lineinfo', '-std=c++17', '--expt-relaxed-constexpr', '-Xcompiler', '-fPIC',
          '-Xcompiler', '-fvisibility=hidden', '-I', CSRC, '-I', INCLUDE]


def nvcc():
    for cand in (os.environ.get('NVCC'), shutil.which('nvcc'), '/usr/local/cuda/bin/nvcc'):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError('nvcc not found')


def _sources():
    return sorted(f for f in os.listdir(CSRC) if f.endswith('.cu'))


def _headers_mtime():
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(('.cuh', '.h'))]
    hs.append(os.path.join(INCLUDE, 'gft.h'))
    return max(os.path.getmtime(h) for h in hs)


def _compile(src, force, hdr_mtime, extra):
    obj = os.path.join(OBJ, src[:-3] + '.o')
    s = os.path.join(CSRC, src)
    if (not force and os.path.exists(obj) and os.path.getmtime(obj) >= max(os.path.getmtime(s), hdr_mtime)):
        return obj, None
    cmd = [nvcc()] + ARCH + CFLAGS + extra + ['-c', s, '-o', obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        return obj, 'compile failed: %s\n%s\n%s' % (' '.join(cmd), r.stdout, r.stderr)
    return obj, None


def build(force=False, jobs=None, verbose=False, extra=()):
    os.makedirs(OBJ, exist_ok=True)
    hdr = _headers_mtime()
    srcs = _sources()
    jobs = jobs or min(len(srcs), os.cpu_count() or 4)
    with cf.ThreadPoolExecutor(jobs) as ex:
        results = list(ex.map(lambda s: _compile(s, force, hdr, list(extra)), srcs))
    errs = [e for _, e in results if e]
    if errs:
        raise RuntimeError('\n'.join(errs))
    objs = [o for o, _ in results]
    if force or not os.path.exists(OUT) or os.path.getmtime(OUT) < max(os.path.getmtime(o) for o in objs):
        cmd = [nvcc()] + ARCH + ['-shared', '-o', OUT] + objs
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError('link failed: %s\n%s\n%s' % (' '.join(cmd), r.stdout, r.stderr))
    if verbose:
        print('built', OUT)
    return OUT


if __name__ == '__main__':
    ap = argparse.ArgumentParser()
    ap.add_argument('--force', action='store_true')
    ap.add_argument('--jobs', type=int, default=None)
    ap.add_argument('--ptxas-v', action='store_true', help='print register/smem usage')
    a = ap.parse_args()
    try:
        build(a.force or a.ptxas_v, a.jobs, verbose=True, extra=['-Xptxas', '-v'] if a.ptxas_v else ())
    except RuntimeError as e:
        print(e, file=sys.stderr)
        sys.exit(1)
