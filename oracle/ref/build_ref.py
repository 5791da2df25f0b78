"""Recipe: build the reference's own CUDA kernels as a test oracle.

ORACLE / TEST INFRASTRUCTURE ONLY.  Nothing here is part of the product.

Step 1 (needs the reference checkout at /root/reference, development container
only): stage the reference's CUDA sources -- phitest/render/cuda/src/*.cu.cc,
their headers, the cuda-samples helper headers and the vendored GLM headers --
unchanged into oracle/_ref/src/, next to a two-header TensorFlow stub written
by this recipe (the kernels only need ``Eigen::GpuDevice``).  oracle/_ref/ is
git-ignored: no reference source enters the repository history.

Step 2 (any machine with nvcc, including the GPU machine, which receives the staged
tree): compile each reference library (resample_grid, raymarch_grid,
reduce_blend) together with the matching C harness of oracle/ref/ into
oracle/_ref/libref_<name>.so (sm_103a).  The TF op glue (.cc files) is not
compiled: the harness calls the reference's kernel launchers directly.

    python oracle/ref/build_ref.py [--stage-only] [--force]
"""
import argparse
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE = os.path.dirname(HERE)
REF_OUT = os.path.join(ORACLE, '_ref')
SRC = os.path.join(REF_OUT, 'src')
REFERENCE = '/root/reference'
REF_CUDA = os.path.join(REFERENCE, 'phitest', 'render', 'cuda', 'src')
REF_GLM = os.path.join(REFERENCE, 'lib', 'glm')

LIBS = {
    'raymarch': ('raymarch_grid.cu.cc', 'harness_raymarch.cu'),
    'resample': ('resample_grid.cu.cc', 'harness_resample.cu'),
    'blend': ('reduce_blend.cu.cc', 'harness_blend.cu'),
}

TF_STUB = '''// Stand-in for the TensorFlow header the reference kernels include: they only
// need Eigen::GpuDevice::stream() (written by oracle/ref/build_ref.py).
#pragma once
#include <cuda_runtime.h>
namespace Eigen {
struct GpuDevice {
    cudaStream_t stream() const { return 0; }
};
}  // namespace Eigen
'''


def reference_present():
    return os.path.isdir(REF_CUDA)


def stage(force=False):
    """Copies the reference sources into oracle/_ref/src (unchanged)."""
    if not os.path.isdir(REF_CUDA):
        return False
    marker = os.path.join(SRC, '.staged')
    if os.path.exists(marker) and not force:
        return True
    if os.path.isdir(SRC):
        shutil.rmtree(SRC)
    os.makedirs(SRC)
    for f in os.listdir(REF_CUDA):
        p = os.path.join(REF_CUDA, f)
        if os.path.isfile(p) and (f.endswith(('.hpp', '.inl', '.h')) or f.endswith('.cu.cc')):
            shutil.copy2(p, os.path.join(SRC, f))
    shutil.copytree(os.path.join(REF_CUDA, 'cuda-samples'), os.path.join(SRC, 'cuda-samples'))
    shutil.copytree(REF_GLM, os.path.join(SRC, 'lib', 'glm'))
    for sub in ('tensorflow/core/framework/tensor_types.h', 'tensorflow/core/platform/types.h'):
        p = os.path.join(SRC, sub)
        os.makedirs(os.path.dirname(p), exist_ok=True)
        with open(p, 'w') as f:
            f.write(TF_STUB)
    open(marker, 'w').close()
    return True


def _nvcc():
    for c in (os.environ.get('NVCC'), shutil.which('nvcc'), '/usr/local/cuda/bin/nvcc'):
        if c and os.path.exists(c):
            return c
    return None


def _build_one(name, force):
    ref_src, harness = LIBS[name]
    out = os.path.join(REF_OUT, 'libref_%s.so' % name)
    srcs = [os.path.join(SRC, ref_src), os.path.join(HERE, harness)]
    if not force and os.path.exists(out) and os.path.getmtime(out) >= max(os.path.getmtime(s) for s in srcs):
        return out, None
    cmd = [_nvcc(), '-gencode', 'arch=compute_103a,code=sm_103a', '-O2', '-std=c++17', '-shared',
           '-Xcompiler', '-fPIC', '-DGOOGLE_CUDA=1', '-w', '-I', SRC, '-I', os.path.join(SRC, 'lib', 'glm'),
           '-x', 'cu'] + srcs + ['-o', out]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        return out, 'build of %s failed:\n%s\n%s' % (name, ' '.join(cmd), r.stderr[-4000:])
    return out, None


def build(force=False, quiet=False):
    """Stages (when the reference is present) and builds the three libraries
    (when staged sources and nvcc are present).  Returns the built paths."""
    stage(force)
    if not os.path.exists(os.path.join(SRC, '.staged')) or _nvcc() is None:
        return []
    with cf.ThreadPoolExecutor(3) as ex:
        res = list(ex.map(lambda n: _build_one(n, force), LIBS))
    errs = [e for _, e in res if e]
    if errs:
        raise RuntimeError('\n'.join(errs))
    if not quiet:
        for o, _ in res:
            print('built', o)
    return [o for o, _ in res]


if __name__ == '__main__':
    ap = argparse.ArgumentParser()
    ap.add_argument('--stage-only', action='store_true')
    ap.add_argument('--force', action='store_true')
    a = ap.parse_args()
    if a.stage_only:
        print('staged' if stage(a.force) else 'reference not present')
        sys.exit(0)
    build(a.force)
