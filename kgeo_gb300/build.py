"""Build the kgeo_gb300 CUDA library (libkgeo_gb300.so) for sm_103a with nvcc.

The library is built in-tree: objects go to kgeo_gb300/_build/, the shared library
to kgeo_gb300/libkgeo_gb300.so. Translation units compile in parallel.
"""
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, 'csrc')
BUILD = os.path.join(PKG, '_build')
LIB = os.path.join(PKG, 'libkgeo_gb300.so')

ARCH = ['-gencode', 'arch=compute_103a,code=sm_103a']
COMMON = ['-O3', '-lineinfo', '-std=c++17', '-Xcompiler', '-fPIC', '-I', os.path.join(ROOT, 'include')]

# (source, extra flags). The per-ray setup keeps FMA contraction off so its roundings
# follow numpy's one-operation-at-a-time arithmetic.
UNITS = [
    ('kg_setup.cu', ['-fmad=false']),
    ('kg_image.cu', ['-fmad=false']),
    ('kg_image_adj.cu', ['-fmad=false']),
    ('kg_samples.cu', []),
    ('kg_abi.cu', []),
    ('kg_peak.cu', []),
    ('kg_noalloc.cu', []),
    ('kg_batch.cu', []),
    ('kg_curves.cu', ['-fmad=false']),
    ('kg_jet.cu', ['-fmad=false']),
    ('kg_jetimg.cu', ['-fmad=false']),
]


# Per-thread stack every kernel must fit: CUDA's default cudaLimitStackSize is 1024 bytes and the
# library never raises it. A kernel whose call chain (ptxas' "cumulative stack size") grows past
# it faults with an illegal address at launch, so the build refuses it, with a margin.
STACK_BUDGET = 960


def check_resources(log):
    """Parse ptxas -v output: {kernel: (registers, cumulative stack bytes, spill store bytes)}."""
    import re
    out, entry, spill = {}, None, 0
    for line in log.splitlines():
        m = re.search(r"Compiling entry function '(\S+)'", line)
        if m:
            entry, spill = m.group(1), 0
            continue
        m = re.search(r'(\d+) bytes spill stores', line)
        if m and entry:
            spill = int(m.group(1))
            continue
        m = re.search(r'Used (\d+) registers', line)
        if m and entry:
            st = re.search(r'(\d+) bytes cumulative stack size', line)
            out[entry] = (int(m.group(1)), int(st.group(1)) if st else 0, spill)
            entry = None
    return out


def nvcc():
    for cand in (shutil.which('nvcc'), '/usr/local/cuda/bin/nvcc'):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError('nvcc not found: the kgeo_gb300 CUDA library cannot be built')


def _compile(args):
    src, extra, verbose = args
    obj = os.path.join(BUILD, src.replace('.cu', '.o'))
    cmd = [nvcc(), '-Xptxas=-v', *ARCH, *COMMON, *extra, '-c', os.path.join(CSRC, src), '-o', obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError('nvcc failed for %s:\n%s\n%s' % (src, ' '.join(cmd), r.stderr))
    if 'cannot be statically determined' in r.stderr:
        raise RuntimeError('%s: a kernel whose stack is not known at compile time (recursion or an '
                           'indirect call); the library keeps every stack static' % src)
    over = {k: v for k, v in check_resources(r.stderr).items() if v[1] > STACK_BUDGET}
    if over:
        raise RuntimeError('%s: per-thread stack above %d bytes (CUDA default limit 1024): %s'
                           % (src, STACK_BUDGET, over))
    return obj, r.stderr


def build(verbose=False, force=False):
    """Compile every translation unit and link libkgeo_gb300.so. Returns the library path."""
    os.makedirs(BUILD, exist_ok=True)
    srcs = [os.path.join(CSRC, f) for f in os.listdir(CSRC)] + [os.path.join(ROOT, 'include', 'kgeo_gb300.h')]
    newest = max(os.path.getmtime(p) for p in srcs)
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= newest and os.path.getmtime(LIB) >= os.path.getmtime(__file__):
        return LIB
    with ThreadPoolExecutor(max_workers=len(UNITS)) as ex:
        results = list(ex.map(_compile, [(s, e, verbose) for s, e in UNITS]))
    with open(os.path.join(BUILD, 'ptxas.log'), 'w') as f:
        for obj, log in results:
            f.write(log)
    if verbose:
        for obj, log in results:
            sys.stderr.write(log)
    tmp = LIB + '.tmp'
    cmd = [nvcc(), *ARCH, '-shared', '-o', tmp] + [o for o, _ in results]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError('link failed:\n%s\n%s' % (' '.join(cmd), r.stderr))
    os.replace(tmp, LIB)
    return LIB


if __name__ == '__main__':
    print(build(verbose='-v' in sys.argv, force='-f' in sys.argv))
