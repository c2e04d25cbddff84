"""Builds libpmx.so (the CUDA kernels and their C ABI) in-tree for sm_103a.

Each ``csrc/*.cu`` translation unit is compiled in parallel with nvcc, then
linked against cuFFT into ``pmwd_gb300/libpmx.so``.  No cmake, no torch
extension machinery: the library has a plain C ABI (``include/pmx.h``).
"""

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, 'csrc')
OUT_DIR = os.path.join(HERE, '_build')
LIB = os.path.join(HERE, 'libpmx.so')

ARCH = ['-gencode', 'arch=compute_103a,code=sm_103a']
NVCC_FLAGS = ['-O3', '-lineinfo', '-std=c++17', '-Xcompiler', '-fPIC', '-Xcompiler', '-O2',
              '--expt-relaxed-constexpr']


def nvcc_path():
    for cand in (os.environ.get('NVCC'),
                 os.path.join(os.environ.get('CUDA_HOME', '/usr/local/cuda'), 'bin', 'nvcc'),
                 shutil.which('nvcc')):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError('nvcc not found (set CUDA_HOME or NVCC)')


def sources():
    return sorted(os.path.join(SRC, f) for f in os.listdir(SRC) if f.endswith('.cu'))


def _run(cmd, verbose):
    if verbose:
        print(' '.join(cmd), flush=True)
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError(f'command failed ({r.returncode}): {" ".join(cmd)}\n{r.stdout}')
    if verbose and r.stdout.strip():
        print(r.stdout, flush=True)
    return r.stdout


def build(verbose=False, extra_flags=()):
    """Compile and link libpmx.so; returns its path."""
    nvcc = nvcc_path()
    os.makedirs(OUT_DIR, exist_ok=True)
    srcs = sources()
    objs = [os.path.join(OUT_DIR, os.path.basename(s)[:-3] + '.o') for s in srcs]
    cmds = [[nvcc, *ARCH, *NVCC_FLAGS, *extra_flags, '-c', s, '-o', o]
            for s, o in zip(srcs, objs)]
    with ThreadPoolExecutor(max_workers=min(8, len(cmds))) as ex:
        list(ex.map(lambda c: _run(c, verbose), cmds))
    tmp = LIB + '.tmp'
    _run([nvcc, *ARCH, '-shared', '-o', tmp, *objs, '-lcufft', '-lcudart'], verbose)
    os.replace(tmp, LIB)
    return LIB


if __name__ == '__main__':
    print(build(verbose='-v' in sys.argv))
