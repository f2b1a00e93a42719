"""Builds libntgb300.so (the sm_103a kernels behind include/nt_gb300.h) in-tree.

Every .cu file under csrc/ is compiled to an object in parallel with
``nvcc -gencode arch=compute_103a,code=sm_103a -lineinfo`` and linked into one
shared library next to this file. Objects are rebuilt only when a source or a
header is newer. No torch headers are involved: the library is a plain C ABI.
"""
from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, 'csrc')
INCLUDE = os.path.join(ROOT, 'include')
BUILD = os.path.join(HERE, '_build')
LIB = os.path.join(HERE, 'libntgb300.so')

ARCH = ['-gencode', 'arch=compute_103a,code=sm_103a']
NVCC_FLAGS = ['-O3', '-std=c++17', '-lineinfo', '--expt-relaxed-constexpr',
              '-Xcompiler', '-fPIC', '-Xptxas', '-warn-spills']


def nvcc() -> str:
    for cand in (os.environ.get('NVCC'), shutil.which('nvcc'), '/usr/local/cuda/bin/nvcc'):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError('nvcc not found: the nt_gb300 CUDA library cannot be built')


def _newest(paths) -> float:
    return max((os.path.getmtime(p) for p in paths), default=0.0)


def build(verbose: bool = False, force: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    sources = sorted(glob.glob(os.path.join(CSRC, '*.cu')))
    headers = glob.glob(os.path.join(CSRC, '*.cuh')) + glob.glob(os.path.join(INCLUDE, '*.h'))
    hdr_time = _newest(headers)
    exe = nvcc()

    def compile_one(src: str) -> str:
        obj = os.path.join(BUILD, os.path.basename(src)[:-3] + '.o')
        if (not force and os.path.exists(obj)
                and os.path.getmtime(obj) >= max(os.path.getmtime(src), hdr_time)):
            return obj
        cmd = [exe, *ARCH, *NVCC_FLAGS, '-I', INCLUDE, '-I', CSRC, '-c', src, '-o', obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if verbose or r.returncode != 0:
            sys.stderr.write(r.stdout + r.stderr)
        if r.returncode != 0:
            raise RuntimeError(f'nvcc failed on {os.path.basename(src)}')
        return obj

    with cf.ThreadPoolExecutor(max_workers=min(8, len(sources))) as ex:
        objs = list(ex.map(compile_one, sources))
    if force or not os.path.exists(LIB) or os.path.getmtime(LIB) < _newest(objs):
        cmd = [exe, *ARCH, '-shared', '-o', LIB, *objs, '-lcudart_static', '-ldl', '-lrt',
               '-lpthread']
        r = subprocess.run(cmd, capture_output=True, text=True)
        if verbose or r.returncode != 0:
            sys.stderr.write(r.stdout + r.stderr)
        if r.returncode != 0:
            raise RuntimeError('linking libntgb300.so failed')
    return LIB


if __name__ == '__main__':
    print(build(verbose='-v' in sys.argv, force='-f' in sys.argv))
