"""Build ``libcdgpu.so`` in-tree with nvcc for sm_103a.

Translation units compile in parallel; the library links the CUDA runtime
dynamically.  ``build()`` is idempotent: it rebuilds only when a source or
header is newer than the library.
"""
import concurrent.futures
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, 'csrc')
BUILD = os.path.join(PKG, '_build')
LIB = os.path.join(PKG, 'libcdgpu.so')
SOURCES = ['cd_kernels.cu', 'cd_api.cu', 'cd_adjoint.cu', 'cd_states.cu']
HEADERS = [os.path.join(CSRC, h) for h in ('cd_internal.cuh', 'cd_cull.cuh', 'cd_math.h',
                                           'cd_noise.h')] + [os.path.join(ROOT, 'include', 'cdgpu.h')]
ARCH = ['-gencode', 'arch=compute_103a,code=sm_103a']
FLAGS = ['-O3', '-lineinfo', '-std=c++17', '--fmad=false', '-Xcompiler', '-fPIC,-O2',
         '-I', os.path.join(ROOT, 'include')]


def nvcc():
    exe = shutil.which('nvcc')
    if exe is None and os.path.exists('/usr/local/cuda/bin/nvcc'):
        exe = '/usr/local/cuda/bin/nvcc'
    if exe is None:
        raise RuntimeError('nvcc not found: the CUDA toolkit is required to build libcdgpu')
    return exe


def _stale():
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    deps = [os.path.join(CSRC, s) for s in SOURCES] + HEADERS
    return any(os.path.getmtime(d) > t for d in deps)


def build(force=False, verbose=False, extra_flags=()):
    """Compile and link libcdgpu.so; returns its path."""
    if not force and not _stale():
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    cc = nvcc()

    def compile_one(src):
        obj = os.path.join(BUILD, os.path.splitext(src)[0] + '.o')
        cmd = [cc] + ARCH + FLAGS + list(extra_flags) + ['-c', os.path.join(CSRC, src), '-o', obj]
        if verbose:
            print(' '.join(cmd))
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError('nvcc failed for %s:\n%s%s' % (src, r.stdout, r.stderr))
        return obj

    with concurrent.futures.ThreadPoolExecutor(len(SOURCES)) as ex:
        objs = list(ex.map(compile_one, SOURCES))
    tmp = LIB + '.tmp'
    cmd = [cc] + ARCH + ['-shared', '-cudart', 'shared', '-o', tmp] + objs
    if verbose:
        print(' '.join(cmd))
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError('nvcc link failed:\n%s%s' % (r.stdout, r.stderr))
    os.replace(tmp, LIB)
    return LIB


if __name__ == '__main__':
    build(force='--force' in sys.argv, verbose=True)
