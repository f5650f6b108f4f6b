"""Builds the engine's shared library (liboit_gb300.so) in-tree with nvcc.

Every CUDA translation unit is compiled for sm_103a only and in parallel;
host C++ is compiled with -ffp-contract=off so scene generation gives the same
bits on x86-64 and aarch64 hosts.
"""
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(PKG, 'csrc')
LIB = os.path.join(PKG, 'liboit_gb300.so')
BUILD = os.path.join(PKG, '_objs')

CU_SOURCES = ['setup_bin.cu', 'raster_a.cu', 'raster_b.cu', 'raster_c.cu', 'composite.cu', 'resolve.cu',
              'verify.cu', 'arrival.cu', 'noalloc.cu']
CPP_SOURCES = ['engine.cpp', 'scene.cpp']
ARCH = ['-gencode', 'arch=compute_103a,code=sm_103a']


def nvcc():
    for cand in (os.environ.get('NVCC'), shutil.which('nvcc'), '/usr/local/cuda/bin/nvcc'):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError('nvcc not found')


def _newer(target, sources):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(s) > t for s in sources)


def _headers():
    return [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(('.h', '.cuh', '.inc'))] + [
        os.path.join(PKG, '..', 'include', 'oit_gb300.h')]


def build(verbose=False, force=False):
    os.makedirs(BUILD, exist_ok=True)
    cc = nvcc()
    hdrs = _headers()
    jobs = []
    objs = []
    for src in CU_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD, src + '.o')
        objs.append(o)
        if force or _newer(o, [s] + hdrs):
            jobs.append([cc, *ARCH, '-O3', '-lineinfo', '-std=c++17', '-Xcompiler', '-fPIC,-ffp-contract=off',
                         '-c', s, '-o', o])
    for src in CPP_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD, src + '.o')
        objs.append(o)
        if force or _newer(o, [s] + hdrs):
            jobs.append([cc, '-x', 'c++', '-O2', '-std=c++17', '-Xcompiler', '-fPIC,-ffp-contract=off,-Wall',
                         '-c', s, '-o', o])

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError('build failed: %s\n%s%s' % (' '.join(cmd), r.stdout, r.stderr))
        if verbose:
            sys.stderr.write(r.stdout + r.stderr)
        return r

    with ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        list(ex.map(run, jobs))
    if force or jobs or _newer(LIB, objs):
        run([cc, *ARCH, '-shared', '-o', LIB, *objs, '-lcudart'])
    return LIB


if __name__ == '__main__':
    print(build(verbose='-v' in sys.argv, force='-f' in sys.argv))
