"""Build libmusg.so in-tree for GB300 (sm_103a).

The CUDA translation units are compiled by nvcc with ``-gencode
arch=compute_103a,code=sm_103a``, the host C++ by g++, all in parallel, and linked
into ``muspectre_gb300/libmusg.so`` (static CUDA runtime, no PyTorch dependency).
Rebuilds only when a source is newer than the library.

    python -m muspectre_gb300.build [--force]
"""
from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, 'csrc')
ROOT = os.path.dirname(HERE)
INCLUDE = os.path.join(ROOT, 'include')
BUILD = os.path.join(HERE, '_build')
LIB = os.path.join(HERE, 'libmusg.so')

ARCH = ['-gencode', 'arch=compute_103a,code=sm_103a']


def _nvcc():
    for cand in (os.environ.get('NVCC'), shutil.which('nvcc'), '/usr/local/cuda/bin/nvcc'):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError('nvcc not found: the CUDA toolkit is required to build libmusg')


def _cuda_root(nvcc):
    return os.path.dirname(os.path.dirname(os.path.realpath(nvcc)))


def sources():
    cu = sorted(glob.glob(os.path.join(CSRC, '*.cu')))
    cpp = sorted(glob.glob(os.path.join(CSRC, '*.cpp')))
    deps = cu + cpp + glob.glob(os.path.join(CSRC, '*.cuh')) + glob.glob(os.path.join(CSRC, '*.h')) + \
        glob.glob(os.path.join(INCLUDE, '*.h'))
    return cu, cpp, deps


def _run(cmd):
    p = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if p.returncode != 0:
        raise RuntimeError('build step failed: %s\n%s' % (' '.join(cmd), p.stdout))
    return p.stdout


def up_to_date():
    if not os.path.exists(LIB):
        return False
    t = os.path.getmtime(LIB)
    _, _, deps = sources()
    return all(os.path.getmtime(d) <= t for d in deps)


def build(force=False, verbose=False, jobs=None):
    if not force and up_to_date():
        return LIB
    nvcc = _nvcc()
    cuda = _cuda_root(nvcc)
    os.makedirs(BUILD, exist_ok=True)
    cu, cpp, _ = sources()
    common = ['-std=c++17', '-O3', '-I', CSRC, '-I', INCLUDE]
    cmds = []
    objs = []
    for src in cu:
        obj = os.path.join(BUILD, os.path.basename(src) + '.o')
        objs.append(obj)
        cmds.append([nvcc] + ARCH + common + ['-lineinfo', '-Xcompiler', '-fPIC', '-c', src, '-o', obj])
    for src in cpp:
        obj = os.path.join(BUILD, os.path.basename(src) + '.o')
        objs.append(obj)
        cmds.append(['g++'] + common + ['-fPIC', '-Wall', '-I', os.path.join(cuda, 'include'), '-c', src, '-o', obj])
    jobs = jobs or max(1, min(len(cmds), os.cpu_count() or 4))
    with cf.ThreadPoolExecutor(jobs) as ex:
        for out in ex.map(_run, cmds):
            if verbose and out.strip():
                print(out)
    tmp = LIB + '.tmp'
    _run([nvcc] + ARCH + ['-shared', '-o', tmp] + objs + ['-lcudart_static', '-lrt', '-lpthread', '-ldl'])
    os.replace(tmp, LIB)
    return LIB


if __name__ == '__main__':
    print(build(force='--force' in sys.argv, verbose=True))
