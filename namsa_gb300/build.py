"""In-tree build of libmsx.so (the CUDA engine) for sm_103a.

Each translation unit under ``csrc/`` is compiled by nvcc in parallel into
``_build/`` and linked into ``namsa_gb300/libmsx.so``.  Objects are rebuilt
when a source or header is newer.  Run ``python -m namsa_gb300.build``.
"""
from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, 'csrc')
BUILD = os.path.join(PKG, '_build')
LIB = os.path.join(PKG, 'libmsx.so')
ARCH = ['-gencode', 'arch=compute_103a,code=sm_103a']
FLAGS = ['-std=c++17', '-O3', '-lineinfo', '-Xcompiler', '-fPIC', '-Xcompiler', '-fvisibility=hidden',
         '-I', os.path.join(ROOT, 'include'), '-I', CSRC]


def _nvcc():
    for cand in [os.environ.get('NVCC'), shutil.which('nvcc'), '/usr/local/cuda/bin/nvcc']:
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError('nvcc not found: the CUDA toolkit is required to build libmsx.so')


def _stale(obj, deps):
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose=False, jobs=None):
    nvcc = _nvcc()
    os.makedirs(BUILD, exist_ok=True)
    sources = sorted(glob.glob(os.path.join(CSRC, '*.cu')))
    headers = glob.glob(os.path.join(CSRC, '*.cuh')) + glob.glob(os.path.join(CSRC, '*.h')) + \
        glob.glob(os.path.join(ROOT, 'include', '*.h'))
    objs, cmds = [], []
    for src in sources:
        obj = os.path.join(BUILD, os.path.basename(src)[:-3] + '.o')
        objs.append(obj)
        if _stale(obj, [src] + headers):
            cmds.append([nvcc, *ARCH, *FLAGS, '-c', src, '-o', obj])

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError('nvcc failed:\n' + ' '.join(cmd) + '\n' + r.stdout + r.stderr)
        if verbose:
            print(' '.join(cmd[-3:]), flush=True)
        return r

    with cf.ThreadPoolExecutor(max_workers=jobs or min(len(cmds), os.cpu_count() or 4) or 1) as ex:
        list(ex.map(run, cmds))
    if cmds or _stale(LIB, objs):
        tmp = LIB + '.tmp'
        run([nvcc, *ARCH, '-shared', '-Xcompiler', '-fPIC', '-o', tmp, *objs])
        os.replace(tmp, LIB)
    return LIB


if __name__ == '__main__':
    print(build(verbose='-v' in sys.argv))
