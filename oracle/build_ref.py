"""Build the reference-GPU harness libraries -- TEST INFRASTRUCTURE ONLY.

For every workload rendered into ``oracle/_ref/`` by ``oracle/render_ref_kernels.py``
(``workloads.json``), compile ``oracle/refgpu_harness.cu`` together with the
rendered reference kernels and the stand-in ``oracle/pycuda-complex.hpp`` into
``oracle/_ref/libnamsa_refgpu_<tag>.so`` (sm_103a, linked with cuFFT).  When the
reference checkout is present the sources are rendered first; elsewhere the
rendered files already in ``oracle/_ref/`` are used, and with none there the
build is skipped (the tests that need the harness skip with that reason).
"""
from __future__ import annotations

import json
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, '_ref')
HARNESS = os.path.join(HERE, 'refgpu_harness.cu')
SHIM = os.path.join(HERE, 'pycuda-complex.hpp')


def lib_path(tag):
    return os.path.join(OUT, f'libnamsa_refgpu_{tag}.so')


def _nvcc():
    for cand in [os.environ.get('NVCC'), shutil.which('nvcc'), '/usr/local/cuda/bin/nvcc']:
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError('nvcc not found')


def commands():
    meta_path = os.path.join(OUT, 'workloads.json')
    if not os.path.exists(meta_path):
        return []
    meta = json.load(open(meta_path))
    nvcc = _nvcc()
    cmds = []
    for tag, p in meta.items():
        probe = f'ref_probe_kernels_{tag}.cu'
        pot = f'ref_potential_kernels_{tag}.cu'
        out = lib_path(tag)
        deps = [HARNESS, SHIM, os.path.join(OUT, probe), os.path.join(OUT, pot), meta_path]
        if os.path.exists(out) and all(os.path.getmtime(d) <= os.path.getmtime(out) for d in deps):
            continue
        cmds.append([nvcc, '-gencode', 'arch=compute_103a,code=sm_103a', '-O3', '-std=c++17', '-shared',
                     '-Xcompiler', '-fPIC', '-w', '-I', HERE, '-I', OUT,
                     f'-DREF_NY={p["ny"]}', f'-DREF_NX={p["nx"]}', f'-DREF_S={p["num_slices"]}',
                     f'-DREF_POT_Y={p["pot_y"]}', f'-DREF_POT_X={p["pot_x"]}', f'-DREF_SITES={p["sites_size"]}',
                     f'-DREF_PROBE_SRC="{probe}"', f'-DREF_POT_SRC="{pot}"',
                     HARNESS, '-o', out, '-lcufft'])
    return cmds


def build(render=True):
    if render:
        sys.path.insert(0, os.path.dirname(HERE))
        from oracle import render_ref_kernels as R
        if R.available():
            meta = os.path.join(OUT, 'workloads.json')
            srcs = [os.path.join(HERE, 'render_ref_kernels.py')]
            if not os.path.exists(meta) or any(os.path.getmtime(s) > os.path.getmtime(meta) for s in srcs):
                R.render()
    cmds = commands()
    procs = [subprocess.Popen(c, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True) for c in cmds]
    for c, p in zip(cmds, procs):
        out, _ = p.communicate()
        if p.returncode != 0:
            raise RuntimeError('reference harness build failed:\n' + ' '.join(c) + '\n' + out)
    return [c[-2] for c in cmds]


if __name__ == '__main__':
    print(build())
