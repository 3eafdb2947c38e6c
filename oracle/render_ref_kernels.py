"""Render the reference's CUDA kernel templates for the reference-GPU harness -- TEST INFRASTRUCTURE ONLY.

The reference compiles its kernels at run time: jinja2 fills the grid size (and,
for the potential kernel, the window shape, the padded site-list length and the
slice count) into namsa/probe_kernels.cu and namsa/potential_kernels.cu, and
pycuda's SourceModule compiles the result (namsa/cuda_kernels.py:8-57).  This
script performs the same rendering, with the same template variables, for the
workloads the parity tests use, and writes the rendered sources into
``oracle/_ref/`` (git-ignored, never part of the product):

  c1  Si 4x4x20 cells (face-inclusive), 256^2, 100 keV, t = a/4 (80 slices)
  c2  Si 8x8x50 cells (face-inclusive), 512^2, 200 keV, t = a/4 (199 slices)
  c4  SrTiO3 12x12x16 cells, 256^2, 300 keV, t = a/2 (three species)
  c5  SrTiO3 18x12x8 cells (x, y, z), a rectangular 256 x 384 (y, x) grid, 200 keV
  c6  Si 12x12x20 cells (face-inclusive), 768^2, 300 keV, t = a/4 (80 slices)
  c7  SrTiO3 40x40x12 cells, 1024^2, 300 keV, t = a/2 (24 slices)
  c8  a seeded random cubic crystal (seed 1: a = 5.56 A, Au, B, Si and Tm, 16 atoms per
      cell), 22x11x18 cells, a rectangular 384 x 768 (y, x) grid, 120 keV, t = 1.5 A

plus ``oracle/_ref/workloads.json`` with the rendered parameters.  The sources
are then compiled against the stand-in header ``oracle/pycuda-complex.hpp`` and
the harness ``oracle/refgpu_harness.cu`` by ``oracle/build_ref.py``.

The rendering needs a reference checkout, named by the ``NAMSA_REFERENCE``
environment variable or the first argument (``python oracle/render_ref_kernels.py
CHECKOUT``); machines without one use the rendered files already present in
``oracle/_ref/``.
"""
from __future__ import annotations

import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
OUT = os.path.join(HERE, '_ref')
REFERENCE = os.environ.get('NAMSA_REFERENCE')

A_SI = 5.431
A_STO = 3.905
WORKLOADS = {
    'c1': dict(crystal='si', cells=(4, 4, 20), n=256, kv=100.0, semi=20e-3, slice_t=A_SI / 4),
    'c2': dict(crystal='si', cells=(8, 8, 50), n=512, kv=200.0, semi=30e-3, slice_t=A_SI / 4),
    'c4': dict(crystal='srtio3', cells=(12, 12, 16), n=256, kv=300.0, semi=25e-3, slice_t=A_STO / 2),
    'c5': dict(crystal='srtio3', cells=(18, 12, 8), n=(256, 384), kv=200.0, semi=25e-3, slice_t=A_STO / 2),
    'c6': dict(crystal='si', cells=(12, 12, 20), n=768, kv=300.0, semi=25e-3, slice_t=A_SI / 4),
    'c7': dict(crystal='srtio3', cells=(40, 40, 12), n=1024, kv=300.0, semi=25e-3, slice_t=A_STO / 2),
    'c8': dict(crystal='random1', cells=(22, 11, 18), n=(384, 768), kv=120.0, semi=20e-3, slice_t=1.5),
}


def supercell(crystal, cells):
    from oracle import msa_oracle as O
    if crystal.startswith('random'):
        return O.random_supercell(int(crystal[len('random'):]), *cells)
    return O.si_supercell(*cells) if crystal == 'si' else O.srtio3_supercell(*cells)


def workload_params(tag):
    """Grid, window shape, slice count and padded site-list length of a workload,
    computed with the oracle's restatement of the reference's set-up."""
    sys.path.insert(0, ROOT)
    from oracle import msa_oracle as O
    w = WORKLOADS[tag]
    ny, nx = w['n'] if isinstance(w['n'], tuple) else (w['n'], w['n'])
    sc = supercell(w['crystal'], w['cells'])
    xyz = np.column_stack([sc['x'], sc['y'], sc['z']]).astype(np.float32)
    geom = O.Geometry(xyz, sc['atomic_number'], w['kv'], w['semi'], [ny, nx])
    kirk = np.load(os.path.join(ROOT, 'namsa_gb300', 'data', 'kirkland_params.npy'))
    _, win = O.atom_windows(geom, kirk)
    t = w['slice_t']
    sites = O.slice_sites_gpu(geom, t)
    max_sites = max(len(s) for s in sites)
    return dict(tag=tag, ny=ny, nx=nx, pot_y=int(win.shape[1]), pot_x=int(win.shape[2]),
                num_slices=len(sites), sites_size=3 * max_sites, species=int(win.shape[0]),
                crystal=w['crystal'], cells=list(w['cells']), kv=w['kv'], semi=w['semi'], slice_t=t)


def render(reference=None, out=OUT):
    from jinja2 import Template
    reference = reference or REFERENCE
    if not reference:
        raise RuntimeError('no reference checkout: set NAMSA_REFERENCE or pass its path')
    os.makedirs(out, exist_ok=True)
    with open(os.path.join(reference, 'namsa', 'probe_kernels.cu')) as f:
        probe_t = Template(f.read())
    with open(os.path.join(reference, 'namsa', 'potential_kernels.cu')) as f:
        pot_t = Template(f.read())
    meta = {}
    for tag in WORKLOADS:
        p = workload_params(tag)
        # same variables as ProbeKernels / PotentialKernels (namsa/cuda_kernels.py:16-19, 42-51)
        probe_src = probe_t.render(type='pycuda::complex<float>', y_sampling=np.int32(p['ny']),
                                   x_sampling=np.int32(p['nx']))
        pot_src = pot_t.render(y_sampling=np.int32(p['ny']), x_sampling=np.int32(p['nx']),
                               pot_shape_y=np.int32(p['pot_y']), pot_shape_x=np.int32(p['pot_x']),
                               sites_size=np.int32(p['sites_size']), num_slices=np.int32(p['num_slices']))
        with open(os.path.join(out, f'ref_probe_kernels_{tag}.cu'), 'w') as f:
            f.write(probe_src)
        with open(os.path.join(out, f'ref_potential_kernels_{tag}.cu'), 'w') as f:
            f.write(pot_src)
        meta[tag] = p
    with open(os.path.join(out, 'workloads.json'), 'w') as f:
        json.dump(meta, f, indent=1)
    return meta


def available(reference=None):
    reference = reference or REFERENCE
    return bool(reference) and os.path.exists(os.path.join(reference, 'namsa', 'probe_kernels.cu'))


if __name__ == '__main__':
    print(json.dumps(render(*sys.argv[1:2]), indent=1))
