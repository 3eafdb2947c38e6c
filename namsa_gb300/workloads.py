"""Uneven multi-crystal batches (many materials on one GPU).

The reference distributes materials over MPI ranks, one crystal at a time per
GPU (scripts/sim_batch.py:201, scripts/summit_scripts/sim_prod.py:157-224).
Here a list of crystals of different grid size, thickness, slice thickness,
voltage and probe count is prepared on one GPU and run as one graph
(``engine.Batch``).

``random_batch`` draws the seeded batch: cubic cells with a ~ U[3, 8]
Angstrom, 1-4 species with Z ~ U{3..83}, 2-16 atoms at uniform fractional
positions; grids from {256, 384, 512, 768}^2 reached by lateral tiling at
about 0.12 Angstrom per pixel; thickness ~ U[50, 500] Angstrom; slice
thickness ~ U[1, 2] Angstrom; voltage from {80, 120, 200, 300} kV; 16-256
probe positions over one unit cell.
"""
from __future__ import annotations

import math

import numpy as np
import torch

from . import engine, structures
from .msa import MSAGPU

GRIDS = (256, 384, 512, 768)
VOLTAGES_KV = (80, 120, 200, 300)
PROBE = {'smooth_apert': True, 'apert_smooth': 50, 'spherical_phase': True,
         'aberration_dict': {'C1': 0., 'C3': 0., 'C5': 0.}, 'scherzer': False}


def random_crystal(rng, grids=GRIDS, thickness=(50., 500.), slice_t=(1., 2.), voltages=VOLTAGES_KV,
                   probes=(16, 256), pixel=0.12):
    """Parameters of one random crystal of the uneven batch."""
    basis, species, a = structures.random_cubic(rng)
    n = int(rng.choice(grids))
    m = max(1, int(round(n * pixel / a)))           # lateral cells
    thick = rng.uniform(*thickness)
    nz = max(1, int(math.ceil(thick / a)))
    return dict(basis=basis, species=species, a=a, n=n, cells=(m, m, nz), slice_t=float(rng.uniform(*slice_t)),
                kv=int(rng.choice(voltages)), probes=int(rng.integers(probes[0], probes[1] + 1)),
                positions_seed=int(rng.integers(1 << 31)))


def prepare(spec, device, semi_angle=25e-3, crop=None):
    """Build the transmission stack, probe and positions of one crystal on `device`."""
    sc = structures.tile(spec['basis'], spec['species'], spec['cells'], spec['a'])
    sim = MSAGPU(spec['kv'], semi_angle, sc, sampling=np.array([spec['n'], spec['n']]), debye_waller=False)
    sim.setup_device(device.index if device.index is not None else 0)
    sim.calc_atomic_potentials()
    sim.build_potential_slices(spec['slice_t'])
    sim.build_probe(PROBE)
    prng = np.random.default_rng(spec['positions_seed'])
    pos = prng.uniform(0, spec['a'], size=(spec['probes'], 2)).astype(np.float32)
    c = crop or spec['n']
    job = dict(trans=sim.trans, psik=sim.psi_k_dev, norm=sim.norm_dev,
               positions=torch.from_numpy(pos).to(device), kmax=np.float32(sim.kmax), lam=sim.Lambda,
               slice_t=spec['slice_t'], k_band=np.float32(sim.kmax / 3),
               out=torch.empty((spec['probes'], c, c), dtype=torch.float32, device=device))
    return sim, job


def random_batch(seed, count=64, device=None, crop=None, **kw):
    """`count` seeded random crystals ready for engine.Batch.run; returns (specs, sims, jobs)."""
    device = device or torch.device('cuda', torch.cuda.current_device())
    rng = np.random.default_rng(seed)
    specs = [random_crystal(rng, **kw) for _ in range(count)]
    sims, jobs = [], []
    for s in specs:
        sim, job = prepare(s, device, crop=crop)
        sims.append(sim)
        jobs.append(job)
    return specs, sims, jobs


def work_units(jobs):
    """Total probe-slices and probe-slice-pixels of a job list."""
    ps = sum(j['positions'].shape[0] * j['trans'].shape[0] for j in jobs)
    psp = sum(j['positions'].shape[0] * j['trans'].shape[0] * j['trans'].shape[1] * j['trans'].shape[2] for j in jobs)
    return ps, psp
