"""Learned coarse-slice corrector: training data, training and corrected multislice.

A coarse step propagates through one slice four times as thick as the fine
one (the transmission of four fine slices and the Fresnel propagator of
their summed thickness).  It is four times cheaper but its splitting error
grows with the thickness.  The corrector network (``engine.Corrector``,
kernels in csrc/msx_corrector.cu) maps the wave after a coarse step, together
with that step's transmission, to the wave after the four fine steps.  Plain
fine-slice multislice generates the training pairs on the device and judges
the corrected result.

Waves handed to the network are scaled to unit mean intensity per pixel
(multiplied by sqrt(N / norm), norm = sum |psi_0|^2).
"""
from __future__ import annotations

import math
import time

import numpy as np
import torch

from . import engine, structures
from .msa import MSAGPU

PROBE = {'smooth_apert': True, 'apert_smooth': 50, 'spherical_phase': True,
         'aberration_dict': {'C1': 0., 'C3': 0., 'C5': 0.}, 'scherzer': False}


def init_params(C, L, seed=0, K=8):
    """Seeded initial parameters in the library's layout: fan-in scaled linear
    maps, spectral weights ~ 1/C, and a zero output layer (the untrained
    network returns the coarse wave exactly)."""
    rng = np.random.default_rng(seed)
    parts = [rng.standard_normal((C, 4)) / 2.0, np.zeros(C)]
    for _ in range(L):
        parts += [rng.standard_normal((K, K, C, C)) / C, rng.standard_normal((K, K, C, C)) / C,
                  rng.standard_normal((C, C)) / math.sqrt(C), np.zeros(C)]
    parts += [rng.standard_normal((C, C)) / math.sqrt(C), np.zeros(C),
              np.zeros((2, C)), np.zeros(2)]
    return np.concatenate([p.ravel() for p in parts]).astype(np.float32)


class Crystal:
    """A crystal prepared at fine and coarse slicing on one grid."""

    def __init__(self, sites, n, slice_t, kv=200, semi_angle=20e-3, device=None, ratio=4):
        self.sim = MSAGPU(kv, semi_angle, sites, sampling=np.array([n, n]), debye_waller=False)
        dev = device or torch.device('cuda', torch.cuda.current_device())
        self.sim.setup_device(dev.index if dev.index is not None else 0)
        self.sim.calc_atomic_potentials()
        self.sim.build_potential_slices(ratio * slice_t)
        self.trans_coarse = self.sim.trans
        self.sim.build_potential_slices(slice_t)
        self.trans_fine = self.sim.trans
        self.sim.build_probe(PROBE)
        self.n, self.ratio, self.slice_t = n, ratio, slice_t
        self.coarse_steps = self.trans_coarse.shape[0]
        kmax = np.float32(self.sim.kmax)
        kband = np.float32(self.sim.kmax / 3)
        self.kmax = kmax
        self.ptab_fine = engine.propagator_table(n, n, kmax, self.sim.Lambda, slice_t, kband)
        self.ptab_coarse = engine.propagator_table(n, n, kmax, self.sim.Lambda, ratio * slice_t, kband)
        self.scale = math.sqrt(n * n / self.sim.normalization)
        self.plan = engine.Plan(n, n)

    def waves(self, positions):
        pos = torch.as_tensor(np.asarray(positions, np.float32), device=self.trans_fine.device)
        return self.plan.probe_waves(self.sim.psi_k_dev, pos, self.kmax)

    def pairs(self, positions, steps=None):
        """(psi_coarse, psi_fine, coarse-slice index) for every coarse step of every
        position, scaled to unit mean intensity."""
        w = self.waves(positions)
        steps = self.coarse_steps if steps is None else min(steps, self.coarse_steps)
        out_c, out_f, idx = [], [], []
        for k in range(steps):
            c = w.clone()
            self.plan.step_waves(c, self.trans_coarse[k], self.ptab_coarse)
            for j in range(self.ratio * k, self.ratio * (k + 1)):
                self.plan.step_waves(w, self.trans_fine[j], self.ptab_fine)
            out_c.append(c * self.scale)
            out_f.append(w * self.scale)
            idx.append(torch.full((w.shape[0],), k, dtype=torch.long, device=w.device))
        return torch.cat(out_c), torch.cat(out_f), torch.cat(idx)


def training_crystals(n=256, seed=0, random_count=6):
    """Si [001], SrTiO3 [001] and seeded random cubic crystals on an n x n grid,
    about 1000 Angstrom thick."""
    rng = np.random.default_rng(seed)
    cells = max(1, int(round(n * 0.085 / 5.431)))
    out = [('Si[001]', structures.silicon((cells, cells, 184)), 5.431 / 4, 5.431)]
    cs = max(1, int(round(n * 0.085 / 3.905)))
    out.append(('SrTiO3[001]', structures.srtio3((cs, cs, 256)), 3.905 / 2, 3.905))
    for i in range(random_count):
        basis, species, a = structures.random_cubic(rng)
        m = max(1, int(round(n * 0.1 / a)))
        nz = int(math.ceil(1000.0 / a))
        out.append((f'random{i}', structures.tile(basis, species, (m, m, nz), a), float(rng.uniform(1.0, 2.0)), a))
    return out


def train(net, data_c, data_f, data_t, steps, batch, lr=1e-3, seed=0, log=None):
    """Adam on random batches of pairs; every pair is weighted by the inverse of its
    own coarse error, so the loss is the mean ratio (corrected error / coarse error)
    and 1 means no gain.  Returns the per-step losses."""
    g = torch.Generator(device='cpu').manual_seed(seed)
    n = data_c.shape[0]
    losses = []
    for s in range(steps):
        idx = torch.randint(0, n, (batch,), generator=g).to(data_c.device)
        c, f, t = data_c[idx].contiguous(), data_f[idx].contiguous(), data_t[idx].contiguous()
        w = 1.0 / (f - c).abs().pow(2).sum((1, 2)).clamp_min(1e-20).float()
        loss = net.loss_grad(c, t, f, float(batch), weights=w.contiguous())
        net.adam(lr=lr * (0.5 * (1 + math.cos(math.pi * s / steps))))
        losses.append(float(loss.item()))
        if log and s % 100 == 0:
            log(f'step {s} loss {losses[-1]:.4f}')
    return losses


def rollout_pairs(net, crystal, positions, steps=None):
    """Pairs taken along the corrector's own trajectory: at every coarse step the
    target is four fine steps from the current corrected wave.  Training on them
    teaches the network the states it meets when it is applied repeatedly."""
    w = crystal.waves(positions)
    steps = crystal.coarse_steps if steps is None else min(steps, crystal.coarse_steps)
    out_c, out_f, idx = [], [], []
    B = w.shape[0]
    for k in range(steps):
        c = w.clone()
        crystal.plan.step_waves(c, crystal.trans_coarse[k], crystal.ptab_coarse)
        f = w.clone()
        for j in range(crystal.ratio * k, crystal.ratio * (k + 1)):
            crystal.plan.step_waves(f, crystal.trans_fine[j], crystal.ptab_fine)
        cs, fs = c * crystal.scale, f * crystal.scale
        out_c.append(cs)
        out_f.append(fs)
        idx.append(torch.full((B,), k, dtype=torch.long, device=w.device))
        nxt = torch.empty_like(cs)
        for b0 in range(0, B, net.max_batch):
            chunk = cs[b0:b0 + net.max_batch].contiguous()
            tc = crystal.trans_coarse[k].expand(chunk.shape[0], -1, -1).contiguous()
            nxt[b0:b0 + net.max_batch] = net.forward(chunk, tc)
        w = (nxt / crystal.scale).contiguous()
    return torch.cat(out_c), torch.cat(out_f), torch.cat(idx)


def corrected_multislice(net, crystal, positions, steps=None, use_net=True):
    """CBED of coarse-step multislice with (or without) the corrector."""
    w = crystal.waves(positions) * crystal.scale
    steps = crystal.coarse_steps if steps is None else steps
    B = w.shape[0]
    for k in range(steps):
        crystal.plan.step_waves(w, crystal.trans_coarse[k], crystal.ptab_coarse)
        if use_net:
            for b0 in range(0, B, net.max_batch):
                chunk = w[b0:b0 + net.max_batch].contiguous()
                tc = crystal.trans_coarse[k].expand(chunk.shape[0], -1, -1).contiguous()
                w[b0:b0 + net.max_batch] = net.forward(chunk, tc)
    w = (w / crystal.scale).contiguous()
    return crystal.plan.cbed_waves(w, crystal.sim.norm_dev)


def fine_multislice(crystal, positions, steps=None):
    """CBED of plain fine-slice multislice (the fused engine path) through the
    same thickness as `steps` coarse steps."""
    steps = crystal.coarse_steps if steps is None else steps
    sim = crystal.sim
    pos = torch.as_tensor(np.asarray(positions, np.float32), device=crystal.trans_fine.device)
    trans = crystal.trans_fine[:crystal.ratio * steps].contiguous()
    return crystal.plan.multislice(trans, sim.psi_k_dev, sim.norm_dev, pos, crystal.kmax, sim.Lambda,
                                   crystal.slice_t, np.float32(sim.kmax / 3))


def rel_l2(a, b):
    a, b = a.double(), b.double()
    return (torch.linalg.vector_norm(a - b, dim=(1, 2)) / torch.linalg.vector_norm(b, dim=(1, 2))).cpu().numpy()


def timed(fn, reps=3):
    fn()  # first call outside the timing (lazy set-up)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(reps):
        out = fn()
    torch.cuda.synchronize()
    return out, (time.perf_counter() - t0) / reps
