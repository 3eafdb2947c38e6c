"""Learned coarse-slice corrector: data, rollout training and corrected multislice.

A coarse step propagates through one slice ``ratio`` (4) times as thick as the
fine one: the transmission of the fine slices it contains and the Fresnel
propagator of their summed thickness.  It costs a quarter of the fine steps
but its splitting error grows with the thickness.  The corrected coarse step is

    psi <- a_k ifft2(P_c fft2(b_k t_k psi)),   a_k = exp(i Im A_k),  b_k = exp(i Im B_k)

with per-pixel maps A_k, B_k that the corrector network
(``engine.Corrector``, csrc/msx_corrector.cu) computes from the potentials of
the fine slices inside coarse slice k.  The maps depend on the crystal only, so
they fold into the transmission slices of a plain multislice run:

    t'_0 = b_0 t_0,  t'_k = a_{k-1} b_k t_k,  t'_S = a_{S-1}

(unit-modulus factors keep each corrected step norm-preserving like the exact
fine steps; the general factors 1 + M are kept as ``form=0``)

(the extra last slice only multiplies; its propagator phase does not change
the CBED).  The corrected multislice of every probe position therefore runs
through ``Plan.multislice`` at the cost of a coarse-slice run.

Training follows the corrector's own rollouts: a window of K corrected coarse
steps from a fine-slice wave, loss = sum over steps of the relative squared
error against the fine-slice waves at the same depth, back-propagated through
the engine's slice step (``Plan.step_waves``; the adjoint step is the same
transform with the conjugate propagator) into the maps and the network.
Plain fine-slice multislice generates the targets and judges the result.
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
RATIO = 4
# Correction factors: 0 = 1 + M, 1 = exp(i Im M).  The unit-modulus form keeps every corrected
# step norm-preserving, as the exact fine steps are; with 1 + M the total intensity drifted by
# 2 % over 1000 A of Si and long rollouts lost their gain.
FORM = 1


def init_params(net, seed=0, out_scale=1e-2, spec_scale=0.5):
    """Seeded initial parameters in the library's layout (engine.Corrector.views):
    fan-in scaled weights, spectral weights ~ spec_scale / C, zero biases and a
    small output layer, so the untrained maps are close to zero."""
    rng = np.random.default_rng(seed)
    flat = np.zeros(net.count, np.float32)
    v = net.views(torch.from_numpy(flat))
    C, Ci = net.channels, net.in_channels
    for name, t in v.items():
        if name[0] in 'bc':
            continue
        if name == 'W0':
            val = rng.standard_normal(t.shape) / math.sqrt(Ci)
        elif name.startswith('R'):
            val = rng.standard_normal(t.shape) * spec_scale / C
        elif name == 'P2':
            val = rng.standard_normal(t.shape) * out_scale / math.sqrt(C)
        else:
            val = rng.standard_normal(t.shape) / math.sqrt(C)
        t.copy_(torch.from_numpy(val.astype(np.float32)))
    return flat


class Crystal:
    """A crystal prepared at fine and coarse slicing on one grid, with the fine
    potentials the corrector reads."""

    def __init__(self, sites, n, slice_t, kv=200, semi_angle=20e-3, device=None, ratio=RATIO):
        self.sim = MSAGPU(kv, semi_angle, sites, sampling=np.array([n, n]), debye_waller=False)
        dev = device or torch.device('cuda', torch.cuda.current_device())
        self.sim.setup_device(dev.index if dev.index is not None else 0)
        self.sim.calc_atomic_potentials()
        self.sim.build_potential_slices(ratio * slice_t)
        self.trans_coarse = self.sim.trans
        self.sim.build_potential_slices(slice_t, keep_potential=True)
        self.trans_fine = self.sim.trans
        self.pot_fine = self.sim.potential
        self.sim.build_probe(PROBE)
        self.n, self.ratio, self.slice_t = n, ratio, slice_t
        self.coarse_steps = min(self.trans_coarse.shape[0], self.trans_fine.shape[0] // ratio)
        kmax = np.float32(self.sim.kmax)
        kband = np.float32(self.sim.kmax / 3)
        self.kmax, self.kband = kmax, kband
        self.ptab_fine = engine.propagator_table(n, n, kmax, self.sim.Lambda, slice_t, kband)
        self.ptab_coarse = engine.propagator_table(n, n, kmax, self.sim.Lambda, ratio * slice_t, kband)
        self.ptab_coarse_adj = torch.conj_physical(self.ptab_coarse)
        self.ones = torch.ones((n, n), dtype=torch.complex64, device=self.trans_fine.device)
        self.plan = engine.Plan(n, n)
        self._features = None

    def features(self):
        """Network inputs of every coarse slice (S, n, n, ratio + 2): sigma V of its fine
        slices, their sum, and the fine slice thickness in Angstrom / 2."""
        if self._features is None:
            pot = self.pot_fine[:self.ratio * self.coarse_steps].contiguous()
            self._features = engine.corrector_features(pot, self.ratio, float(self.sim.sigma), self.slice_t / 2.0)
        return self._features

    def waves(self, positions):
        pos = torch.as_tensor(np.asarray(positions, np.float32), device=self.trans_fine.device)
        return self.plan.probe_waves(self.sim.psi_k_dev, pos, self.kmax)

    def trajectory(self, positions, steps=None):
        """Fine-slice waves at every coarse boundary: (steps + 1, P, n, n) complex64."""
        steps = self.coarse_steps if steps is None else min(steps, self.coarse_steps)
        w = self.waves(positions)
        out = torch.empty((steps + 1,) + tuple(w.shape), dtype=torch.complex64, device=w.device)
        out[0] = w
        for k in range(steps):
            for j in range(self.ratio * k, self.ratio * (k + 1)):
                self.plan.step_waves(w, self.trans_fine[j], self.ptab_fine)
            out[k + 1] = w
        return out

    def effective_slices(self, maps, form=FORM):
        """Transmission slices of the corrected multislice (S + 1, n, n) from the maps (S, n, n, 4)
        (form 0: factors 1 + M; form 1: unit-modulus factors exp(i Im M))."""
        S = maps.shape[0]
        out = torch.empty((S + 1, self.n, self.n), dtype=torch.complex64, device=maps.device)
        for k in range(S):
            engine.map_trans(self.trans_coarse[k], maps[k], 1, out=out[k], form=form)
            if k > 0:
                engine.map_trans(out[k].clone(), maps[k - 1], 0, out=out[k], form=form)
        engine.map_trans(self.ones, maps[S - 1], 0, out=out[S], form=form)
        return out


def wave_norms(traj):
    """sum |f|^2 of every wave of a trajectory (steps + 1, P, n, n), as a host array (steps + 1, P)."""
    zero = torch.zeros_like(traj[0, :1])
    adj = torch.empty_like(zero)
    buf = torch.zeros(1, dtype=torch.float32, device=traj.device)
    out = np.zeros(traj.shape[:2])
    for k in range(traj.shape[0]):
        for p in range(traj.shape[1]):
            engine.residual(zero, traj[k, p:p + 1], 1.0, adj, buf)
            out[k, p] = float(buf.item())
    return out


def distinct_slices(features):
    """The coarse slices whose network inputs are bitwise equal to an earlier slice's (the
    repeated slices of a periodic crystal): returns (first, index), `first` the slices
    that start a group and `index[s]` the group of slice s.  Candidates share a weighted
    sum of their inputs' bit patterns; every candidate is confirmed by exact comparison,
    and an unconfirmed one keeps a group of its own."""
    S = features.shape[0]
    flat = features.reshape(S, -1)
    # integer key: the bit patterns times fixed weights, summed exactly in int64 (bitwise
    # equal slices get equal keys whatever the summation order)
    w = 1 + torch.arange(flat.shape[1], device=flat.device) % 251
    B = 16  # slices per chunk: bounds the temporaries
    keys = torch.cat([(flat[i:i + B].contiguous().view(torch.int32).to(torch.int64) * w).sum(1)
                      for i in range(0, S, B)]).tolist()
    cand, seen = [], {}
    for s in range(S):
        cand.append(seen.setdefault(keys[s], s))
    idx = torch.as_tensor(cand, device=flat.device)
    same = torch.cat([(flat[i:i + B] == flat[idx[i:i + B]]).all(1) for i in range(0, S, B)]).tolist()
    first, index, group = [], [], {}
    for s in range(S):
        c = cand[s] if same[s] else s
        if c not in group:
            group[c] = len(first)
            first.append(c)
        index.append(group[c])
    return first, index


def crystal_maps(net, crystal, dedup=True):
    """Correction maps of every coarse slice of a crystal.  The network runs once per
    distinct slice (once per slice with dedup=False): equal inputs give equal maps."""
    f = crystal.features()
    S = f.shape[0]
    if dedup:
        first, index = distinct_slices(f)
        if len(first) < S:
            u = crystal_maps_of(net, f[first].contiguous())
            return u[torch.as_tensor(index, device=f.device)].contiguous()
    return crystal_maps_of(net, f)


def crystal_maps_of(net, f):
    """Network maps (S, n, n, 4) of the inputs f (S, n, n, channels), max_samples at a time."""
    S = f.shape[0]
    out = torch.empty((S,) + tuple(f.shape[1:3]) + (4,), dtype=torch.float32, device=f.device)
    for s0 in range(0, S, net.max_samples):
        net.forward(f[s0:s0 + net.max_samples].contiguous(), out=out[s0:s0 + net.max_samples])
    return out


def corrected_multislice(net, crystal, positions, steps=None, maps=None, trans=None, form=FORM):
    """CBED of the corrected coarse-slice multislice through `steps` coarse slices,
    run by Plan.multislice on the effective transmission slices."""
    steps = crystal.coarse_steps if steps is None else steps
    if trans is None:
        maps = crystal_maps(net, crystal) if maps is None else maps
        trans = crystal.effective_slices(maps[:steps].contiguous(), form)
    sim = crystal.sim
    pos = torch.as_tensor(np.asarray(positions, np.float32), device=crystal.trans_fine.device)
    return crystal.plan.multislice(trans, sim.psi_k_dev, sim.norm_dev, pos, crystal.kmax, sim.Lambda,
                                   crystal.ratio * crystal.slice_t, crystal.kband)


def coarse_multislice(crystal, positions, steps=None):
    """CBED of plain coarse-slice multislice through `steps` coarse slices."""
    steps = crystal.coarse_steps if steps is None else steps
    sim = crystal.sim
    pos = torch.as_tensor(np.asarray(positions, np.float32), device=crystal.trans_fine.device)
    return crystal.plan.multislice(crystal.trans_coarse[:steps].contiguous(), sim.psi_k_dev, sim.norm_dev, pos,
                                   crystal.kmax, sim.Lambda, crystal.ratio * crystal.slice_t, crystal.kband)


def fine_multislice(crystal, positions, steps=None):
    """CBED of plain fine-slice multislice (the error reference) through the same
    thickness as `steps` coarse steps."""
    steps = crystal.coarse_steps if steps is None else steps
    sim = crystal.sim
    pos = torch.as_tensor(np.asarray(positions, np.float32), device=crystal.trans_fine.device)
    trans = crystal.trans_fine[:crystal.ratio * steps].contiguous()
    return crystal.plan.multislice(trans, sim.psi_k_dev, sim.norm_dev, pos, crystal.kmax, sim.Lambda,
                                   crystal.slice_t, crystal.kband)


class RolloutTrainer:
    """Windowed rollout training of a corrector over a set of crystals."""

    def __init__(self, net, crystals, trajectories, window=8, waves=8, seed=0, form=FORM):
        self.net, self.crystals, self.traj = net, crystals, trajectories
        self.norms = [wave_norms(t) for t in trajectories]
        self.K, self.B, self.form = window, waves, form
        self.rng = np.random.default_rng(seed)
        n = crystals[0].n
        dev = crystals[0].trans_fine.device
        self.loss_buf = torch.zeros(1, dtype=torch.float32, device=dev)
        self.n = n

    def step(self, lr, windows=2):
        """One Adam step on `windows` random rollout windows; returns the loss, the mean
        over windows and steps of the squared relative wave error."""
        net, K, B = self.net, self.K, self.B
        picks = []
        for _ in range(windows):
            c = int(self.rng.integers(len(self.crystals)))
            cr, tr = self.crystals[c], self.traj[c]
            k0 = int(self.rng.integers(0, tr.shape[0] - K))
            bi = self.rng.choice(tr.shape[1], size=min(B, tr.shape[1]), replace=False)
            b = torch.as_tensor(bi, device=tr.device)
            picks.append((cr, tr, k0, b, self.norms[c][:, bi].sum(1)))
        feats = torch.cat([cr.features()[k0:k0 + K] for cr, tr, k0, b, nrm in picks]).contiguous()
        maps = net.forward(feats)
        dmaps = torch.zeros_like(maps)
        total = 0.0
        for w, (cr, tr, k0, b, nrm) in enumerate(picks):
            total += self._window(cr, tr, k0, b, maps[w * K:(w + 1) * K], dmaps[w * K:(w + 1) * K], nrm)
        net.backward(dmaps)
        net.adam(lr=lr)
        return total / windows

    def _window(self, cr, tr, k0, b, maps, dmaps, norms=None):
        """Rollout of K corrected steps from the fine wave at coarse depth k0 (waves b);
        writes d loss / d maps into dmaps and returns the loss, the mean over steps of
        |psi_k - f_k|^2 / |f_k|^2."""
        K, n, form = self.K, self.n, self.form
        psi = tr[k0][b].contiguous()
        nb = psi.shape[0]
        tb = torch.empty((K, n, n), dtype=torch.complex64, device=psi.device)
        w_in = torch.empty((K, nb, n, n), dtype=torch.complex64, device=psi.device)   # t_k psi_k
        u = torch.empty_like(w_in)                                                      # before (1 + A)
        adj = torch.zeros((K + 1, nb, n, n), dtype=torch.complex64, device=psi.device)  # loss adjoints
        loss = 0.0
        for k in range(K):
            s = k0 + k
            engine.map_trans(cr.trans_coarse[s], maps[k], 1, out=tb[k], form=form)
            w_in[k].copy_(psi)
            engine.mul_plane(w_in[k], cr.trans_coarse[s])
            cr.plan.step_waves(psi, tb[k], cr.ptab_coarse)
            u[k].copy_(psi)
            engine.apply_map(psi, maps[k], 0, form=form)
            target = tr[s + 1][b].contiguous()
            if norms is None:
                engine.residual(torch.zeros_like(target), target, 1.0, adj[k + 1], self.loss_buf)
                denom = float(self.loss_buf.item())
            else:
                denom = float(norms[s + 1])
            engine.residual(psi, target, 1.0 / (K * denom), adj[k + 1], self.loss_buf)
            loss += float(self.loss_buf.item())
        g = adj[K].clone()
        for k in range(K - 1, -1, -1):
            engine.map_grad(u[k], g, 0, dmaps[k], form=form, maps=maps[k])
            engine.apply_map(g, maps[k], 0, conj=True, form=form)
            cr.plan.step_waves(g, cr.ones, cr.ptab_coarse_adj)
            engine.map_grad(w_in[k], g, 1, dmaps[k], accumulate=True, form=form, maps=maps[k])
            engine.mul_plane(g, tb[k], conj=True)
            if k > 0:
                g += adj[k]
        return loss


def training_crystals(n=256, seed=0, random_count=6, thickness=1000.0):
    """Si [001], SrTiO3 [001] and seeded random cubic crystals on an n x n grid."""
    rng = np.random.default_rng(seed)
    cells = max(1, int(round(n * 0.085 / 5.431)))
    out = [('Si[001]', structures.silicon((cells, cells, int(math.ceil(thickness / 5.431)))), 5.431 / 4, 5.431)]
    cs = max(1, int(round(n * 0.085 / 3.905)))
    out.append(('SrTiO3[001]', structures.srtio3((cs, cs, int(math.ceil(thickness / 3.905)))), 3.905 / 2, 3.905))
    for i in range(random_count):
        basis, species, a = structures.random_cubic(rng)
        m = max(1, int(round(n * 0.1 / a)))
        nz = int(math.ceil(thickness / a))
        out.append((f'random{i}', structures.tile(basis, species, (m, m, nz), a), float(rng.uniform(1.0, 2.0)), a))
    return out


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
