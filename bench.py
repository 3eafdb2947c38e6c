#!/usr/bin/env python
"""STEM/CBED multislice benchmark: probe positions per second.

Workload (one step): the batched STEM scan of a Si [001] supercell, 8x8 lateral
cells (43.4 Angstrom) and 50 cells thick (199 slices of a/4 -- the reference's
float32 floor of 271.55/1.35775), 512x512 complex64 grid, 200 keV, 30 mrad,
Cs = 1 um, 32x32 probe positions on a uniform grid over one unit cell, all 1024
patterns in one call, each stored as the central 256x256 float32 crop.  The
potential slices and the probe are built once (their build time is reported
separately); a step is probe formation -> 199 slices -> CBED for all 1024
positions.  Inputs are synthetic only in the sense that the crystal is
generated, not read from a CIF file.

`value` is timed on device-resident inputs; `e2e` times the same call through
the C ABI with pinned host buffers (transmission stack, probe, positions in;
CBED stack out) copied inside the timed region.  Under torchrun each rank is
an independent replica scanning its own 1024 positions (weak scaling, no
collective on the data path; barriers only for timing).

`--impl reference` times the reference's CPU algorithm (the oracle's port of
namsa's MSA.multislice process pool, complex64 NumPy FFTs) on the host cores.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = 'STEM probe-positions/sec at ≤1e-3 CBED rel. error vs FP64; learned vs plain'
UNIT = 'probe-positions/s'
A_SI = 5.431
WORKLOAD = 'Si[001] 8x8x50 cells, 512x512 c64, 199 slices (t=a/4), 200 keV, 30 mrad, Cs=1um, 32x32 positions, crop 256'
# DRAM bytes (read + write) per launch of a band-limited pass, from the ncu --set full
# captures summarised in profiles/row_col_tma_passes_si512_g512.md, keyed by (pass,
# line length, schedule index, waves per launch); other keys report null.
NCU_TRAFFIC = {
    ('row', 512, 5, 512): 1.076697e9 + 0.684955e9,   # row_pass_tma_kernel t32_r16x2x16
    ('row', 512, 6, 512): 1.076570e9 + 0.684825e9,   # row_pass_tma_kernel t32_r16x2x16_pair
    ('col', 512, 0, 512): 0.771863e9 + 0.682320e9,   # col_mid_tma_kernel t16_r32x16
}


def parse():
    p = argparse.ArgumentParser()
    p.add_argument('--gpus', type=int, default=1)
    p.add_argument('--steps', type=int, default=5)
    p.add_argument('--warmup', type=int, default=3)
    p.add_argument('--impl', default='ours', choices=['ours', 'reference'])
    p.add_argument('--group', type=int, default=0, help='waves per resident group (0 = library default)')
    p.add_argument('--row-sched', type=int, default=-1)
    p.add_argument('--col-sched', type=int, default=-1)
    p.add_argument('--no-e2e', action='store_true')
    p.add_argument('--no-cpu-baseline', action='store_true')
    p.add_argument('--cpu-sample', type=int, default=0, help='probes per CPU-baseline sample (0 = number of cores)')
    p.add_argument('--probes', type=int, default=1024, help='positions per GPU (the first N of the 32x32 scan)')
    p.add_argument('--no-autotune', dest='autotune', action='store_false',
                   help='keep the library default schedule instead of msx_plan_autotune')
    p.add_argument('--no-tma', action='store_true', help='plain one-CTA-per-tile passes instead of the persistent ones')
    p.add_argument('--workload', default='scan', choices=['scan', 'uneven', 'corrector', 'precision'],
                   help='scan: the 512^2 Si [001] 1024-position scan; uneven: 64 seeded random crystals in one batch')
    p.add_argument('--branches', type=int, default=4, help='concurrent graph branches of the uneven batch')
    p.add_argument('--corr-iters', type=int, default=0, help='corrector training iterations (0 = 600 x steps)')
    p.add_argument('--corr-window', type=int, default=16, help='corrected coarse steps per training rollout window')
    p.add_argument('--corr-positions', type=int, default=64, help='held-out positions of the corrector evaluation')
    p.add_argument('--corr-form', type=int, default=1, choices=[0, 1],
                   help='correction factors: 0 = 1 + M, 1 = unit modulus exp(i Im M)')
    return p.parse_args()


def dist_env():
    rank = int(os.environ.get('RANK', 0))
    world = int(os.environ.get('WORLD_SIZE', 1))
    local = int(os.environ.get('LOCAL_RANK', 0))
    return rank, world, local


def scan_positions(rank):
    """32x32 positions (i a/32, j a/32) in [y, x] order over one unit cell; rank r
    scans the cell r cells along x (replicas scan distinct positions)."""
    ii, jj = np.meshgrid(np.arange(32), np.arange(32), indexing='ij')
    return np.column_stack([ii.ravel() * A_SI / 32, jj.ravel() * A_SI / 32 + (rank % 4) * A_SI]).astype(np.float32)


PROBE = {'smooth_apert': True, 'apert_smooth': 50, 'spherical_phase': True,
         'aberration_dict': {'C1': 0., 'C3': 1e4, 'C5': 0.}, 'scherzer': False}


# ----------------------------------------------------------------------------- clocks
class ClockSampler:
    """nvidia-smi samples of SM clock and throttle reasons while running."""
    QUERY = ('index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,'
             'clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,'
             'clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap')

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(['nvidia-smi', '-i', str(self.index), f'--query-gpu={self.QUERY}',
                                          '--format=csv,noheader,nounits', '-lms', '200'],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except (OSError, FileNotFoundError):
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {'sm_mhz': None, 'sm_max_mhz': None, 'reasons': ['nvidia-smi unavailable']}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], None, set()
        names = ['hw_slowdown', 'hw_thermal_slowdown', 'sw_thermal_slowdown', 'sw_power_cap']
        for ln in self.lines:
            f = [x.strip() for x in ln.split(',')]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax = float(f[2])
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower().startswith('active'):
                    reasons.add(n)
        return {'sm_mhz': float(np.median(sm)) if sm else None, 'sm_max_mhz': smax, 'reasons': sorted(reasons),
                'samples': len(sm)}


# ----------------------------------------------------------------------------- CPU legs
def cpu_sample(V, sim, positions, nprobe, procs):
    """Time the oracle's port of the reference CPU path (namsa/msa.py:280-361) on
    `nprobe` positions with `procs` processes; returns (probes/s, seconds)."""
    from oracle import msa_oracle as O
    geom = O.Geometry.__new__(O.Geometry)
    geom.__dict__.update(dict(sampling=np.asarray(sim.sampling), kmax=float(sim.kmax), lam=float(sim.Lambda),
                              semi_ang=float(sim.semi_ang), sigma=float(sim.sigma), dims=sim.dims,
                              pix_size=sim.pix_size))
    t0 = time.perf_counter()
    O.cbed_cpu_pool(V, geom, PROBE, sim.slice_t, 1 / 3, positions[:nprobe], procs)
    dt = time.perf_counter() - t0
    return nprobe / dt, dt


def build_workload(device_index, need_potential):
    import torch
    from namsa_gb300 import msa as M
    from namsa_gb300 import structures
    sc = structures.silicon((8, 8, 50))
    sim = M.MSAGPU(200, 30e-3, sc, sampling=np.array([512, 512]), debye_waller=False)
    sim.setup_device(device_index)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    sim.calc_atomic_potentials()
    sim.build_potential_slices(A_SI / 4, keep_potential=need_potential)
    sim.build_probe(PROBE)
    torch.cuda.synchronize()
    build_ms = (time.perf_counter() - t0) * 1e3
    return sim, build_ms


def run_reference(args):
    rank, world, local = dist_env()
    if rank != 0:
        return
    import multiprocessing as mp
    procs = mp.cpu_count()
    nprobe = args.cpu_sample or procs
    # potential slices from the oracle itself (no GPU on this leg)
    from oracle import msa_oracle as O
    from namsa_gb300 import structures
    sc = structures.silicon((8, 8, 50))
    geom = O.Geometry(np.column_stack([sc['x'], sc['y'], sc['z']]), sc['atomic_number'], 200., 30e-3, [512, 512])
    _, win = O.atom_windows(geom, np.load(os.path.join(ROOT, 'namsa_gb300', 'data', 'kirkland_params.npy')))
    V = O.potential_slices_cpu(geom, win, A_SI / 4)

    class S:  # the fields cpu_sample reads
        pass
    sim = S()
    sim.sampling, sim.kmax, sim.Lambda, sim.semi_ang = geom.sampling, geom.kmax, geom.lam, 30e-3
    sim.sigma, sim.dims, sim.pix_size, sim.slice_t = geom.sigma, geom.dims, geom.pix_size, A_SI / 4
    pos = scan_positions(0)
    for _ in range(args.warmup):
        cpu_sample(V, sim, pos, nprobe, procs)
    times = []
    for _ in range(args.steps):
        _, dt = cpu_sample(V, sim, pos, nprobe, procs)
        times.append(dt)
    ms = 1e3 * float(np.mean(times))
    value = nprobe / (ms / 1e3)
    line = {'metric': METRIC, 'value': value, 'unit': UNIT, 'n_gpus': args.gpus, 'steps': args.steps,
            'warmup': args.warmup, 'ms_per_step': ms, 'higher_is_better': True, 'scaling': 'weak',
            'vs_baseline': None, 'dtype': 'c64', 'data': 'synthetic (generated Si supercell)',
            'config': {'workload': WORKLOAD, 'sample_probes_per_step': nprobe, 'slices': V.shape[0]},
            'impl': 'reference',
            'cpu_baseline': {'value': value, 'unit': UNIT, 'cores': procs, 'kind': 'port',
                             'sample': f'{nprobe} of the 1024 positions per step, 199 slices, 512^2, '
                                       f'process pool of {procs} (reference CPU MSA path restated in oracle/)'},
            'e2e': {'value': value, 'unit': UNIT, 'h2d_bytes_per_step': 0, 'd2h_bytes_per_step': 0}}
    line['reference_gpu'] = reference_gpu_leg(args)
    print(json.dumps(line), flush=True)


def reference_gpu_leg(args):
    """The reference's own GPU path on this GPU: its rendered kernels and cuFFT in
    MSAGPU.multislice's order (oracle/refgpu_harness.cu), on the same 1024-position
    Si 512^2 scan.  `value` times the device work of one multislice call (probe
    stack, 199 x [t/N, FFT, P, IFFT], final FFT and |.|^2) with CUDA events; `call_ms`
    adds what the reference's call also does each time: the batched cuFFT plan,
    the propagator, the D2H copy of the complex stack and the host-side division
    by the normalisation (namsa/msa.py:767-924)."""
    try:
        import torch
        if not torch.cuda.is_available():
            return {'unavailable': 'no GPU on this host'}
        from oracle import msa_oracle as O
        from oracle import refgpu as R
        ref = R.RefGPU('c2')
    except Exception as e:  # harness not rendered/built here
        return {'unavailable': f'reference GPU harness not available: {e}'.splitlines()[0]}
    torch.cuda.set_device(0)
    meta = ref.meta
    sc = O.si_supercell(*meta['cells'])
    geom = O.Geometry(np.column_stack([sc['x'], sc['y'], sc['z']]), sc['atomic_number'], meta['kv'], meta['semi'],
                      [512, 512])
    _, win = O.atom_windows(geom, np.load(os.path.join(ROOT, 'namsa_gb300', 'data', 'kirkland_params.npy')))
    trans = ref.build_potential(geom, meta['slice_t'], win)
    kmax = np.float32(geom.kmax)
    ab = PROBE['aberration_dict']
    psik, _, _, norm = ref.build_probe(kmax, np.float32(geom.semi_ang / geom.lam), geom.lam, ab['C1'], ab['C3'],
                                       ab['C5'], PROBE['smooth_apert'])
    pos = torch.from_numpy(scan_positions(0)).cuda()
    P = int(pos.shape[0])
    psi = torch.empty((P, 512, 512), dtype=torch.complex64, device='cuda')
    host = torch.empty((P, 512, 512), dtype=torch.complex64, pin_memory=True)
    ctx = ref.context(P)
    try:
        ref.propagator(ctx, kmax, np.float32(geom.kmax / 3), meta['slice_t'], geom.lam)
        for _ in range(max(1, args.warmup)):
            ref.propagate(ctx, trans, psik, pos, kmax, psi)
        st = torch.cuda.current_stream()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record(st)
        for _ in range(args.steps):
            ref.propagate(ctx, trans, psik, pos, kmax, psi)
        e1.record(st)
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / args.steps
    finally:
        ref.destroy(ctx)
    # one whole call as the reference makes it (plan, propagator, beams, D2H, host scaling)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    ctx = ref.context(P)
    try:
        ref.propagator(ctx, kmax, np.float32(geom.kmax / 3), meta['slice_t'], geom.lam)
        ref.propagate(ctx, trans, psik, pos, kmax, psi)
        host.copy_(psi)
        out = (host.numpy() / norm).real.astype(np.float32)
    finally:
        ref.destroy(ctx)
    call_ms = (time.perf_counter() - t0) * 1e3
    del out
    return {'value': P / (ms / 1e3), 'unit': UNIT, 'ms_per_step': ms, 'call_ms': call_ms,
            'call_value': P / (call_ms / 1e3), 'positions': P, 'slices': int(trans.shape[0]),
            'kind': 'reference kernels (rendered from namsa/probe_kernels.cu, potential_kernels.cu) + cuFFT, '
                    'MSAGPU call order, one batch of 1024'}


def run_ours(args):
    import torch
    import torch.distributed as dist
    from namsa_gb300 import engine

    rank, world, local = dist_env()
    torch.cuda.set_device(local)  # before the process group, so NCCL binds this rank's GPU
    dev = torch.device('cuda', local)
    if world > 1:
        dist.init_process_group('nccl', init_method='env://')
    want_cpu = (rank == 0 and world == 1 and not args.no_cpu_baseline)

    sim, build_ms = build_workload(local, need_potential=want_cpu)
    pos_np = scan_positions(rank)[:args.probes]
    P = len(pos_np)
    pos = torch.from_numpy(pos_np).to(dev)
    kmax32 = np.float32(sim.kmax)
    kband = np.float32(sim.kmax / 3)
    plan = engine.Plan(512, 512, args.group)
    plan.set_tma(not args.no_tma)
    r, c, g = plan.schedule
    plan.set_schedule(r if args.row_sched < 0 else args.row_sched, c if args.col_sched < 0 else args.col_sched)
    tuned = None
    if args.autotune:
        sched, ns = plan.autotune(sim.trans, sim.psi_k_dev, sim.norm_dev, pos, kmax32, sim.Lambda, sim.slice_t, kband)
        tuned = {'row': engine.schedules(512)[sched[0]], 'col': engine.schedules(512)[sched[1]], 'group': sched[2],
                 'ns_per_wave_slice': ns}
    crop = 256
    out = torch.empty((P, crop, crop), dtype=torch.float32, device=dev)

    def step(o=out):
        plan.multislice(sim.trans, sim.psi_k_dev, sim.norm_dev, pos, kmax32, sim.Lambda, sim.slice_t, kband,
                        crop=crop, out=o)

    for _ in range(max(args.warmup, 3)):
        step()
    torch.cuda.synchronize()
    if world > 1:
        dist.barrier()
    clocks = ClockSampler(local)
    clocks.start()
    time.sleep(0.3)
    st = torch.cuda.current_stream()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    if world > 1:
        dist.barrier()
    e0.record(st)
    for _ in range(args.steps):
        step()
    e1.record(st)
    torch.cuda.synchronize()
    if world > 1:
        dist.barrier()
    clk = clocks.stop()
    ms = e0.elapsed_time(e1) / args.steps
    t = torch.tensor([ms], dtype=torch.float64, device=dev)
    if world > 1:
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
    ms_max = float(t.item())
    value = world * P / (ms_max / 1e3)

    # ---- end to end through the C ABI with pinned host buffers
    e2e = None
    if not args.no_e2e:
        h_trans = sim.trans.cpu().pin_memory()
        h_psik = sim.psi_k_dev.cpu().pin_memory()
        h_pos = torch.from_numpy(pos_np).pin_memory()
        h_out = torch.empty((P, crop, crop), dtype=torch.float32).pin_memory()
        norm_value = float(sim.norm_dev.item())

        def e2e_step():
            # the host-buffer entry point: chunked slice uploads overlap the first group,
            # each group's patterns are downloaded while the next one computes
            plan.multislice_host(h_trans, h_psik, norm_value, h_pos, kmax32, sim.Lambda, sim.slice_t, kband,
                                 crop=crop, out=h_out)
        for _ in range(2):
            e2e_step()
        torch.cuda.synchronize()
        if world > 1:
            dist.barrier()
        e0.record(st)
        for _ in range(args.steps):
            e2e_step()
        e1.record(st)
        torch.cuda.synchronize()
        t2 = torch.tensor([e0.elapsed_time(e1) / args.steps], dtype=torch.float64, device=dev)
        if world > 1:
            dist.all_reduce(t2, op=dist.ReduceOp.MAX)
        bi = h_trans.numel() * 8 + h_psik.numel() * 8 + h_pos.numel() * 4
        bo = h_out.numel() * 4
        e2e = {'value': world * P / (float(t2.item()) / 1e3), 'unit': UNIT, 'h2d_bytes_per_step': int(bi),
               'd2h_bytes_per_step': int(bo), 'ms_per_step': float(t2.item())}
        del h_trans

    # ---- dominant pass timing and roofline
    row_ms, col_ms, gw = plan.profile(sim.trans, sim.psi_k_dev, sim.norm_dev, pos, kmax32, sim.Lambda, sim.slice_t,
                                      kband, iters=40)
    N = 512 * 512
    dom = 'row' if row_ms >= col_ms else 'col'
    dom_ms = max(row_ms, col_ms)
    # From the second slice on the passes keep only the column tiles [lo, hi) that
    # the bandwidth mask can reach (a fraction fb of the columns): the row pass reads
    # whole rows and writes that range, the column pass reads and writes that range.
    lo, hi = engine.band_columns(512, kmax32, kband, engine.col_tile(512, plan.schedule[1]))
    fb = (hi - lo) / 512.0
    row_bytes = 8.0 * N * gw * (1.0 + fb) + 8.0 * N
    col_bytes = 16.0 * N * gw * fb + 8.0 * 512
    alg_bytes = row_bytes if dom == 'row' else col_bytes
    line_flops = (10.0 * N * math.log2(512) + 15.0 * N) * gw  # both transforms of every line of one pass
    alg_flops = line_flops if dom == 'row' else line_flops * fb
    peaks = {}
    pk_path = os.path.join(ROOT, 'MEASURED_PEAKS.json')
    if os.path.exists(pk_path):
        peaks = json.load(open(pk_path))
    hbm_peak = peaks.get('hbm_gbs')
    peak_src = 'measured' if hbm_peak else 'fallback'
    hbm_peak = hbm_peak or 6800.0
    achieved = alg_bytes / (dom_ms / 1e3) / 1e9
    sm_clock = (clk.get('sm_mhz') or 1900.0)
    sm_count = torch.cuda.get_device_properties(torch.cuda.current_device()).multi_processor_count
    fp32_peak = sm_count * 128 * 2 * sm_clock * 1e6 / 1e12
    roof = {'bound': 'hbm', 'achieved': achieved, 'peak': hbm_peak, 'unit': 'GB/s', 'frac': achieved / hbm_peak,
            'traffic': NCU_TRAFFIC.get((dom, 512, plan.schedule[0] if dom == 'row' else plan.schedule[1], gw)),
            'kernel': f'{dom}_pass_kernel (512, {gw} waves per launch)', 'peak_source': f'{peak_src} hbm_gbs',
            'band_columns': [lo, hi], 'algorithmic_bytes_per_launch': alg_bytes,
            'launch_ms': dom_ms, 'row_pass_ms': row_ms, 'col_pass_ms': col_ms,
            'fp32': {'achieved_tflops': alg_flops / (dom_ms / 1e3) / 1e12, 'peak_tflops': fp32_peak,
                     'frac': alg_flops / (dom_ms / 1e3) / 1e12 / fp32_peak,
                     'peak_source': f'nominal {sm_count} SM x 128 FP32 lanes x 2 at the sampled {sm_clock:.0f} MHz'}}

    groups = math.ceil(P / plan.schedule[2])
    launches = args.steps * (1 + groups * (1 + 2 * sim.num_slices))
    line = {'metric': METRIC, 'value': value, 'unit': UNIT, 'n_gpus': world, 'steps': args.steps,
            'warmup': args.warmup, 'ms_per_step': ms_max, 'higher_is_better': True, 'scaling': 'weak',
            'vs_baseline': None, 'dtype': 'c64',
            'data': 'synthetic (generated Si supercell; inputs resident in HBM for value, pinned host for e2e)',
            'config': {'workload': WORKLOAD, 'global_batch': world * P, 'probes_per_gpu': P,
                       'grid': [512, 512], 'slices': int(sim.num_slices), 'crop': crop,
                       'parallelism': f'replicas x{world}' if world > 1 else 'single GPU',
                       'l2': 'inputs larger than L2 (transmission stack 398 MiB, CBED out 256 MiB)',
                       'schedule': {'row': engine.schedules(512)[plan.schedule[0]],
                                    'col': engine.schedules(512)[plan.schedule[1]], 'group': plan.schedule[2]},
                       'potential_and_probe_build_ms': build_ms, 'autotuned': tuned,
                       'passes': 'plain' if args.no_tma else 'persistent TMA-pipelined'},
            'gpu_launches': int(launches), 'clocks': clk, 'e2e': e2e, 'roofline': roof}

    if want_cpu:
        import multiprocessing as mp
        procs = mp.cpu_count()
        nprobe = args.cpu_sample or procs
        V = sim.potential.cpu().numpy()
        v, dt = cpu_sample(V, sim, pos_np, nprobe, procs)
        line['cpu_baseline'] = {'value': v, 'unit': UNIT, 'cores': procs, 'kind': 'port',
                                'sample': f'{nprobe} of the 1024 positions, 199 slices, 512^2, {dt:.1f} s wall, '
                                          f'reference CPU MSA path (oracle port), process pool of {procs}'}
    if rank == 0:
        print(json.dumps(line), flush=True)
    plan.close()
    if world > 1:
        dist.destroy_process_group()


def uneven_breakdown(jobs, batch_ms, reps=3):
    """Per grid size: the batch's jobs run one at a time through an autotuned plan of
    that size (the standalone time of each job), and the same probe-slices at the rate
    of a homogeneous 512-position run of that size (the matched homogeneous time)."""
    import torch
    from namsa_gb300 import engine
    st = torch.cuda.current_stream()
    out = {}
    for n in sorted({j['trans'].shape[1] for j in jobs}):
        js = [j for j in jobs if j['trans'].shape[1] == n]
        big = max(js, key=lambda j: j['positions'].shape[0])
        plan = engine.Plan(n, n)
        plan.autotune(big['trans'], big['psik'], big['norm'], big['positions'], big['kmax'], big['lam'],
                      big['slice_t'], big['k_band'])

        def timed_ms(fn):
            fn()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(st)
            for _ in range(reps):
                fn()
            e1.record(st)
            torch.cuda.synchronize()
            return e0.elapsed_time(e1) / reps
        alone = 0.0
        pslices = 0
        for j in js:
            alone += timed_ms(lambda j=j: plan.multislice(j['trans'], j['psik'], j['norm'], j['positions'], j['kmax'],
                                                          j['lam'], j['slice_t'], j['k_band'], out=j['out']))
            pslices += j['positions'].shape[0] * j['trans'].shape[0]
        # homogeneous rate: 512 positions through the first (up to) 32 slices of the largest job
        S = min(32, big['trans'].shape[0])
        pos = big['positions'][torch.arange(512, device=big['positions'].device) % big['positions'].shape[0]]
        pos = (pos + 0.01 * torch.arange(512, device=pos.device, dtype=torch.float32)[:, None]).contiguous()
        plan2 = engine.Plan(n, n)
        plan2.autotune(big['trans'][:S].contiguous(), big['psik'], big['norm'], pos, big['kmax'], big['lam'],
                       big['slice_t'], big['k_band'])
        hom = timed_ms(lambda: plan2.multislice(big['trans'][:S].contiguous(), big['psik'], big['norm'], pos,
                                                big['kmax'], big['lam'], big['slice_t'], big['k_band']))
        ns_ps = hom * 1e6 / (512 * S)
        out[str(n)] = {'jobs': len(js), 'probe_slices': pslices, 'standalone_ms': alone,
                       'homogeneous_ns_per_probe_slice': ns_ps, 'matched_homogeneous_ms': pslices * ns_ps / 1e6}
        plan.close()
        plan2.close()
    tot_alone = sum(v['standalone_ms'] for v in out.values())
    tot_hom = sum(v['matched_homogeneous_ms'] for v in out.values())
    return {'per_grid': out, 'batch_ms': batch_ms, 'sum_standalone_ms': tot_alone, 'sum_matched_homogeneous_ms': tot_hom,
            'batch_rate_vs_standalone': tot_alone / batch_ms, 'batch_rate_vs_matched_homogeneous': tot_hom / batch_ms}


def run_uneven(args):
    """64 seeded random crystals (grids 256..768^2, 50-500 A, 80-300 kV, 16-256
    positions each) in one graph-captured batch; probes/s over the whole batch."""
    import torch
    from namsa_gb300 import engine, workloads
    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    dev = torch.device('cuda', local)
    t0 = time.perf_counter()
    specs, sims, jobs = workloads.random_batch(1234 + rank, count=64, device=dev)
    torch.cuda.synchronize()
    build_s = time.perf_counter() - t0
    batch = engine.Batch(branches=args.branches)
    tuned = None
    if args.autotune:
        t1 = time.perf_counter()
        batch.autotune(jobs)
        torch.cuda.synchronize()
        tuned = time.perf_counter() - t1
    for _ in range(max(args.warmup, 3)):
        batch.run(jobs)
    torch.cuda.synchronize()
    st = torch.cuda.current_stream()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(st)
    for _ in range(args.steps):
        batch.run(jobs)
    e1.record(st)
    torch.cuda.synchronize()
    batch.check()
    ms = e0.elapsed_time(e1) / args.steps
    P = sum(j['positions'].shape[0] for j in jobs)
    ps, psp = workloads.work_units(jobs)
    grids = {}
    for s in specs:
        grids[s['n']] = grids.get(s['n'], 0) + 1
    breakdown = uneven_breakdown(jobs, ms) if args.autotune else None
    line = {'metric': METRIC, 'value': P / (ms / 1e3), 'unit': UNIT, 'n_gpus': 1, 'steps': args.steps,
            'warmup': args.warmup, 'ms_per_step': ms, 'higher_is_better': True, 'scaling': 'weak',
            'vs_baseline': None, 'dtype': 'c64', 'data': 'synthetic (64 seeded random cubic crystals)',
            'config': {'workload': 'uneven batch of 64 random crystals, one CUDA graph', 'probes': P,
                       'probe_slices': ps, 'probe_slice_pixels_per_s': psp / (ms / 1e3),
                       'grids': grids, 'branches': args.branches, 'build_s': build_s,
                       'autotune_s': tuned, 'breakdown': breakdown}}
    print(json.dumps(line), flush=True)
    batch.close()


def run_corrector(args):
    """Learned coarse-slice corrector (256^2, 200 keV, 4x-thick slices): train it by
    windowed rollouts on device-generated fine-slice trajectories of Si [001],
    SrTiO3 [001] and seeded random crystals about 1000 A thick, then compare, on
    held-out positions, plain coarse slicing and the corrected coarse slicing
    (production multislice on the effective transmission slices) with plain
    fine slicing (the error reference): CBED error at 200, 500 and 1000 A and
    probe-positions/s of each form."""
    import torch
    from namsa_gb300 import corrector as CR, engine
    torch.cuda.set_device(0)
    n, C, L = 256, 32, 4
    t0 = time.perf_counter()
    specs = CR.training_crystals(n, seed=0, random_count=4, thickness=1000.0)
    crystals, trajs = [], []
    rng = np.random.default_rng(1)
    for name, sites, t, a in specs:
        cr = CR.Crystal(sites, n, t)
        crystals.append((name, cr, a))
        trajs.append(cr.trajectory(rng.uniform(0, a, size=(22, 2))))
    torch.cuda.synchronize()
    gen_s = time.perf_counter() - t0
    pairs = int(sum((tr.shape[0] - 1) * tr.shape[1] for tr in trajs))
    net = engine.Corrector(n, n, 6, C, L, 32, 64, max_samples=max(16, 2 * args.corr_window))
    net.params.copy_(torch.from_numpy(CR.init_params(net, seed=0)))
    trainer = CR.RolloutTrainer(net, [c for _, c, _ in crystals], trajs, window=args.corr_window, waves=8, seed=0,
                                form=args.corr_form)
    iters = args.corr_iters if args.corr_iters > 0 else max(1, args.steps) * 600
    t1 = time.perf_counter()
    losses = [trainer.step(lr=2e-3 * 0.5 * (1 + math.cos(math.pi * i / iters))) for i in range(iters)]
    torch.cuda.synchronize()
    train_s = time.perf_counter() - t1
    net.check()
    res = {}
    for name, cr, a in crystals[:3]:  # Si [001], SrTiO3 [001] and the first random crystal
        pos = np.random.default_rng(7).uniform(0, a, size=(args.corr_positions, 2))
        maps, net_s = CR.timed(lambda: CR.crystal_maps(net, cr))
        maps_every, net_every_s = CR.timed(lambda: CR.crystal_maps(net, cr, dedup=False))
        distinct = len(CR.distinct_slices(cr.features())[0])
        out = {'network_s_per_crystal': net_s, 'network_s_every_slice': net_every_s,
               'distinct_slices': distinct, 'maps_equal_every_slice': bool(torch.equal(maps, maps_every)),
               'coarse_slices': int(cr.coarse_steps)}
        for thick in (200.0, 500.0, 1000.0):
            steps = min(cr.coarse_steps, int(round(thick / (cr.ratio * cr.slice_t))))
            trans = cr.effective_slices(maps[:steps].contiguous(), args.corr_form)
            ref, t_fine = CR.timed(lambda: CR.fine_multislice(cr, pos, steps))
            coarse, t_coarse = CR.timed(lambda: CR.coarse_multislice(cr, pos, steps))
            corr, t_corr = CR.timed(lambda: CR.corrected_multislice(net, cr, pos, steps, trans=trans))
            out[f'{thick:.0f}A'] = {
                'thickness_A': steps * cr.ratio * cr.slice_t, 'positions': len(pos),
                'err_coarse_vs_fine': float(CR.rel_l2(coarse, ref).mean()),
                'err_corrected_vs_fine': float(CR.rel_l2(corr, ref).mean()),
                'intensity_coarse_over_fine': float((coarse.double().sum() / ref.double().sum()).item()),
                'intensity_corrected_over_fine': float((corr.double().sum() / ref.double().sum()).item()),
                'fine_probes_per_s': len(pos) / t_fine, 'coarse_probes_per_s': len(pos) / t_coarse,
                'corrected_probes_per_s': len(pos) / t_corr,
                'speedup_corrected_vs_fine': t_fine / t_corr,
                'speedup_incl_network_per_1024_positions': (t_fine * 1024 / len(pos)) /
                                                           (t_corr * 1024 / len(pos) +
                                                            net_s * steps / cr.coarse_steps),
                'speedup_incl_network_every_slice_per_1024_positions': (t_fine * 1024 / len(pos)) /
                                                                      (t_corr * 1024 / len(pos) +
                                                                       net_every_s * steps / cr.coarse_steps)}
        res[name] = out
    si = res['Si[001]']['1000A']
    line = {'metric': METRIC, 'value': si['corrected_probes_per_s'], 'unit': UNIT, 'n_gpus': 1,
            'steps': args.steps, 'warmup': 0, 'higher_is_better': True, 'scaling': 'weak', 'vs_baseline': None,
            'dtype': 'c64 multislice, bf16 network (fp32 accumulation)',
            'data': 'synthetic (device-generated fine-slice trajectories)',
            'config': {'workload': 'learned coarse-slice corrector, 256^2, 200 keV, 4x slices', 'pairs': pairs,
                       'generate_s': gen_s, 'train_s': train_s, 'train_iters': iters,
                       'loss_first': float(np.mean(losses[:10])), 'loss_last': float(np.mean(losses[-50:])),
                       'window': args.corr_window, 'map_form': ['1 + M', 'exp(i Im M)'][args.corr_form],
                       'channels': C, 'layers': L, 'modes': '32 x 64 (kx x ky)', 'results': res}}
    print(json.dumps(line), flush=True)
    net.close()


def run_precision(args):
    """SrTiO3 [001], 400 A thick, t = a/2, 300 keV, 25 mrad: CBED error against the
    FP64 oracle of (a) the FP32 FFT engine at 1024^2 (64 cells, 64 positions) and,
    on 512^2 sub-runs (32 cells), (b) the FP32 engine and (c) the split-BF16
    tensor-core DFT stages.  The FP64 oracle runs on the host for a sample of
    positions."""
    import torch
    from namsa_gb300 import corrector as CR, engine, structures
    from oracle import msa_oracle as O
    torch.cuda.set_device(0)
    a = 3.905
    rng = np.random.default_rng(0)
    out = {}
    for n, cells, forms in [(512, 32, ('fp32_fft', 'bf16x3_tensor_core', 'bf16x3_tensor_core_compensated')),
                            (1024, 64, ('fp32_fft',))]:
        sc = structures.srtio3((cells, cells, int(np.ceil(400 / a))))
        cr = CR.Crystal(sc, n, a / 2, kv=300, semi_angle=25e-3, ratio=1)
        pos = rng.uniform(0, a, size=(64, 2)).astype(np.float32)
        sample = np.arange(0, 64, 32) if n == 1024 else np.arange(0, 64, 16)
        xyz = np.column_stack([sc['x'], sc['y'], sc['z']]).astype(np.float32)
        geom = O.Geometry(xyz, sc['atomic_number'], 300., 25e-3, [n, n])
        P, _ = O.propagator_gpu(geom, a / 2, 1 / 3)
        psik, _, norm = O.probe_gpu(geom, CR.PROBE)
        t0 = time.perf_counter()
        ref = O.multislice_gpu(cr.trans_fine.cpu().numpy().astype(np.complex128), psik, P, pos[sample], norm, geom)
        oracle_s = time.perf_counter() - t0
        res = {'slices': int(cr.trans_fine.shape[0]), 'positions': 64, 'oracle_positions': len(sample),
               'oracle_s': oracle_s}
        for form in forms:
            torch.cuda.synchronize()
            t1 = time.perf_counter()
            if form == 'fp32_fft':
                got = CR.fine_multislice(cr, pos)
            else:
                engine.tc_set_compensation(form.endswith('compensated'))
                w = cr.waves(pos)
                for s in range(cr.trans_fine.shape[0]):
                    engine.step_waves_tc(w, cr.trans_fine[s], cr.ptab_fine)
                got = cr.plan.cbed_waves(w, cr.sim.norm_dev)
                engine.tc_check()
                engine.tc_set_compensation(True)
            torch.cuda.synchronize()
            dt = time.perf_counter() - t1
            g = got.cpu().numpy()[sample]
            e = O.rel_l2(g, ref)
            # total-intensity ratio: a value below 1 is a systematic loss of norm
            # (rounding towards zero), not random rounding noise
            ratio = g.reshape(len(sample), -1).sum(1) / ref.reshape(len(sample), -1).sum(1)
            res[form] = {'rel_l2_mean': float(e.mean()), 'rel_l2_max': float(e.max()),
                         'max_abs': float(np.abs(g - ref).max()), 'max_ref': float(np.abs(ref).max()),
                         'intensity_ratio': float(ratio.mean()), 'probes_per_s': 64 / dt}
        out[f'{n}x{n}'] = res
    line = {'metric': METRIC, 'value': out['1024x1024']['fp32_fft']['probes_per_s'], 'unit': UNIT, 'n_gpus': 1,
            'steps': 1, 'warmup': 0, 'higher_is_better': True, 'scaling': 'weak', 'vs_baseline': None,
            'dtype': 'c64', 'data': 'synthetic (generated SrTiO3 supercell)',
            'config': {'workload': 'precision study SrTiO3[001] 400 A, 300 keV, 25 mrad', 'results': out}}
    print(json.dumps(line), flush=True)


def main():
    args = parse()
    if args.impl == 'reference':
        run_reference(args)
    elif args.workload == 'uneven':
        run_uneven(args)
    elif args.workload == 'corrector':
        run_corrector(args)
    elif args.workload == 'precision':
        run_precision(args)
    else:
        run_ours(args)


if __name__ == '__main__':
    main()
