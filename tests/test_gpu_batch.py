"""Uneven batches (engine.Batch / msx_batch_run): every job of a mixed list of
crystals gives the same CBED stack as its own msx_multislice call, graph
replays are bit-identical, and one job is checked against the FP64 oracle."""
import numpy as np
import pytest
import torch

from namsa_gb300 import engine, workloads
from oracle import msa_oracle as O

pytestmark = pytest.mark.gpu


def small_batch(seed, count):
    dev = torch.device('cuda', 0)
    torch.cuda.set_device(0)
    return workloads.random_batch(seed, count=count, device=dev, grids=(64, 128, 256), thickness=(8., 30.),
                                  probes=(2, 7))


def test_batch_matches_single_calls_and_replays():
    specs, sims, jobs = small_batch(11, 7)
    batch = engine.Batch(branches=3)
    outs = [o.clone() for o in batch.run(jobs)]
    torch.cuda.synchronize()
    batch.check()
    for j in jobs:
        j['out'].fill_(float('nan'))
    outs2 = batch.run(jobs)  # replay of the captured graph
    torch.cuda.synchronize()
    for a, b in zip(outs, outs2):
        assert torch.equal(a, b)
    for j, o in zip(jobs, outs):
        plan = engine.Plan(j['trans'].shape[1], j['trans'].shape[2])
        ref = plan.multislice(j['trans'], j['psik'], j['norm'], j['positions'], j['kmax'], j['lam'], j['slice_t'],
                              j['k_band'])
        torch.cuda.synchronize()
        assert torch.equal(ref, o)
        plan.close()
    batch.close()


def test_batch_job_vs_fp64_oracle():
    specs, sims, jobs = small_batch(5, 3)
    batch = engine.Batch(branches=2)
    batch.run(jobs)
    torch.cuda.synchronize()
    j, sim = jobs[0], sims[0]
    n = j['trans'].shape[1]
    g = O.Geometry.__new__(O.Geometry)
    g.sampling, g.kmax, g.lam = np.array([n, n]), float(sim.kmax), float(sim.Lambda)
    P, _ = O.propagator_gpu(g, j['slice_t'], 1 / 3)
    ref = O.multislice_gpu(j['trans'].cpu().numpy().astype(np.complex128),
                           j['psik'].cpu().numpy().astype(np.complex128), P, j['positions'].cpu().numpy(),
                           float(j['norm'].item()), g)
    err = O.rel_l2(j['out'].cpu().numpy(), ref)
    assert err.max() < 2e-5, err
    batch.close()


def test_batch_autotune_keeps_results():
    """msx_batch_autotune picks a schedule per grid size; the batch then still
    matches single default-schedule calls to FP32 rounding."""
    specs, sims, jobs = small_batch(17, 6)
    batch = engine.Batch(branches=2)
    batch.autotune(jobs, iters=2)
    outs = [o.clone() for o in batch.run(jobs)]
    torch.cuda.synchronize()
    batch.check()
    for j, o in zip(jobs, outs):
        plan = engine.Plan(j['trans'].shape[1], j['trans'].shape[2])
        ref = plan.multislice(j['trans'], j['psik'], j['norm'], j['positions'], j['kmax'], j['lam'], j['slice_t'],
                              j['k_band'])
        torch.cuda.synchronize()
        err = (torch.linalg.vector_norm((o - ref).double()) / torch.linalg.vector_norm(ref.double())).item()
        assert err < 1e-5, err
        plan.close()
    batch.close()
