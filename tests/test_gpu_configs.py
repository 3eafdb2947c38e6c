"""The uneven-batch and precision-study workloads at their stated sizes, against
the FP64 oracle.

* Uneven batch: seeded random cubic crystals on 256^2, 384^2, 512^2 and 768^2
  grids at 200-300 keV, 50-500 Angstrom thick with 1-2 Angstrom slices, run in
  one graph-captured batch; two positions of every job against the FP64 oracle
  (relative L2 <= 1e-4: FP32 rounding grows with the slice count, about 2e-7 per
  slice, and these jobs run up to ~400 slices) and every job against its own
  plan call.
* Precision study: SrTiO3 [001], 64 x 64 cells (250 Angstrom), 400 Angstrom
  thick at a/2 (206 slices: the crystal is tiled face-inclusive to 103 cells), 300 keV, 25 mrad, on the 1024^2 grid with the FP32
  engine (<= 1e-4 against FP64 on 2 positions) and on a 512^2 sub-run (32 x 32
  cells) with every per-slice DFT on the split-BF16 tensor cores (<= 1e-3, the
  CBED bar).
"""
import numpy as np
import pytest
import torch

from namsa_gb300 import corrector as CR, engine, structures, workloads
from oracle import msa_oracle as O

pytestmark = pytest.mark.gpu
A_STO = 3.905


def _oracle_geom(n, sim):
    g = O.Geometry.__new__(O.Geometry)
    g.sampling, g.kmax, g.lam = np.array([n, n]), float(sim.kmax), float(sim.Lambda)
    return g


def test_uneven_batch_at_stated_grid_sizes_vs_fp64():
    torch.cuda.set_device(0)
    dev = torch.device('cuda', 0)
    rng = np.random.default_rng(2024)
    specs = []
    for n, thick in [(768, (50., 90.)), (512, (150., 260.)), (384, (300., 500.)), (256, (50., 500.)),
                     (512, (50., 120.))]:
        specs.append(workloads.random_crystal(rng, grids=(n,), thickness=thick, voltages=(200, 300),
                                              probes=(16, 48)))
    sims, jobs = [], []
    for s in specs:
        sim, job = workloads.prepare(s, dev)
        sims.append(sim)
        jobs.append(job)
    assert {j['trans'].shape[1] for j in jobs} == {256, 384, 512, 768}
    batch = engine.Batch(branches=4)
    outs = [o.clone() for o in batch.run(jobs)]
    torch.cuda.synchronize()
    batch.check()
    for spec, sim, j, o in zip(specs, sims, jobs, outs):
        n = j['trans'].shape[1]
        plan = engine.Plan(n, n)
        single = plan.multislice(j['trans'], j['psik'], j['norm'], j['positions'], j['kmax'], j['lam'],
                                 j['slice_t'], j['k_band'])
        torch.cuda.synchronize()
        plan.close()
        err1 = (torch.linalg.vector_norm((o - single).double()) / torch.linalg.vector_norm(single.double())).item()
        assert err1 < 1e-5, (n, err1)
        g = _oracle_geom(n, sim)
        P, _ = O.propagator_gpu(g, j['slice_t'], 1 / 3)
        pick = [0, j['positions'].shape[0] - 1]
        ref = O.multislice_gpu(j['trans'].cpu().numpy().astype(np.complex128),
                               j['psik'].cpu().numpy().astype(np.complex128), P,
                               j['positions'].cpu().numpy()[pick], float(j['norm'].item()), g)
        err = O.rel_l2(o.cpu().numpy()[pick], ref)
        assert err.max() < 1e-4, (n, spec['kv'], j['trans'].shape[0], err)
    batch.close()
    for s in sims:
        s.close()


@pytest.fixture(scope='module')
def srtio3_1024():
    torch.cuda.set_device(0)
    sc = structures.srtio3((64, 64, int(np.ceil(400 / A_STO))))
    cr = CR.Crystal(sc, 1024, A_STO / 2, kv=300, semi_angle=25e-3, ratio=1)
    yield sc, cr


def test_precision_study_fp32_1024_vs_fp64(srtio3_1024):
    sc, cr = srtio3_1024
    assert cr.trans_fine.shape == (206, 1024, 1024)
    pos = np.array([[0.3, 1.1], [2.9, 3.4]], np.float32)
    got = CR.fine_multislice(cr, pos).cpu().numpy()
    xyz = np.column_stack([sc['x'], sc['y'], sc['z']]).astype(np.float32)
    geom = O.Geometry(xyz, sc['atomic_number'], 300., 25e-3, [1024, 1024])
    P, _ = O.propagator_gpu(geom, A_STO / 2, 1 / 3)
    psik, _, norm = O.probe_gpu(geom, CR.PROBE)
    ref = O.multislice_gpu(cr.trans_fine.cpu().numpy().astype(np.complex128), psik, P, pos, norm, geom)
    err = O.rel_l2(got, ref)
    assert err.max() < 1e-4, err


def test_precision_study_split_bf16_512_subrun_vs_fp64():
    torch.cuda.set_device(0)
    sc = structures.srtio3((32, 32, int(np.ceil(400 / A_STO))))
    cr = CR.Crystal(sc, 512, A_STO / 2, kv=300, semi_angle=25e-3, ratio=1)
    pos = np.array([[0.3, 1.1], [2.9, 3.4]], np.float32)
    w = cr.waves(pos)
    for s in range(cr.trans_fine.shape[0]):
        engine.step_waves_tc(w, cr.trans_fine[s], cr.ptab_fine)
    got = cr.plan.cbed_waves(w, cr.sim.norm_dev).cpu().numpy()
    engine.tc_check()
    xyz = np.column_stack([sc['x'], sc['y'], sc['z']]).astype(np.float32)
    geom = O.Geometry(xyz, sc['atomic_number'], 300., 25e-3, [512, 512])
    P, _ = O.propagator_gpu(geom, A_STO / 2, 1 / 3)
    psik, _, norm = O.probe_gpu(geom, CR.PROBE)
    ref = O.multislice_gpu(cr.trans_fine.cpu().numpy().astype(np.complex128), psik, P, pos, norm, geom)
    err = O.rel_l2(got, ref)
    assert cr.trans_fine.shape[0] == 206
    assert err.max() < 1e-3, err
