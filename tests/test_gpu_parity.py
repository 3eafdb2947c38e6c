"""Parity of the CUDA engine (through the libmsx C ABI) with the oracle.

Tolerances: integer/discrete results (summed potential V, masks) are compared
bit for bit; floating results against the FP64 oracle with the relative L2
bounds stated per test (the bar for the CBED metric is 1e-3 vs FP64; the
FP32 engine is held to 1e-4 or tighter)."""
import numpy as np
import pytest
import torch

from namsa_gb300 import _lib, engine
from namsa_gb300 import msa as M
from oracle import msa_oracle as O

pytestmark = pytest.mark.gpu
DEV = 'cuda'
KIRK = M.kirkland_table()


def geom_of(ny, nx, kmax, lam):
    g = O.Geometry.__new__(O.Geometry)
    g.sampling = np.array([ny, nx])
    g.kmax = kmax
    g.lam = lam
    return g


def crystal_geom(sc, energy, semi, n):
    xyz = np.column_stack([sc['x'], sc['y'], sc['z']]).astype(np.float32)
    return O.Geometry(xyz, sc['atomic_number'], energy, semi, n)


def engine_cbed(trans, psik, norm, pos, kmax, lam, slice_t, bandwidth, crop=None, group=0, sched=(0, 0), graph=True,
                tma=True):
    ny, nx = psik.shape
    plan = engine.Plan(ny, nx, group)
    plan.set_schedule(sched[0], sched[1])
    plan.set_graph(graph)
    plan.set_tma(tma)
    out = plan.multislice(torch.from_numpy(np.ascontiguousarray(trans.astype(np.complex64))).to(DEV),
                          torch.from_numpy(np.ascontiguousarray(psik.astype(np.complex64))).to(DEV),
                          torch.tensor([norm], dtype=torch.float64, device=DEV),
                          torch.from_numpy(np.ascontiguousarray(pos.astype(np.float32))).to(DEV),
                          np.float32(kmax), lam, slice_t, np.float32(bandwidth * kmax), crop=crop)
    res = out.cpu().numpy()
    plan.check()
    plan.close()
    return res


def random_case(ny, nx, S, P, seed, lam=0.025, slice_t=1.5):
    rng = np.random.default_rng(seed)
    kmax = float(min(ny, nx)) / 20.0
    g = geom_of(ny, nx, kmax, lam)
    g.semi_ang = 0.025
    pd = {'smooth_apert': True, 'spherical_phase': True, 'aberration_dict': {'C1': 15., 'C3': 1e4, 'C5': 0.},
          'scherzer': False}
    psik, _, norm = O.probe_gpu(g, pd)
    psik = psik.astype(np.complex64)
    norm = float(np.sum(np.abs(np.fft.ifft2(psik.astype(np.complex128)) * ny * nx) ** 2))
    V = rng.standard_normal((S, ny, nx))
    trans = np.exp(0.3j * V).astype(np.complex64)
    pos = rng.uniform(-8, 8, size=(P, 2)).astype(np.float32)
    return g, trans, psik, norm, pos, kmax, lam, slice_t


def oracle_cbed(g, trans, psik, norm, pos, slice_t, bandwidth, crop=None):
    P, _ = O.propagator_gpu(g, slice_t, bandwidth)
    return O.multislice_gpu(trans.astype(np.complex128), psik.astype(np.complex128), P, pos, norm, g, crop=crop)


# ----------------------------------------------------------------------------- setup kernels
@pytest.mark.parametrize('zs,pix', [((14,), (0.08486, 0.08486)), ((8, 22, 38, 79), (0.061, 0.0732))])
def test_atom_windows(zs, pix):
    n0, n1 = M.window_grid(np.array(pix))
    coeff = torch.from_numpy(np.ascontiguousarray(KIRK[np.array(zs) - 1])).to(DEV)
    w = engine.atom_windows(coeff, n0, n1).cpu().numpy()
    for i, z in enumerate(zs):
        ref = O.atom_potential(KIRK[z - 1], np.array(pix))
        assert w[i].shape == ref.shape
        assert np.abs(w[i] - ref).max() <= 4e-7 * np.abs(ref).max()


@pytest.mark.parametrize('case', ['si_small', 'srtio3_rect'])
def test_transmission_bit_exact(case):
    if case == 'si_small':
        sc, energy, n, t = O.si_supercell(2, 2, 4), 100., (128, 128), 5.431 / 4
    else:
        sc, energy, n, t = O.srtio3_supercell(4, 3, 3), 300., (256, 384), 3.905 / 2
    geom = crystal_geom(sc, energy, 20e-3, n)
    _, win = O.atom_windows(geom, KIRK)
    S = geom.num_slices(t)
    sites, offs = M.slice_sites(geom.xyz, geom.Z, geom.pix_size, t, S)
    trans, V = engine.build_transmission(torch.from_numpy(sites).to(DEV), torch.from_numpy(offs).to(DEV),
                                         torch.from_numpy(win).to(DEV), n[0], n[1], np.float32(geom.sigma),
                                         want_potential=True)
    Vref = O.potential_slices_gpu(O.slice_sites_gpu(geom, t), win, n, mode='f32')
    np.testing.assert_array_equal(V.cpu().numpy(), Vref)
    tref = O.transmission(Vref, geom.sigma, mode='f32')
    assert np.abs(trans.cpu().numpy() - tref).max() < 5e-7


@pytest.mark.parametrize('smooth,scherzer', [(True, False), (False, True)])
def test_probe(smooth, scherzer):
    sc = O.si_supercell(8, 8, 1)
    geom = crystal_geom(sc, 200., 30e-3, (512, 512))
    pd = {'smooth_apert': smooth, 'spherical_phase': True, 'aberration_dict': {'C1': 10., 'C3': 1e4, 'C5': 1e5},
          'scherzer': scherzer}
    psik_ref, ap_ref, norm_ref = O.probe_gpu(geom, pd)
    C1 = O.scherzer_defocus(geom.lam, 1e4) if scherzer else 10.
    psik, ap, norm = engine.build_probe(512, 512, np.float32(geom.kmax), geom.lam, np.float32(geom.semi_ang / geom.lam),
                                        C1, 1e4, 1e5, smooth)
    assert np.abs(psik.cpu().numpy() - psik_ref).max() < 1e-6
    assert np.abs(ap.cpu().numpy() - ap_ref).max() < 1e-6
    if not smooth:
        np.testing.assert_array_equal(ap.cpu().numpy(), ap_ref)
    assert abs(norm.item() - norm_ref) < 1e-6 * norm_ref


# ----------------------------------------------------------------------------- multislice
@pytest.mark.parametrize('n', [64, 128, 256, 384, 512, 768, 1024])
def test_multislice_every_size_and_schedule(n):
    g, trans, psik, norm, pos, kmax, lam, st = random_case(n, n, S=3, P=3, seed=n)
    ref = oracle_cbed(g, trans, psik, norm, pos, st, 1 / 3)
    for k in range(len(engine.schedules(n))):
        for tma in (True, False):
            got = engine_cbed(trans, psik, norm, pos, kmax, lam, st, 1 / 3, sched=(k, k), tma=tma)
            err = O.rel_l2(got, ref)
            assert err.max() < 2e-5, (n, k, tma, err)


@pytest.mark.parametrize('ny,nx,bandwidth,P', [(512, 512, 0.45, 13), (512, 512, 1.0, 13), (384, 512, 1 / 3, 9)])
def test_paired_row_schedule(ny, nx, bandwidth, P):
    """The paired 512 row transform (its radix-2 stage by warp shuffles, schedule
    t32_r16x2x16_pair) against the FP64 oracle: groups that fill the last tile of 8
    rows only in part, a wide band and no band limit, and a rectangular grid whose
    rows are 512 long."""
    k = engine.schedules(512).index('t32_r16x2x16_pair')
    g, trans, psik, norm, pos, kmax, lam, st = random_case(ny, nx, S=4, P=P, seed=ny + P)
    ref = oracle_cbed(g, trans, psik, norm, pos, st, bandwidth)
    got = engine_cbed(trans, psik, norm, pos, kmax, lam, st, bandwidth, group=P, sched=(k, 0))
    err = O.rel_l2(got, ref)
    assert err.max() < 2e-5, err


@pytest.mark.parametrize('ny,nx', [(256, 512), (384, 768), (128, 64)])
def test_multislice_rectangular(ny, nx):
    g, trans, psik, norm, pos, kmax, lam, st = random_case(ny, nx, S=4, P=2, seed=ny + nx)
    ref = oracle_cbed(g, trans, psik, norm, pos, st, 1 / 3)
    got = engine_cbed(trans, psik, norm, pos, kmax, lam, st, 1 / 3)
    assert O.rel_l2(got, ref).max() < 2e-5


def test_groups_crop_graph_determinism():
    g, trans, psik, norm, pos, kmax, lam, st = random_case(128, 128, S=5, P=7, seed=3)
    ref = oracle_cbed(g, trans, psik, norm, pos, st, 0.4, crop=64)
    a = engine_cbed(trans, psik, norm, pos, kmax, lam, st, 0.4, crop=64, group=3)
    b = engine_cbed(trans, psik, norm, pos, kmax, lam, st, 0.4, crop=64, group=3, graph=False)
    c = engine_cbed(trans, psik, norm, pos, kmax, lam, st, 0.4, crop=64, group=7)
    d = engine_cbed(trans, psik, norm, pos, kmax, lam, st, 0.4, crop=64, group=7, tma=False)
    e = engine_cbed(trans, psik, norm, pos, kmax, lam, st, 0.4, crop=64, group=3, tma=False)
    assert a.shape == (7, 64, 64)
    assert O.rel_l2(a, ref).max() < 2e-5 and O.rel_l2(d, ref).max() < 2e-5
    np.testing.assert_array_equal(a, b)
    np.testing.assert_array_equal(a, c)
    np.testing.assert_array_equal(d, e)


def test_zero_slices_and_single_probe():
    g, trans, psik, norm, pos, kmax, lam, st = random_case(64, 64, S=0, P=1, seed=5)
    trans = np.zeros((0, 64, 64), np.complex64)
    ref = oracle_cbed(g, trans, psik, norm, pos, st, 1 / 3)
    got = engine_cbed(trans, psik, norm, pos, kmax, lam, st, 1 / 3)
    assert O.rel_l2(got, ref).max() < 1e-6


def test_errors_surface_as_exceptions():
    with pytest.raises(_lib.MsxError) as e:
        engine.Plan(500, 512)
    assert e.value.code == _lib.MSX_ERR_UNSUPPORTED
    g, trans, psik, norm, pos, kmax, lam, st = random_case(64, 64, S=1, P=1, seed=6)
    plan = engine.Plan(64, 64)
    with pytest.raises(_lib.MsxError):
        plan.multislice(torch.from_numpy(trans).to(DEV), torch.from_numpy(psik).to(DEV),
                        torch.tensor([norm], dtype=torch.float64, device=DEV), torch.from_numpy(pos).to(DEV),
                        np.float32(kmax), lam, st, np.float32(kmax / 3), crop=100)


def test_bounded_wait_runs_out_and_the_context_stays_usable():
    """A wait with nothing arriving runs out after its limit (2^22 cycles here) and
    is reported as MSX_ERR_TIMEOUT; the same wait with an arrival succeeds, and
    the context keeps running passes afterwards."""
    with pytest.raises(_lib.MsxError) as e:
        engine.selftest_wait(False, 22)
    assert e.value.code == _lib.MSX_ERR_TIMEOUT
    engine.selftest_wait(True, 22)
    g, trans, psik, norm, pos, kmax, lam, st = random_case(64, 64, S=2, P=2, seed=9)
    plan = engine.Plan(64, 64)
    out = plan.multislice(torch.from_numpy(trans).to(DEV), torch.from_numpy(psik).to(DEV),
                          torch.tensor([norm], dtype=torch.float64, device=DEV), torch.from_numpy(pos).to(DEV),
                          np.float32(kmax), lam, st, np.float32(kmax / 3))
    plan.check()
    assert torch.isfinite(out).all() and out.sum().item() > 0
    plan.close()


@pytest.mark.parametrize('pinned', [True, False])
def test_host_buffer_multislice_matches_device_call(pinned):
    """msx_multislice_host (chunked uploads overlapping the first group, per-group
    downloads) gives exactly the device call's CBEDs: 20 slices in 3 upload chunks,
    7 positions in groups of 3, a central crop."""
    g, trans, psik, norm, pos, kmax, lam, st = random_case(128, 128, S=20, P=7, seed=12)
    plan = engine.Plan(128, 128, 3)
    want = plan.multislice(torch.from_numpy(trans).to(DEV), torch.from_numpy(psik).to(DEV),
                           torch.tensor([norm], dtype=torch.float64, device=DEV), torch.from_numpy(pos).to(DEV),
                           np.float32(kmax), lam, st, np.float32(kmax / 3), crop=96).cpu().numpy()
    host = (lambda a: torch.from_numpy(a).pin_memory()) if pinned else torch.from_numpy
    h_trans, h_psik, h_pos = host(trans), host(psik), host(pos)
    got = plan.multislice_host(h_trans, h_psik, norm, h_pos, np.float32(kmax), lam, st, np.float32(kmax / 3), crop=96)
    torch.cuda.synchronize()
    plan.check()
    np.testing.assert_array_equal(got.numpy(), want)
    # the same buffers with new contents: a repeated call (a graph replay when the
    # buffers are page-locked) reads the host memory again
    pos2 = (pos[::-1] + np.float32(0.37)).copy()
    h_pos.copy_(torch.from_numpy(pos2))
    want2 = plan.multislice(torch.from_numpy(trans).to(DEV), torch.from_numpy(psik).to(DEV),
                            torch.tensor([norm], dtype=torch.float64, device=DEV), torch.from_numpy(pos2).to(DEV),
                            np.float32(kmax), lam, st, np.float32(kmax / 3), crop=96).cpu().numpy()
    out = torch.empty_like(got)
    if pinned:
        out = out.pin_memory()
    for _ in range(2):
        got2 = plan.multislice_host(h_trans, h_psik, norm, h_pos, np.float32(kmax), lam, st, np.float32(kmax / 3),
                                    crop=96, out=out)
        torch.cuda.synchronize()
        plan.check()
        np.testing.assert_array_equal(got2.numpy(), want2)
    assert not np.array_equal(want2, want)
    plan.close()


def test_band_limited_passes_with_an_aperture_wider_than_the_band():
    """From the second slice on the persistent passes skip the columns beyond the
    bandwidth mask.  With a probe aperture wider than the mask (k_semi > k_band)
    the first slice still covers every column: the result equals the plain
    full-grid passes and the FP64 oracle."""
    rng = np.random.default_rng(21)
    n, S, P = 256, 6, 3
    kmax = n / 20.0
    g = geom_of(n, n, kmax, 0.025)
    g.semi_ang = 0.12  # k_semi = 4.8 / Angstrom > k_band = kmax / 3 = 4.27
    pd = {'smooth_apert': True, 'spherical_phase': True, 'aberration_dict': {'C1': 5., 'C3': 1e4, 'C5': 0.},
          'scherzer': False}
    psik, _, _ = O.probe_gpu(g, pd)
    psik = psik.astype(np.complex64)
    norm = float(np.sum(np.abs(np.fft.ifft2(psik.astype(np.complex128)) * n * n) ** 2))
    trans = np.exp(0.3j * rng.standard_normal((S, n, n))).astype(np.complex64)
    pos = rng.uniform(-6, 6, size=(P, 2)).astype(np.float32)
    st = 1.5
    args = (torch.from_numpy(trans).to(DEV), torch.from_numpy(psik).to(DEV),
            torch.tensor([norm], dtype=torch.float64, device=DEV), torch.from_numpy(pos).to(DEV),
            np.float32(kmax), 0.025, st, np.float32(kmax / 3))
    lo, hi = engine.band_columns(n, np.float32(kmax), np.float32(kmax / 3), engine.col_tile(n, 0))
    assert hi - lo < n  # the band really excludes columns here
    plan = engine.Plan(n, n)
    got = plan.multislice(*args).cpu().numpy()
    plan.set_tma(False)
    full = plan.multislice(*args).cpu().numpy()
    plan.check()
    plan.close()
    assert np.abs(got - full).max() <= 1e-6 * np.abs(full).max()
    ref = oracle_cbed(g, trans, psik, norm, pos, st, 1 / 3)
    assert O.rel_l2(got, ref).max() < 2e-5


def test_failed_workspace_allocation_keeps_the_plan_usable():
    """Host-side allocation failure: a 65535-wave group of 1024^2 waves (512 GiB)
    cannot be allocated.  set_schedule reports MSX_ERR_ALLOC and the plan keeps its
    previous group and workspace, so it still computes correct CBEDs."""
    g, trans, psik, norm, pos, kmax, lam, st = random_case(1024, 1024, S=1, P=2, seed=11)
    plan = engine.Plan(1024, 1024, 4)
    with pytest.raises(_lib.MsxError) as e:
        plan.set_schedule(group=65535)
    assert e.value.code == _lib.MSX_ERR_ALLOC
    assert plan.schedule[2] == 4
    got = plan.multislice(torch.from_numpy(trans).to(DEV), torch.from_numpy(psik).to(DEV),
                          torch.tensor([norm], dtype=torch.float64, device=DEV), torch.from_numpy(pos).to(DEV),
                          np.float32(kmax), lam, st, np.float32(kmax / 3)).cpu().numpy()
    plan.check()
    P, _ = O.propagator_gpu(g, st, 1 / 3)
    ref = O.multislice_gpu(trans.astype(np.complex128), psik, P, pos, norm, g)
    assert O.rel_l2(got, ref).max() < 2e-5
    plan.close()


def test_nan_inputs_are_flagged_by_check_simulation():
    """A NaN in the probe propagates into every pattern; check_simulation reports it."""
    sc = O.si_supercell(2, 2, 2)
    sim = M.MSAGPU(200, 25e-3, sc, sampling=np.array([64, 64]), debye_waller=False)
    sim.setup_device(0)
    sim.calc_atomic_potentials()
    sim.build_potential_slices(5.431 / 4)
    sim.build_probe({'smooth_apert': True, 'apert_smooth': 50, 'spherical_phase': True,
                     'aberration_dict': {'C1': 0., 'C3': 0., 'C5': 0.}, 'scherzer': False})
    sim.psi_k_dev[3, 5] = float('nan')
    sim.probe_positions = np.zeros((2, 2))
    sim.num_probes = 2
    sim.multislice()
    with pytest.warns(RuntimeWarning, match='not finite'):
        prob = sim.check_simulation()
    assert not np.isfinite(prob).any()
    sim.close()


# ----------------------------------------------------------------------------- full pipelines
def test_config1_pipeline_vs_fp64():
    """Plain single-probe CBED, Si [001] 4x4x20 cells, 256^2, 80 slices, 100 keV,
    20 mrad, probe at the cell centre: the MSAGPU surface end to end against
    the FP64 oracle (its own windows, slices, probe and propagation)."""
    sc = O.si_supercell(4, 4, 20)
    t = 5.431 / 4
    pd = {'smooth_apert': True, 'apert_smooth': 50, 'spherical_phase': True,
          'aberration_dict': {'C1': 0., 'C3': 0., 'C5': 0.}, 'scherzer': False}
    sim = M.MSAGPU(100, 20e-3, sc, sampling=np.array([256, 256]), debye_waller=False)
    sim.setup_device(0)
    sim.calc_atomic_potentials()
    sim.build_potential_slices(t)
    assert sim.num_slices == 80
    sim.build_probe(pd)
    sim.probe_positions = np.array([[0., 0.]])
    sim.num_probes = 1
    sim.multislice(bandwidth=1 / 3)
    got = sim.probes

    geom = crystal_geom(sc, 100., 20e-3, (256, 256))
    _, win = O.atom_windows(geom, KIRK)
    V = O.potential_slices_gpu(O.slice_sites_gpu(geom, t), win, geom.sampling, mode='f64')
    tr = O.transmission(V, geom.sigma)
    psik, _, norm = O.probe_gpu(geom, pd)
    P, _ = O.propagator_gpu(geom, t, 1 / 3)
    ref = O.multislice_gpu(tr, psik, P, np.array([[0., 0.]]), norm, geom)
    err = O.rel_l2(got, ref)
    assert got.shape == (1, 256, 256)
    assert err.max() < 1e-4, err
    assert 0.9 < got.sum() <= 1.0 + 1e-5


def test_config2_scan_sampled_vs_fp64():
    """Batched STEM scan, Si [001] 8x8x50 cells, 512^2, 199 slices, 200 keV,
    30 mrad, Cs 1 um, 32x32 positions over one unit cell, central 256^2 crop.
    All 1024 patterns run; 4 of them are checked against the FP64 oracle,
    all of them for finiteness, range and run-to-run bit identity."""
    a = 5.431
    sc = O.si_supercell(8, 8, 50)
    t = a / 4
    pd = {'smooth_apert': True, 'apert_smooth': 50, 'spherical_phase': True,
          'aberration_dict': {'C1': 0., 'C3': 1e4, 'C5': 0.}, 'scherzer': False}
    sim = M.MSAGPU(200, 30e-3, sc, sampling=np.array([512, 512]), debye_waller=False)
    sim.setup_device(0)
    sim.calc_atomic_potentials()
    sim.build_potential_slices(t)
    assert sim.num_slices == 199
    sim.build_probe(pd)
    ii, jj = np.meshgrid(np.arange(32), np.arange(32), indexing='ij')
    sim.probe_positions = np.column_stack([ii.ravel() * a / 32, jj.ravel() * a / 32])
    sim.num_probes = 1024
    sim.multislice(bandwidth=1 / 3, crop=256)
    got = sim.probes.copy()
    sim.multislice(bandwidth=1 / 3, crop=256)
    np.testing.assert_array_equal(sim.probes, got)
    assert got.shape == (1024, 256, 256) and np.isfinite(got).all() and got.min() >= 0
    tot = got.astype(np.float64).sum((1, 2))
    assert (tot > 0.5).all() and (tot < 1.0 + 1e-5).all()

    geom = crystal_geom(sc, 200., 30e-3, (512, 512))
    tr = sim.trans.cpu().numpy().astype(np.complex128)
    psik, _, norm = O.probe_gpu(geom, pd)
    P, _ = O.propagator_gpu(geom, t, 1 / 3)
    pick = np.array([0, 333, 517, 1023])
    ref = O.multislice_gpu(tr, psik, P, sim.probe_positions[pick], norm, geom, crop=256)
    err = O.rel_l2(got[pick], ref)
    assert err.max() < 1e-4, err


def test_detector_signals_match_oracle():
    """Fused detector epilogue (msx_multislice_detect) against the oracle's
    integrate_cbed (namsa/msa.py:426-439, pinned to the reference class by
    tests/golden/detector.npz) applied to the FP64 oracle's CBED stack of the same
    inputs, with the reference's own annuli and a smooth weight map."""
    g, trans, psik, norm, pos, kmax, lam, st = random_case(256, 256, S=4, P=6, seed=21)
    kpix = np.array([kmax, kmax]) / 256
    det = [O.annular_detector(np.array([256, 256]), kpix, lam, a, b) for a, b in [(0.02, 0.05), (0.05, 0.09),
                                                                                   (0.0, 0.02)]]
    ky, kx = np.mgrid[-128:128, -128:128]
    det.append(np.exp(-(kx ** 2 + ky ** 2) / 900.0))
    det = np.stack(det).astype(np.float32)
    P, _ = O.propagator_gpu(g, st, 0.45)
    cbed = O.multislice_gpu(trans.astype(np.complex128), psik.astype(np.complex128), P, pos, norm, g)
    ref = np.stack([O.integrate_cbed(cbed, (6,), d) for d in det], axis=1)
    plan = engine.Plan(256, 256, 2)
    sig = plan.detect(torch.from_numpy(trans).to(DEV), torch.from_numpy(psik).to(DEV),
                      torch.tensor([norm], dtype=torch.float64, device=DEV), torch.from_numpy(pos).to(DEV),
                      np.float32(kmax), lam, st, np.float32(0.45 * kmax), torch.from_numpy(det).to(DEV)).cpu().numpy()
    plan.close()
    assert sig.shape == (6, 4)
    assert np.abs(sig - ref).max() <= 2e-5 * np.abs(ref).max()
    # the facade's stored-stack form agrees with the fused one
    assert np.abs(sig[:, :3] - np.einsum('pyx,dyx->pd', cbed, det[:3].astype(np.float64))).max() <= 2e-5 * np.abs(ref).max()


def test_real_space_stepping_matches_multislice():
    """probe_waves + step_waves per slice + cbed_waves reproduce msx_multislice."""
    g, trans, psik, norm, pos, kmax, lam, st = random_case(128, 128, S=4, P=3, seed=31)
    ref = engine_cbed(trans, psik, norm, pos, kmax, lam, st, 1 / 3)
    plan = engine.Plan(128, 128)
    d_trans = torch.from_numpy(trans).to(DEV)
    d_psik = torch.from_numpy(psik).to(DEV)
    d_norm = torch.tensor([norm], dtype=torch.float64, device=DEV)
    ptab = engine.propagator_table(128, 128, np.float32(kmax), lam, st, np.float32(kmax / 3))
    w = plan.probe_waves(d_psik, torch.from_numpy(pos).to(DEV), np.float32(kmax))
    for s in range(trans.shape[0]):
        plan.step_waves(w, d_trans[s], ptab)
    got = plan.cbed_waves(w, d_norm).cpu().numpy()
    plan.close()
    assert O.rel_l2(got, ref).max() < 2e-6


@pytest.mark.parametrize('ny,nx', [(256, 256), (256, 384)])
def test_probe_stack_without_transmission(ny, nx):
    """multislice(transmit=False) returns the unit-norm complex64 probe stack of
    every position with no slice applied (namsa/msa.py:959-964, 970, 914-915),
    checked against the FP64 oracle's probe formation."""
    sc = O.srtio3_supercell(6, 6, 2)
    pd = {'smooth_apert': True, 'apert_smooth': 50, 'spherical_phase': True,
          'aberration_dict': {'C1': 25., 'C3': 2e4, 'C5': 0.}, 'scherzer': False}
    sim = M.MSAGPU(200, 25e-3, sc, sampling=np.array([ny, nx]), debye_waller=False)
    sim.setup_device(0)
    sim.calc_atomic_potentials()
    sim.build_potential_slices(3.905 / 2)
    sim.build_probe(pd)
    sim.generate_probe_positions(grid_steps=np.array([3, 4]))
    sim.multislice(transmit=False)
    got = sim.probes
    assert got.dtype == np.complex64 and got.shape == (12, ny, nx)

    geom = crystal_geom(sc, 200., 25e-3, (ny, nx))
    psik, _, norm = O.probe_gpu(geom, pd)
    ref = O.probe_stack_gpu(psik, sim.probe_positions.astype(np.float32), norm, geom)  # the engine's float32 positions
    err = np.linalg.norm((got - ref).reshape(12, -1), axis=1) / np.linalg.norm(ref.reshape(12, -1), axis=1)
    assert err.max() < 5e-6, err
    np.testing.assert_allclose(np.sum(np.abs(got.astype(np.complex128)) ** 2, axis=(1, 2)), 1.0, rtol=1e-5)
    # a CBED run afterwards still returns the float32 stack
    sim.multislice(crop=128)
    assert sim.probes.dtype == np.float32 and sim.probes.shape == (12, 128, 128)
    sim.close()


def test_integrate_cbed_of_a_stored_stack_matches_oracle():
    """MSAGPU.integrate_cbed and check_simulation reduce the stored CBED stack in libmsx
    (msx_integrate_cbed); the signals equal the oracle's integrate_cbed (namsa/msa.py:426-439)
    of the same stack, and the per-pattern sums its float64 sums."""
    sc = O.si_supercell(4, 4, 3)
    pd = {'smooth_apert': True, 'apert_smooth': 50, 'spherical_phase': True,
          'aberration_dict': {'C1': 0., 'C3': 1e4, 'C5': 0.}, 'scherzer': False}
    sim = M.MSAGPU(200, 30e-3, sc, sampling=np.array([128, 128]), debye_waller=False)
    sim.setup_device(0)
    sim.calc_atomic_potentials()
    sim.build_potential_slices(5.431 / 4)
    sim.build_probe(pd)
    sim.generate_probe_positions(grid_steps=np.array([3, 2]))
    sim.multislice()
    stack = sim.probes.astype(np.float64)
    img, det = sim.integrate_cbed(detector_params={'inner_angle': 20e-3, 'outer_angle': 60e-3})
    ref = O.integrate_cbed(stack, sim.grid_steps, det)
    np.testing.assert_allclose(img, ref, rtol=1e-10)
    np.testing.assert_array_equal(det, O.annular_detector(sim.sampling, sim.kpix_size, sim.Lambda, 20e-3, 60e-3))
    np.testing.assert_allclose(sim.check_simulation(), stack.sum((1, 2)), rtol=1e-10)
    sim.close()
