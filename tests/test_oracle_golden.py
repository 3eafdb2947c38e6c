"""The oracle against the golden fixtures made from the reference's own CPU code
(tests/golden/make_golden.py).  CPU only."""
import os

import numpy as np
import pytest

from oracle import msa_oracle as O

G = os.path.join(os.path.dirname(__file__), 'golden')
KIRK = os.path.join(os.path.dirname(os.path.dirname(__file__)), 'namsa_gb300', 'data', 'kirkland_params.npy')
PD_SMALL = {'smooth_apert': True, 'apert_smooth': 50, 'spherical_phase': True,
            'aberration_dict': {'C1': 20., 'C3': 1e4, 'C5': 0.}, 'scherzer': False}
PD_CFG1 = {'smooth_apert': True, 'apert_smooth': 50, 'spherical_phase': True,
           'aberration_dict': {'C1': 0., 'C3': 0., 'C5': 0.}, 'scherzer': False}


@pytest.fixture(scope='module')
def kirk():
    return np.load(KIRK)


def test_optics():
    g = np.load(os.path.join(G, 'optics.npz'))
    np.testing.assert_allclose(O.voltage2lambda(g['volts']), g['lam'], rtol=1e-15)
    np.testing.assert_allclose(O.sigma_int(g['volts']), g['sigma'], rtol=1e-15)
    np.testing.assert_allclose(O.scherzer_defocus(g['lam'], 1e4), g['scherzer_c1'], rtol=1e-15)


def test_small_geometry_windows_slices(kirk):
    g = np.load(os.path.join(G, 'si_small.npz'))
    geom = O.Geometry(g['xyz'], g['Z'], float(g['energy']), float(g['semi_angle']), g['sampling'])
    np.testing.assert_array_equal(geom.dims, g['dims'])
    assert geom.kmax == g['kmax'] and geom.sigma == g['sigma']
    np.testing.assert_array_equal(geom.pix_size, g['pix_size'])
    _, win = O.atom_windows(geom, kirk)
    np.testing.assert_array_equal(win[0], g['window'])
    V = O.potential_slices_cpu(geom, win, float(g['slice_t']))
    np.testing.assert_array_equal(V, g['V'])


def test_small_probe_and_exit_waves(kirk):
    g = np.load(os.path.join(G, 'si_small.npz'))
    geom = O.Geometry(g['xyz'], g['Z'], float(g['energy']), float(g['semi_angle']), g['sampling'])
    px, pk, ap = O.probe_cpu(geom, PD_SMALL, g['positions'][1])
    assert np.abs(px - g['probe_x']).max() < 1e-6 * np.abs(g['probe_x']).max()
    assert np.abs(pk - g['probe_k']).max() < 1e-6
    assert np.abs(ap - g['aperture']).max() < 1e-6
    Pm = O.propagator_cpu(geom, float(g['slice_t']), 1 / 3)
    for i, pos in enumerate(g['positions']):
        # the CPU path unpacks [y, x] positions as (x, y) (msa.py:225 with msa.py:265)
        p0, _, _ = O.probe_cpu(geom, PD_SMALL, pos)
        w = O.exit_wave_cpu(g['V'], geom.sigma, p0, Pm)
        assert np.linalg.norm(w - g['waves'][i]) / np.linalg.norm(w) < 1e-5


def test_config1_exit_wave(kirk):
    g = np.load(os.path.join(G, 'si_config1.npz'))
    sc = O.si_supercell(4, 4, 20)
    geom = O.Geometry(np.column_stack([sc['x'], sc['y'], sc['z']]), sc['atomic_number'], 100., 20e-3, [256, 256])
    assert geom.num_slices(float(g['slice_t'])) == int(g['num_slices']) == 80
    np.testing.assert_array_equal(geom.dims, g['dims'])
    _, win = O.atom_windows(geom, kirk)
    np.testing.assert_array_equal(win[0], g['window'])
    V = O.potential_slices_cpu(geom, win, float(g['slice_t']))
    np.testing.assert_array_equal(V.astype(np.float64).sum((1, 2)), g['V_sum'])
    np.testing.assert_array_equal(V[:, ::37, :], g['V_rows'])
    p0, _, _ = O.probe_cpu(geom, PD_CFG1, (0., 0.))
    w = O.exit_wave_cpu(V, geom.sigma, p0, O.propagator_cpu(geom, float(g['slice_t']), 1 / 3))
    assert np.linalg.norm(w - g['wave']) / np.linalg.norm(w) < 2e-5


@pytest.mark.parametrize('name,kw', [
    ('steps', dict(probe_step=np.array([0.5, 0.5]), probe_range=np.array([[0.25, 0.75], [0.25, 0.75]]))),
    ('steps2', dict(probe_step=np.array([1.0, 0.7]), probe_range=np.array([[0., 1.], [0.1, 0.6]]))),
    ('grid', dict(grid_steps=np.array([8, 8]))),
    ('grid2', dict(grid_steps=np.array([4, 6]), fraction=0.25, origin=np.array([0.1, 0.2]))),
])
def test_positions(name, kw):
    g = np.load(os.path.join(G, 'positions.npz'))
    pos, st, rg = O.generate_probe_positions(g['dims'], **kw)
    np.testing.assert_array_equal(pos, g[name + '_pos'])
    np.testing.assert_array_equal(st, g[name + '_steps'])
    np.testing.assert_array_equal(rg, g[name + '_range'])


def test_gpu_conventions_self_consistency(kirk):
    """GPU-convention pieces: the float32 accumulation mode matches the float64
    one to rounding, the fftshift carrier and Parseval normalisation hold."""
    sc = O.si_supercell(2, 2, 2)
    geom = O.Geometry(np.column_stack([sc['x'], sc['y'], sc['z']]), sc['atomic_number'], 200., 25e-3, [64, 64])
    _, win = O.atom_windows(geom, kirk)
    sites = O.slice_sites_gpu(geom, 5.431 / 4)
    V32 = O.potential_slices_gpu(sites, win, geom.sampling, mode='f32')
    V64 = O.potential_slices_gpu(sites, win, geom.sampling, mode='f64')
    assert np.abs(V32 - V64).max() < 1e-5 * np.abs(V64).max()
    pd = dict(PD_SMALL, scherzer=True)
    psik, ap, norm = O.probe_gpu(geom, pd)
    assert abs(norm - 64 * 64 * np.sum(np.abs(psik) ** 2)) < 1e-9 * norm


def test_postprocessing_matches_reference():
    g = np.load(os.path.join(G, 'postproc.npz'))
    np.testing.assert_array_equal(O.process_cbed(g['cbed']), g['cbed_out'])
    np.testing.assert_array_equal(O.process_potential(g['trans']), g['pot_out'])


def test_integrated_potential_matches_reference():
    g = np.load(os.path.join(G, 'integrated.npz'))
    out = O.integrate_potential_slices(g['pot'], g['z'], float(g['slice_t']))
    assert out.shape == g['slices'].shape
    np.testing.assert_allclose(out, g['slices'], rtol=2e-6, atol=2e-6)


def test_integrate_cbed_against_reference():
    """Detector epilogue oracle (integrate_cbed, namsa/msa.py:426-439) against the
    reference class's own output: the annulus it builds from the angles, bit for
    bit, and the integrated signals of a seeded CBED stack."""
    g = np.load(os.path.join(G, 'detector.npz'))
    for tag in ('default', 'narrow'):
        det = O.annular_detector(g['sampling'], g['kpix_size'], float(g['Lambda']), float(g[tag + '_inner']),
                                 float(g[tag + '_outer']))
        np.testing.assert_array_equal(det, g[tag + '_detector'])
        sig = O.integrate_cbed(g['cbed'], g['grid_steps'], det)
        assert sig.shape == tuple(g['grid_steps'])
        np.testing.assert_allclose(sig, g[tag + '_signal'], rtol=2e-6)


def test_facade_detector_matches_reference():
    """The MSAGPU surface builds the same annulus as the reference (host code, no GPU)."""
    from namsa_gb300 import msa as M
    g = np.load(os.path.join(G, 'detector.npz'))
    for tag in ('default', 'narrow'):
        det = M.annular_detector(g['sampling'], g['kpix_size'], float(g['Lambda']), float(g[tag + '_inner']),
                                 float(g[tag + '_outer']))
        np.testing.assert_array_equal(det, g[tag + '_detector'])
