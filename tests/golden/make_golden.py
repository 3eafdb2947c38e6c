"""Generate the golden fixtures in this folder from the reference's own CPU code.

Run where a checkout of the reference is available; its path is the first
argument or the environment variable ``NAMSA_REFERENCE``.  The reference package imports
pycuda/skcuda/mpi4py/h5py/pymatgen at module load; none of these is used by
the ``MSA`` CPU class, so they are replaced by empty stub modules, and the
NumPy aliases removed in NumPy 2 (``np.int``, ``np.float``, ``np.bool``) are
restored.  Nothing of the reference is modified.

Fixtures written (all ``.npz``):

* ``optics.npz``      -- wavelength and interaction parameter at five voltages
                         (namsa/optics.py:4-12, 100-108) and Scherzer defocus.
* ``si_small.npz``    -- Si 2x2x4 cells at 128^2, 100 keV, 20 mrad: the Kirkland
                         window, the CPU potential slices, ``build_probe``
                         outputs and exit waves of ``multislice`` at 3 positions.
* ``si_config1.npz``  -- Si 4x4x20 cells at 256^2, 80 slices, 100 keV, 20 mrad,
                         probe at the origin: window, slice checksums and exit wave.
* ``positions.npz``   -- ``generate_probe_positions`` for both of its branches.
* ``postproc.npz``    -- ``process_cbed`` / ``process_potential``
                         (scripts/summit_scripts/utils.py:74-118) on seeded inputs.
* ``integrated.npz``  -- ``MSA.integrate_potential_slices`` (namsa/msa.py:373-424)
                         on a seeded 3-D potential.  SciPy 1.14 removed
                         ``integrate.trapz``; it is aliased to ``trapezoid``
                         (the same rule) for this call.
* ``detector.npz``    -- ``MSA.integrate_cbed`` (namsa/msa.py:426-439) on a seeded
                         CBED stack: the default 50-100 mrad annulus it builds and a
                         20-60 mrad one, with the integrated signals.
* ``cif.npz``         -- the reference's own CIF test inputs and expected unit
                         cells (cif_files/mvc-9418.cif with mvc-9418_P_1_1_1.xyz,
                         the golden of tests/supercell_tests.py:8-21, and
                         cif_files/Si.cif), read as text.
"""
import os
import sys
import types

import numpy as np
import scipy.integrate  # noqa: F401  (imported before the NumPy aliases are restored)
import scipy.special  # noqa: F401

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, '..', '..'))
from oracle.msa_oracle import si_supercell  # noqa: E402


class _Stub(types.ModuleType):
    def __getattr__(self, k):
        if k.startswith('__'):
            raise AttributeError(k)
        return type(k, (), {})


def import_reference(ref_root):
    for name in ['pycuda', 'pycuda.driver', 'pycuda.gpuarray', 'pycuda.compiler', 'pycuda.tools', 'skcuda',
                 'skcuda.fft', 'skcuda.cufft', 'h5py', 'mpi4py', 'pymatgen', 'pymatgen.core', 'pymatgen.io',
                 'pymatgen.io.cif', 'pymatgen.analysis', 'pymatgen.analysis.diffraction',
                 'pymatgen.analysis.diffraction.xrd', 'pymatgen.symmetry', 'pymatgen.symmetry.analyzer']:
        sys.modules.setdefault(name, _Stub(name))
    np.int = int
    np.float = float
    np.bool = bool
    sys.path.insert(0, ref_root)
    import namsa.msa as msa
    import namsa.optics as optics
    return msa, optics


def import_reference_utils(ref_root):
    for name in ['skimage', 'skimage.transform']:
        sys.modules.setdefault(name, _Stub(name))
    sys.path.insert(0, os.path.join(ref_root, 'scripts', 'summit_scripts'))
    import utils as ref_utils
    return ref_utils


def detector_fixture(msa, rng):
    """integrate_cbed of the reference CPU class on a seeded CBED stack."""
    m = msa.MSA(200, 30e-3, si_supercell(2, 2, 1), sampling=np.array([64, 64]), debye_waller=False)
    m.grid_steps = np.array([3, 2])
    cbed = rng.gamma(0.8, 1e-3, size=(6, 64, 64)).astype(np.float32)
    out = {'cbed': cbed, 'grid_steps': m.grid_steps, 'sampling': m.sampling, 'kpix_size': m.kpix_size,
           'Lambda': m.Lambda, 'max_ang': m.max_ang}
    for tag, params in [('default', {'inner_angle': 50e-3, 'outer_angle': 100e-3}),
                        ('narrow', {'inner_angle': 20e-3, 'outer_angle': 60e-3})]:
        m.probes = cbed.copy()
        sig, det = m.integrate_cbed(detector_params=params)
        out[tag + '_inner'] = params['inner_angle']
        out[tag + '_outer'] = params['outer_angle']
        out[tag + '_detector'] = det
        out[tag + '_signal'] = sig
    return out


def cif_fixture(ref_root):
    """The reference's CIF test inputs and expected P1 unit cell, as text and arrays."""
    d = os.path.join(ref_root, 'cif_files')
    with open(os.path.join(d, 'mvc-9418.cif')) as f:
        mvc = f.read()
    with open(os.path.join(d, 'Si.cif')) as f:
        si = f.read()
    xyz = np.loadtxt(os.path.join(d, 'mvc-9418_P_1_1_1.xyz'), skiprows=2,
                     dtype=[('atom_type', '|U16'), ('x', 'f'), ('y', 'f'), ('z', 'f')])
    return {'mvc_cif': np.array(mvc), 'si_cif': np.array(si), 'mvc_types': xyz['atom_type'],
            'mvc_xyz': np.column_stack([xyz['x'], xyz['y'], xyz['z']])}


def main(ref_root=None):
    ref_root = ref_root or os.environ.get('NAMSA_REFERENCE')
    if not ref_root:
        raise SystemExit('usage: make_golden.py REFERENCE_CHECKOUT (or set NAMSA_REFERENCE)')
    msa, optics = import_reference(ref_root)
    volts = np.array([80e3, 100e3, 120e3, 200e3, 300e3])
    np.savez_compressed(os.path.join(HERE, 'optics.npz'), volts=volts,
                        lam=np.array([optics.voltage2Lambda(v) for v in volts]),
                        sigma=np.array([optics.sigma_int(v) for v in volts]),
                        scherzer_c1=np.array([optics.scherzer_params(optics.voltage2Lambda(v), 1e4)[0] for v in volts]))

    pd = {'smooth_apert': True, 'apert_smooth': 50, 'spherical_phase': True,
          'aberration_dict': {'C1': 20., 'C3': 1e4, 'C5': 0.}, 'scherzer': False}

    # small Si case: 2x2x4 cells, 128^2
    sc = si_supercell(2, 2, 4)
    m = msa.MSA(100, 20e-3, sc, sampling=np.array([128, 128]), debye_waller=False)
    m.calc_atomic_potentials()
    t = 5.431 / 4
    m.build_potential_slices(t)
    pos = np.array([[0., 0.], [1.3, -0.7], [-2.1, 2.9]])
    probe_x, probe_k, aperture = m.build_probe(pos[1], pd)
    m.probe_positions = pos
    m.num_probes = len(pos)
    waves = m.multislice(probe_grid=True, save_probes=False, bandwidth=1 / 3)
    np.savez_compressed(os.path.join(HERE, 'si_small.npz'), xyz=np.column_stack([sc['x'], sc['y'], sc['z']]),
                        Z=sc['atomic_number'], sampling=np.array([128, 128]), energy=100., semi_angle=20e-3,
                        slice_t=t, window=m.cached_pots[14], V=m.potential_slices, positions=pos,
                        probe_x=probe_x, probe_k=probe_k, aperture=aperture, waves=waves,
                        dims=m.dims, kmax=m.kmax, pix_size=m.pix_size, sigma=m.sigma)

    # config 1: Si 4x4x20 cells, 256^2, 80 slices, probe at the origin
    sc = si_supercell(4, 4, 20)
    m = msa.MSA(100, 20e-3, sc, sampling=np.array([256, 256]), debye_waller=False)
    m.calc_atomic_potentials()
    m.build_potential_slices(t)
    pd1 = {'smooth_apert': True, 'apert_smooth': 50, 'spherical_phase': True,
           'aberration_dict': {'C1': 0., 'C3': 0., 'C5': 0.}, 'scherzer': False}
    m.build_probe(np.array([0., 0.]), pd1)
    wave = m.multislice(probe_pos=np.array([0., 0.]), probe_grid=False, save_probes=False)
    V = m.potential_slices
    np.savez_compressed(os.path.join(HERE, 'si_config1.npz'), sampling=np.array([256, 256]), energy=100.,
                        semi_angle=20e-3, slice_t=t, window=m.cached_pots[14], V_sum=V.astype(np.float64).sum((1, 2)),
                        V_rows=V[:, ::37, :].copy(), wave=wave, num_slices=V.shape[0],
                        dims=m.dims, kmax=m.kmax, pix_size=m.pix_size, sigma=m.sigma)

    # probe positions, both branches
    res = {}
    m2 = msa.MSA(200, 30e-3, si_supercell(8, 8, 2), sampling=np.array([512, 512]), debye_waller=False)
    for name, kw in [('steps', dict(probe_step=np.array([0.5, 0.5]), probe_range=np.array([[0.25, 0.75], [0.25, 0.75]]))),
                     ('steps2', dict(probe_step=np.array([1.0, 0.7]), probe_range=np.array([[0., 1.], [0.1, 0.6]]))),
                     ('grid', dict(grid_steps=np.array([8, 8]))),
                     ('grid2', dict(grid_steps=np.array([4, 6]), fraction=0.25, origin=np.array([0.1, 0.2])))]:
        m2.generate_probe_positions(**kw)
        res[name + '_pos'] = m2.probe_positions
        res[name + '_steps'] = m2.grid_steps
        res[name + '_range'] = m2.grid_range
    res['dims'] = m2.dims
    np.savez_compressed(os.path.join(HERE, 'positions.npz'), **res)

    # dataset post-processing
    ru = import_reference_utils(ref_root)
    rng = np.random.default_rng(7)
    cbed = rng.gamma(0.7, 1e-4, size=(3, 32, 40)).astype(np.float32)
    trans = np.exp(1j * rng.uniform(0, 0.4, size=(4, 64, 64))).astype(np.complex64)
    np.savez_compressed(os.path.join(HERE, 'postproc.npz'), cbed=cbed, cbed_out=ru.process_cbed(cbed),
                        trans=trans, pot_out=ru.process_potential(trans))

    # integrated potential slices
    import scipy.integrate as si
    si.trapz = si.trapezoid
    m3 = msa.MSA(200, 20e-3, si_supercell(1, 1, 1), sampling=np.array([48, 48]), debye_waller=False)
    pot = rng.uniform(0, 2, size=(31, 50, 48)).astype(np.float32)
    zc = np.linspace(0, 12.0, 31)
    yc = np.linspace(0, 9.0, 50)
    xc = np.linspace(0, 8.5, 48)
    out = m3.integrate_potential_slices(pot, (zc, yc, xc), 2.5, output=True)
    np.savez_compressed(os.path.join(HERE, 'integrated.npz'), pot=pot, z=zc, y=yc, x=xc, slice_t=2.5,
                        slices=out, sigma=m3.sigma, sampling=m3.sampling, dims=m3.dims)

    np.savez_compressed(os.path.join(HERE, 'detector.npz'), **detector_fixture(msa, np.random.default_rng(11)))
    np.savez_compressed(os.path.join(HERE, 'cif.npz'), **cif_fixture(ref_root))
    print('golden fixtures written to', HERE)


if __name__ == '__main__':
    main(*sys.argv[1:])
