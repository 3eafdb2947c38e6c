"""CIF reader and orthogonal tiling (namsa_gb300/cif.py) against the reference's
own CIF golden (tests/supercell_tests.py:8-21: cif_files/mvc-9418.cif expanded
to its P1 unit cell, compared with mvc-9418_P_1_1_1.xyz at 2 decimals) and a
centred cell given by its symmetry operations (Si, F d -3 m).  CPU only."""
import os

import numpy as np
import pytest

from namsa_gb300 import cif, structures

G = os.path.join(os.path.dirname(__file__), 'golden')


@pytest.fixture(scope='module')
def fixture():
    return np.load(os.path.join(G, 'cif.npz'))


def test_p1_unit_cell_matches_reference_golden(fixture):
    c = cif.read_cif(str(fixture['mvc_cif']))
    np.testing.assert_allclose(c.lattice_const, [5.62367184, 8.81191945, 11.49202588])
    assert len(c.sym_ops) == 1 and len(c.sites) == 45
    uc = cif.unit_cell(c)
    got = np.round(np.column_stack([uc['x'], uc['y'], uc['z']]).astype(np.float32), 2)
    want = np.round(fixture['mvc_xyz'], 2)
    np.testing.assert_array_equal(got, want)
    np.testing.assert_array_equal(uc['atom_type'], fixture['mvc_types'])
    assert set(uc['atomic_number']) == {26, 14, 51, 8}
    assert np.all(uc['DW'] == np.float32(0.07)) and np.all(uc['occ'] == 1)


def test_centred_cell_by_symmetry_operations(fixture):
    c = cif.read_cif(str(fixture['si_cif']))
    assert len(c.sym_ops) == 192 and c.orthogonal
    uc = cif.unit_cell(c)
    frac = np.column_stack([uc['frac_x'], uc['frac_y'], uc['frac_z']])
    assert len(uc) == 8
    assert {tuple(r) for r in np.round(frac, 6) % 1.0} == {tuple(r) for r in np.round(structures.DIAMOND_BASIS, 6)}
    sc = cif.orthogonal_supercell(c, (2, 2, 3))
    ref = structures.tile(structures.DIAMOND_BASIS, np.full(8, 14), (2, 2, 3), 5.43094)
    key = lambda a: np.array(sorted(zip(np.round(a['x'], 4), np.round(a['y'], 4), np.round(a['z'], 4))))
    np.testing.assert_array_equal(key(sc), key(ref))
    assert set(sc['atomic_number']) == {14}


def test_symop_parser_and_errors():
    m = cif.parse_symop('-y+1/4, x+3/4, z+1/4')
    np.testing.assert_allclose(m @ np.array([0.1, 0.2, 0.3, 1.0]), [0.05, 0.85, 0.55, 1.0])
    m = cif.parse_symop('1/2+x, -z, 2*y')
    np.testing.assert_allclose(m @ np.array([0.1, 0.2, 0.3, 1.0]), [0.6, -0.3, 0.4, 1.0])
    with pytest.raises(ValueError):
        cif.parse_symop('x, y')
    with pytest.raises(ValueError):
        cif.atomic_number('Xx')
    assert cif.atomic_number('Fe3+') == 26 and cif.atomic_number('O2-') == 8
    tri = cif.read_cif('data_t\n_cell_length_a 3\n_cell_length_b 4\n_cell_length_c 5\n_cell_angle_alpha 90\n'
                       '_cell_angle_beta 90\n_cell_angle_gamma 120\nloop_\n_atom_site_label\n_atom_site_fract_x\n'
                       '_atom_site_fract_y\n_atom_site_fract_z\nC1 0 0 0\n')
    with pytest.raises(ValueError, match='orthogonal'):
        cif.orthogonal_supercell(tri, (1, 1, 1))


def test_supercell_feeds_the_simulator_surface(fixture):
    """The tiled CIF cell is the structured array MSAGPU takes (no GPU needed for the geometry)."""
    from namsa_gb300 import msa as M
    sc = cif.orthogonal_supercell(cif.read_cif(str(fixture['si_cif'])), (4, 4, 2))
    arr = M.load_supercell(sc)
    dims = np.column_stack([arr['x'], arr['y'], arr['z']]).max(0) - np.column_stack([arr['x'], arr['y'], arr['z']]).min(0)
    np.testing.assert_allclose(dims, [4 * 5.43094, 4 * 5.43094, 2 * 5.43094], rtol=1e-6)
