"""Minimal structure builder for orthogonal supercells (no pymatgen).

Covers what the multislice path consumes from namsa's ``SupercellBuilder``
(namsa/supercell.py:56-464): a structured array with fields atomic_number,
x, y, z, occ, DW for an orthogonal cell tiled along [001], keeping every atom
with 0 <= r <= size on each axis (the inclusive bounds of
``make_orthogonal_supercell``, namsa/supercell.py:444), plus the XYZ text
format read by ``MSA.__init__`` (namsa/msa.py:83-86).
"""
from __future__ import annotations

import numpy as np

XYZ_dtype = [('atomic_number', 'i'), ('x', 'f'), ('y', 'f'), ('z', 'f'), ('occ', 'f'), ('DW', 'f')]

DIAMOND_BASIS = np.array([[0, 0, 0], [0, .5, .5], [.5, 0, .5], [.5, .5, 0],
                          [.25, .25, .25], [.25, .75, .75], [.75, .25, .75], [.75, .75, .25]])
PEROVSKITE_BASIS = np.array([[0, 0, 0], [.5, .5, .5], [.5, .5, 0], [.5, 0, .5], [0, .5, .5]])


def tile(basis, species, cells, a, dw=0.0):
    """Tile a cubic (or orthorhombic, ``a`` a 3-vector) cell ``cells`` = (nx, ny, nz)
    times; fractional ``basis`` (n, 3) with atomic numbers ``species`` (n,)."""
    cells = np.asarray(cells, dtype=np.int64)
    a = np.broadcast_to(np.asarray(a, dtype=np.float64), (3,))
    grid = np.stack(np.meshgrid(*[np.arange(k + 1) for k in cells], indexing='ij'), -1).reshape(-1, 3)
    pos = (grid[:, None, :] + np.asarray(basis)[None, :, :]).reshape(-1, 3) * a
    zz = np.tile(np.asarray(species), len(grid))
    size = cells * a
    keep = np.all((pos >= 0) & (pos <= size + 1e-6), axis=1)
    pos, zz = pos[keep], zz[keep]
    out = np.zeros(len(pos), dtype=XYZ_dtype)
    out['atomic_number'] = zz
    out['x'], out['y'], out['z'] = pos[:, 0], pos[:, 1], pos[:, 2]
    out['occ'] = 1
    out['DW'] = dw
    return out


def silicon(cells, a=5.431):
    """Diamond-cubic Si viewed along [001]."""
    return tile(DIAMOND_BASIS, np.full(len(DIAMOND_BASIS), 14), cells, a)


def srtio3(cells, a=3.905):
    """Cubic perovskite SrTiO3: Sr (0,0,0), Ti (1/2,1/2,1/2), O on the face centres."""
    return tile(PEROVSKITE_BASIS, np.array([38, 22, 8, 8, 8]), cells, a)


def random_cubic(rng, a_range=(3.0, 8.0), species_range=(1, 4), z_range=(3, 83), atoms_range=(2, 16)):
    """A random cubic cell: lattice constant U[a_range], 1-4 species with Z
    uniform in z_range, 2-16 atoms at uniform fractional positions.
    Returns (basis, species, a)."""
    a = rng.uniform(*a_range)
    nspec = rng.integers(species_range[0], species_range[1] + 1)
    zs = rng.integers(z_range[0], z_range[1] + 1, size=nspec)
    nat = rng.integers(atoms_range[0], atoms_range[1] + 1)
    basis = rng.uniform(0, 1, size=(nat, 3))
    species = zs[rng.integers(0, nspec, size=nat)]
    return basis, species, a


def write_xyz(path, sites, comment='namsa_gb300 supercell'):
    """Write the XYZ layout read by the reference (two header lines, one footer line)."""
    with open(path, 'w') as f:
        f.write(f'{len(sites)}\n{comment}\n')
        for r in sites:
            f.write(f"{int(r['atomic_number'])} {r['x']:.6f} {r['y']:.6f} {r['z']:.6f} {r['occ']:.4f} {r['DW']:.4f}\n")
        f.write('-1\n')
