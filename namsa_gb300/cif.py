"""Minimal CIF reader and orthogonal supercell tiling (no pymatgen).

Covers the part of namsa's ``SupercellBuilder`` (namsa/supercell.py:56-465)
that feeds the multislice path:

* ``read_cif`` parses the cell parameters, the symmetry operations
  (``_symmetry_equiv_pos_as_xyz`` or ``_space_group_symop_operation_xyz``)
  and the atom sites of a CIF file (the fields ``SupercellBuilder.__init__``
  reads through pymatgen's ``CifParser``, supercell.py:80-114).
* ``unit_cell`` expands the sites by the symmetry operations like
  ``build_unit_cell`` (supercell.py:233-273): every operation applied to every
  site, wrapped into [0, 1), duplicates removed by their coordinates rounded
  to 2 decimals (in that sorted order), Cartesian positions from the lattice
  matrix.  P1 files and centred cells whose centring translations are listed
  among the operations are both covered.
* ``orthogonal_supercell`` tiles an orthogonal cell (all angles 90 degrees)
  into the structured array ``MSAGPU`` takes, with the inclusive bounds of
  ``make_orthogonal_supercell`` (supercell.py:444).

The lattice matrix follows pymatgen's ``Lattice.from_parameters`` convention,
which ``SupercellBuilder`` inherits (its ``basis`` holds the lattice vectors
as columns): a = (a sin(beta), 0, a cos(beta)),
b = (-b sin(alpha) cos(gamma*), b sin(alpha) sin(gamma*), b cos(alpha)),
c = (0, 0, c) with cos(gamma*) = (cos(alpha) cos(beta) - cos(gamma)) /
(sin(alpha) sin(beta)).

Debye-Waller factors: the reference's parse of ``_atom_site_B_iso_or_equiv``
/ ``_U_iso_or_equiv`` always falls through to its default of 0.07 (it divides
a list of strings by a float inside a ``try``), so ``dw='reference'`` (the
default) reproduces that; ``dw='file'`` takes U_iso, or B_iso / (8 pi^2),
from the file where present.
"""
from __future__ import annotations

import re

import numpy as np

from .structures import XYZ_dtype

# Chemical symbols by atomic number (1..103), the range of the Kirkland table.
SYMBOLS = ('H He Li Be B C N O F Ne Na Mg Al Si P S Cl Ar K Ca Sc Ti V Cr Mn Fe Co Ni Cu Zn Ga Ge As Se Br Kr '
           'Rb Sr Y Zr Nb Mo Tc Ru Rh Pd Ag Cd In Sn Sb Te I Xe Cs Ba La Ce Pr Nd Pm Sm Eu Gd Tb Dy Ho Er Tm Yb '
           'Lu Hf Ta W Re Os Ir Pt Au Hg Tl Pb Bi Po At Rn Fr Ra Ac Th Pa U Np Pu Am Cm Bk Cf Es Fm Md No Lr').split()
Z_OF = {s: i + 1 for i, s in enumerate(SYMBOLS)}

SITES_dtype = [('atom_type', '<U16'), ('atomic_number', 'i'), ('frac_x', 'f'), ('frac_y', 'f'), ('frac_z', 'f'),
               ('occ', 'f'), ('DW', 'f')]
DEFAULT_DW = 0.07


def atomic_number(symbol):
    """Atomic number of a site's type symbol ('Fe', 'Fe3+', 'O2-', 'Si1' ...)."""
    m = re.match(r'([A-Z][a-z]?)', symbol.strip())
    if not m or m.group(1) not in Z_OF:
        raise ValueError(f'unknown element symbol {symbol!r}')
    return Z_OF[m.group(1)]


def _number(tok):
    """CIF numeric value: strips a standard uncertainty in parentheses, '.' and '?' are missing."""
    tok = tok.strip()
    if tok in ('.', '?'):
        return None
    return float(re.sub(r'\(\d+\)$', '', tok))


def _tokens(line):
    """Whitespace-separated tokens of a CIF line; quoted strings stay whole."""
    out, i, n = [], 0, len(line)
    while i < n:
        ch = line[i]
        if ch.isspace():
            i += 1
        elif ch == '#':
            break
        elif ch in '\'"':
            j = i + 1
            while j < n and not (line[j] == ch and (j + 1 == n or line[j + 1].isspace())):
                j += 1
            out.append(line[i + 1:j])
            i = j + 1
        else:
            j = i
            while j < n and not line[j].isspace():
                j += 1
            out.append(line[i:j])
            i = j
    return out


def parse_cif_blocks(text):
    """First data block of a CIF text as {tag: value} for single items and
    {tag: [values]} for loop columns (tags lower-cased)."""
    items = {}
    lines = text.splitlines()
    i, n = 0, len(lines)
    started = False
    while i < n:
        raw = lines[i]
        s = raw.strip()
        if not s or s.startswith('#'):
            i += 1
            continue
        if s.lower().startswith('data_'):
            if started:
                break
            started = True
            i += 1
            continue
        if s.startswith(';'):  # multi-line text field of a previous tag: skip it
            i += 1
            while i < n and not lines[i].startswith(';'):
                i += 1
            i += 1
            continue
        if s.lower() == 'loop_' or s.lower().startswith('loop_'):
            i += 1
            tags = []
            while i < n and lines[i].strip().startswith('_'):
                tags.append(lines[i].strip().split()[0].lower())
                i += 1
            vals = []
            while i < n:
                t = lines[i].strip()
                if not t or t.startswith('#'):
                    i += 1
                    continue
                if t.startswith('_') or t.lower().startswith('loop_') or t.lower().startswith('data_'):
                    break
                if t.startswith(';'):
                    i += 1
                    buf = []
                    while i < n and not lines[i].startswith(';'):
                        buf.append(lines[i])
                        i += 1
                    vals.append('\n'.join(buf))
                    i += 1
                    continue
                vals.extend(_tokens(lines[i]))
                i += 1
            if tags:
                if len(vals) % len(tags):
                    raise ValueError(f'CIF loop over {tags[0]}... has {len(vals)} values for {len(tags)} columns')
                for k, tag in enumerate(tags):
                    items[tag] = vals[k::len(tags)]
            continue
        if s.startswith('_'):
            toks = _tokens(s)
            tag = toks[0].lower()
            if len(toks) > 1:
                items[tag] = ' '.join(toks[1:])
                i += 1
            else:  # value on the next line (possibly a ; text field)
                i += 1
                if i < n and lines[i].startswith(';'):
                    i += 1
                    buf = []
                    while i < n and not lines[i].startswith(';'):
                        buf.append(lines[i])
                        i += 1
                    items[tag] = '\n'.join(buf)
                    i += 1
                elif i < n:
                    items[tag] = ' '.join(_tokens(lines[i]))
                    i += 1
            continue
        i += 1
    return items


def parse_symop(expr):
    """4x4 affine matrix of a symmetry operation such as '-x+1/2, y+1/2, -z'."""
    parts = [p.strip().lower().replace(' ', '') for p in expr.split(',')]
    if len(parts) != 3:
        raise ValueError(f'symmetry operation {expr!r} does not have three components')
    m = np.zeros((4, 4))
    m[3, 3] = 1.0
    for row, p in enumerate(parts):
        for sign, body in re.findall(r'([+-]?)([^+-]+)', p):
            sgn = -1.0 if sign == '-' else 1.0
            var = re.fullmatch(r'(?:(\d*\.?\d+(?:/\d+)?)\*?)?([xyz])', body)
            if var:
                coef = 1.0 if not var.group(1) else _fraction(var.group(1))
                m[row, 'xyz'.index(var.group(2))] += sgn * coef
            else:
                m[row, 3] += sgn * _fraction(body)
    return m


def _fraction(tok):
    if '/' in tok:
        a, b = tok.split('/')
        return float(a) / float(b)
    return float(tok)


def lattice_matrix(a, b, c, alpha, beta, gamma):
    """Rows = lattice vectors a, b, c in Cartesian Angstrom (angles in degrees)."""
    al, be, ga = np.radians([alpha, beta, gamma])
    val = (np.cos(al) * np.cos(be) - np.cos(ga)) / (np.sin(al) * np.sin(be))
    gs = np.arccos(np.clip(val, -1.0, 1.0))
    return np.array([[a * np.sin(be), 0.0, a * np.cos(be)],
                     [-b * np.sin(al) * np.cos(gs), b * np.sin(al) * np.sin(gs), b * np.cos(al)],
                     [0.0, 0.0, c]])


class CifStructure:
    """Cell, symmetry operations and asymmetric-unit sites of a CIF file.

    Attributes: ``lattice_const`` (a, b, c), ``lattice_angles`` (alpha, beta,
    gamma in degrees), ``basis`` (3x3, lattice vectors as columns, like
    ``SupercellBuilder.basis``), ``sym_ops`` (list of 4x4 affine matrices on
    fractional coordinates) and ``sites`` (structured array of SITES_dtype)."""

    def __init__(self, text, dw='reference'):
        items = parse_cif_blocks(text)
        try:
            self.lattice_const = np.array([_number(items['_cell_length_' + k]) for k in 'abc'])
            self.lattice_angles = np.array([_number(items['_cell_angle_' + k]) for k in ('alpha', 'beta', 'gamma')])
        except KeyError as e:
            raise ValueError(f'CIF lacks the cell parameter {e.args[0]}') from None
        self.basis = lattice_matrix(*self.lattice_const, *self.lattice_angles).T
        ops = None
        for tag in ('_symmetry_equiv_pos_as_xyz', '_space_group_symop_operation_xyz', '_space_group_symop.operation_xyz'):
            if tag in items:
                ops = items[tag]
                break
        if ops is None:
            ops = ['x, y, z']
        if isinstance(ops, str):
            ops = [ops]
        self.sym_ops = [parse_symop(o) for o in ops]
        fx, fy, fz = (items.get('_atom_site_fract_' + k) for k in 'xyz')
        if fx is None or fy is None or fz is None:
            raise ValueError('CIF lacks fractional atom-site coordinates (_atom_site_fract_x/y/z)')
        labels = items.get('_atom_site_label', [''] * len(fx))
        symbols = items.get('_atom_site_type_symbol', labels)
        occ = items.get('_atom_site_occupancy', ['1'] * len(fx))
        dws = np.full(len(fx), DEFAULT_DW)
        if dw == 'file':
            if '_atom_site_u_iso_or_equiv' in items:
                dws = np.array([_number(v) or DEFAULT_DW for v in items['_atom_site_u_iso_or_equiv']])
            elif '_atom_site_b_iso_or_equiv' in items:
                dws = np.array([(_number(v) / (8 * np.pi ** 2)) if _number(v) is not None else DEFAULT_DW
                                for v in items['_atom_site_b_iso_or_equiv']])
        elif dw != 'reference':
            raise ValueError("dw must be 'reference' or 'file'")
        rows = []
        for sym, x, y, z, o, d in zip(symbols, fx, fy, fz, occ, dws):
            o = _number(o)
            rows.append((sym, atomic_number(sym), _number(x), _number(y), _number(z), 1.0 if o is None else o, d))
        self.sites = np.array(rows, dtype=SITES_dtype)

    @property
    def orthogonal(self):
        return bool(np.all(np.abs(self.lattice_angles - 90.0) < 1e-6))


def read_cif(path_or_text, dw='reference'):
    """CifStructure of a CIF file path or of CIF text."""
    text = path_or_text
    if '\n' not in path_or_text and not path_or_text.lstrip().startswith(('data_', '#', '_', 'loop_')):
        with open(path_or_text) as f:
            text = f.read()
    return CifStructure(text, dw=dw)


def unit_cell(cif):
    """Symmetry-expanded unit cell (supercell.py:233-273).

    Returns a structured array with fields atom_type, atomic_number,
    frac_x/y/z, x, y, z (Cartesian Angstrom), occ, DW.  Per site, positions
    keep the order of the unique rounded coordinates."""
    dtype = SITES_dtype[:5] + [('x', 'f8'), ('y', 'f8'), ('z', 'f8')] + SITES_dtype[5:]
    out = []
    for site in cif.sites:
        p = np.array([site['frac_x'], site['frac_y'], site['frac_z'], 1.0], dtype=np.float64)
        sym = np.array([op @ p for op in cif.sym_ops])[:, :3]
        sym -= sym // 1
        _, idx = np.unique(np.round(sym, 2), return_index=True, axis=0)
        uc = sym[idx]
        xyz = (cif.basis @ uc.T).T
        for f, r in zip(uc, xyz):
            out.append((site['atom_type'], site['atomic_number'], f[0], f[1], f[2], r[0], r[1], r[2], site['occ'],
                        site['DW']))
    return np.array(out, dtype=dtype)


def orthogonal_supercell(cif, cells):
    """XYZ structured array (atomic_number, x, y, z, occ, DW) of an orthogonal
    cell tiled ``cells`` = (nx, ny, nz) times along a, b, c, keeping every atom
    with 0 <= r <= size on each axis (supercell.py:444)."""
    if not cif.orthogonal:
        raise ValueError('orthogonal_supercell needs a cell with all angles at 90 degrees, got %s'
                         % np.round(cif.lattice_angles, 4).tolist())
    uc = unit_cell(cif)
    cells = np.asarray(cells, dtype=np.int64)
    a = cif.lattice_const
    frac = np.column_stack([uc['frac_x'], uc['frac_y'], uc['frac_z']]).astype(np.float64)
    grid = np.stack(np.meshgrid(*[np.arange(k + 1) for k in cells], indexing='ij'), -1).reshape(-1, 3)
    pos = (grid[:, None, :] + frac[None, :, :]).reshape(-1, 3) * a
    rep = lambda f: np.tile(uc[f], len(grid))
    size = cells * a
    keep = np.all((pos >= 0) & (pos <= size + 1e-6), axis=1)
    out = np.zeros(int(keep.sum()), dtype=XYZ_dtype)
    out['atomic_number'] = rep('atomic_number')[keep]
    out['x'], out['y'], out['z'] = pos[keep, 0], pos[keep, 1], pos[keep, 2]
    out['occ'] = rep('occ')[keep]
    out['DW'] = rep('DW')[keep]
    return out
