"""Host-side logic of the MSAGPU surface against the oracle and the golden
fixtures made from the reference.  CPU only (no CUDA calls)."""
import os

import numpy as np
import pytest

from namsa_gb300 import msa as M
from namsa_gb300 import optics
from oracle import msa_oracle as O

G = os.path.join(os.path.dirname(__file__), 'golden')


def test_optics_match_golden():
    g = np.load(os.path.join(G, 'optics.npz'))
    np.testing.assert_allclose(optics.voltage2Lambda(g['volts']), g['lam'], rtol=1e-15)
    np.testing.assert_allclose(optics.sigma_int(g['volts']), g['sigma'], rtol=1e-15)
    np.testing.assert_allclose(optics.scherzer_defocus(g['lam'], 1e4), g['scherzer_c1'], rtol=1e-15)


def test_kirkland_table():
    k = M.kirkland_table()
    assert k.shape == (103, 4, 3) and k.dtype == np.float64
    assert np.all(k[:, 1] > 0) and np.all(k[:, 3] > 0)


@pytest.mark.parametrize('cells,n,t,expected', [((4, 4, 20), 256, 5.431 / 4, 80), ((8, 8, 50), 512, 5.431 / 4, 199)])
def test_num_slices(cells, n, t, expected):
    sc = O.si_supercell(*cells)
    xyz = np.column_stack([sc['x'], sc['y'], sc['z']]).astype(np.float32)
    dims = xyz.max(0) - xyz.min(0)
    assert M.num_slices_of(dims[-1], t) == expected
    geom = O.Geometry(xyz, sc['atomic_number'], 100., 20e-3, [n, n])
    assert geom.num_slices(t) == expected


def test_slice_sites_match_oracle():
    sc = O.srtio3_supercell(3, 3, 4)
    xyz = np.column_stack([sc['x'], sc['y'], sc['z']]).astype(np.float32)
    geom = O.Geometry(xyz, sc['atomic_number'], 300., 25e-3, [128, 128])
    t = 3.905 / 2
    S = geom.num_slices(t)
    sites, offs = M.slice_sites(xyz, sc['atomic_number'], geom.pix_size, t, S)
    ref = O.slice_sites_gpu(geom, t)
    assert len(offs) == S + 1 and offs[-1] == sum(len(r) for r in ref)
    for s in range(S):
        np.testing.assert_array_equal(sites[offs[s]:offs[s + 1], :3], ref[s])
    assert sites.dtype == np.int32 and sites.shape[1] == 4


def test_window_grid():
    sc = O.si_supercell(4, 4, 20)
    xyz = np.column_stack([sc['x'], sc['y'], sc['z']]).astype(np.float32)
    geom = O.Geometry(xyz, sc['atomic_number'], 100., 20e-3, [256, 256])
    assert M.window_grid(geom.pix_size) == (188, 188)


@pytest.mark.parametrize('name,kw', [
    ('steps', dict(probe_step=np.array([0.5, 0.5]), probe_range=np.array([[0.25, 0.75], [0.25, 0.75]]))),
    ('grid2', dict(grid_steps=np.array([4, 6]), fraction=0.25, origin=np.array([0.1, 0.2]))),
])
def test_positions_match_golden(name, kw):
    g = np.load(os.path.join(G, 'positions.npz'))
    pos, st, rg = M.probe_positions_grid(g['dims'], **kw)
    np.testing.assert_array_equal(pos, g[name + '_pos'])
    np.testing.assert_array_equal(st, g[name + '_steps'])
    np.testing.assert_array_equal(rg, g[name + '_range'])


def test_plan_heuristic():
    # 1024 probes of 512^2 need 2 GiB: with 3 GB free the reference halves... by 0.75 steps
    n = M.max_probes_for(1024, np.array([512, 512]), 0, 3e9)
    assert n * 512 * 512 * 8 / 1024e6 <= 0.5 * 3e9 / 1024e6
    assert int(n / 0.75) * 512 * 512 * 8 / 1024e6 > 0.5 * 3e9 / 1024e6 or n == 1024
    assert M.max_probes_for(10, np.array([64, 64]), 0, 1e12) == 10


def test_supercell_loader_and_detector(tmp_path):
    sc = O.si_supercell(1, 1, 1)
    arr = M.load_supercell(sc)
    assert arr is not sc and len(arr) == len(sc)
    p = tmp_path / 'si.xyz'
    with open(p, 'w') as f:
        f.write(f'{len(sc)}\ncomment\n')
        for r in sc:
            f.write(f"{r['atomic_number']} {r['x']} {r['y']} {r['z']} {r['occ']} {r['DW']}\n")
        f.write('-1\n')
    arr2 = M.load_supercell(str(p))
    np.testing.assert_allclose(arr2['x'], sc['x'], rtol=1e-6)
    det = M.annular_detector(np.array([64, 64]), np.array([0.1, 0.1]), 0.025, 0.05, 0.1)
    assert det.shape == (64, 64) and det.dtype == bool and 0 < det.sum() < 64 * 64


def _col_wavefronts(words):
    slots = {}
    for w in set(words):
        slots.setdefault(w % 16, set()).add(w)
    return max(len(v) for v in slots.values())


@pytest.mark.parametrize('n,rads', [(256, (16, 16)), (384, (8, 8, 6)), (512, (32, 16))])
def test_warp_column_layout_is_bank_conflict_free(n, rads):
    """Index-level check of the warp-owned column pass layout (csrc/msx_tma.cuh,
    col_mid_warp_kernel): 16 threads per column, lane = 2 t + c_local, tile rows of
    16 complex64 stored with the 128-byte swizzle (chunk j of row r at j ^ (r & 7)),
    exchange slot of element i at row i ^ ((i >> log2(first radix)) & 7).  Every
    warp access (natural-order load, Stockham scatters and gathers of each stage)
    must take two 128-byte wavefronts, the minimum for 32 eight-byte lanes."""
    T = 16
    E = n // T
    sh = int(np.log2(rads[0]))

    def perm(i):
        return i ^ ((i >> sh) & 7)

    def addr(row, c):
        return row * 16 + (((c >> 1) ^ (row & 7)) << 1) + (c & 1)

    assert sorted(perm(i) for i in range(n)) == list(range(n))
    for warp in range(8):
        lanes = [(l >> 1, 2 * warp + (l & 1)) for l in range(32)]
        for m in range(E):
            assert _col_wavefronts([addr(t + T * m, c) for t, c in lanes]) == 2
        ns = 1
        for si, R in enumerate(rads):
            if si < len(rads) - 1:
                for q in range(E // R):
                    for r in range(R):
                        ws = []
                        for t, c in lanes:
                            j = t + T * q
                            ws.append(addr(perm((j // ns) * ns * R + (j % ns) + r * ns), c))
                        assert _col_wavefronts(ws) == 2
                for m in range(E):
                    assert _col_wavefronts([addr(perm(t + T * m), c) for t, c in lanes]) == 2
            ns *= R


def test_band_columns_contain_every_column_the_mask_keeps():
    """msx_band_columns: every column with a row that passes the float32 mask test
    (|k| on the centred grid, as the device computes it) lies inside [x_lo, x_hi);
    the range is tile-aligned and inside the grid."""
    from namsa_gb300 import engine
    rng = np.random.default_rng(5)
    for _ in range(60):
        nx = int(rng.choice([64, 128, 256, 384, 512, 768, 1024]))
        ny = int(rng.choice([64, 256, 512]))
        tile = int(rng.choice([8, 16, 32]))
        kmax = np.float32(rng.uniform(2, 40))
        k_band = np.float32(kmax * rng.uniform(0.05, 0.6))
        lo, hi = engine.band_columns(nx, kmax, k_band, tile)
        assert 0 <= lo < hi <= nx and lo % tile == 0 and (hi % tile == 0 or hi == nx)
        km = np.float64(kmax)
        kx = np.arange(nx, dtype=np.float64) * km / (nx - 1) - km / 2.0
        ky = np.arange(ny, dtype=np.float64) * km / (ny - 1) - km / 2.0
        k = np.sqrt(kx[None, :] * kx[None, :] + ky[:, None] * ky[:, None]).astype(np.float32)
        kept = np.nonzero((k < k_band).any(axis=0))[0]
        if kept.size:
            assert lo <= kept.min() and kept.max() < hi, (nx, tile, lo, hi, kept.min(), kept.max())


def test_distinct_slices_groups_bitwise_equal_inputs():
    """The corrector runs its network once per group of coarse slices with bitwise equal
    inputs; a slice that differs in one value keeps its own group."""
    import torch
    from namsa_gb300 import corrector as CR
    g = torch.Generator().manual_seed(0)
    f = torch.randn(8, 6, 5, 6, generator=g)
    f[3] = f[0]
    f[5] = f[1]
    f[4] = f[0].clone()
    f[4][2, 3, 1] += 0.25
    f[6] = f[4]
    f[7] = f[0]
    first, index = CR.distinct_slices(f)
    assert first == [0, 1, 2, 4]
    assert index == [0, 1, 2, 0, 3, 1, 3, 0]
    for s, j in enumerate(index):
        assert torch.equal(f[s], f[first[j]])
