"""msx_multislice_noalloc, the entry point for callers that cannot allocate
device memory (their memory belongs to their own pool or allocator, their host
forbids allocation in callbacks, or they cannot afford cudaMalloc's implicit
device synchronisation).  It must give the same CBED stack as msx_multislice
with a plan and as the FP64 oracle, and keep doing so on back-to-back calls
that reuse its static scratch.  The cases cover every radix layout of the
first schedule of each line length (two-stage 256, 512 and 1024, three-stage
384 and 768), a rectangular grid, ragged groups and the probe-only branch.
Collected last so a failure here leaves every other test run."""
import ctypes

import numpy as np
import pytest
import torch

from namsa_gb300 import _lib, engine
from oracle import msa_oracle as O

pytestmark = pytest.mark.gpu
DEV = 'cuda'
_vp = ctypes.c_void_p
LAM = 0.025
SLICE_T = 1.5
BW = 1 / 3


def _geom(ny, nx, kmax):
    g = O.Geometry.__new__(O.Geometry)
    g.sampling = np.array([ny, nx])
    g.kmax = kmax
    g.lam = LAM
    return g


def _case(ny, nx, S, P, seed):
    rng = np.random.default_rng(seed)
    kmax = np.float32(min(ny, nx) / 20.0)
    ky = O.kgrid_gpu(kmax, ny)[:, None]
    kx = O.kgrid_gpu(kmax, nx)[None, :]
    k = np.sqrt(ky ** 2 + kx ** 2)
    psik = ((k < 1.0) * np.exp(-1j * 3.0 * k ** 2)).astype(np.complex64)
    norm = float(ny * nx * np.sum(np.abs(psik.astype(np.complex128)) ** 2))
    trans = np.exp(0.3j * rng.standard_normal((S, ny, nx))).astype(np.complex64)
    pos = rng.uniform(-8, 8, size=(P, 2)).astype(np.float32)
    return trans, psik, norm, pos, kmax


def _noalloc(trans, S, psik, norm, pos, kmax, k_band, crop, out):
    ny, nx = psik.shape
    rc = _lib.load().msx_multislice_noalloc(
        _vp(trans.data_ptr()), S, _vp(psik.data_ptr()), _vp(norm.data_ptr()), _vp(pos.data_ptr()),
        pos.shape[0], ny, nx, float(kmax), LAM, SLICE_T, float(k_band), _vp(out.data_ptr()), crop[0], crop[1],
        _vp(torch.cuda.current_stream().cuda_stream))
    _lib.check(rc)
    return out


def _rel_l2(a, b):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    return (np.linalg.norm((a - b).reshape(len(a), -1), axis=1) / np.linalg.norm(b.reshape(len(b), -1), axis=1)).max()


@pytest.mark.parametrize('ny,nx,S,P,crop', [(256, 256, 6, 70, 128), (384, 512, 3, 9, 256), (512, 512, 3, 7, 256),
                                            (768, 768, 2, 3, 512), (1024, 1024, 2, 5, 512), (256, 256, 0, 4, 256)])
def test_noalloc_matches_plan_and_oracle_twice(ny, nx, S, P, crop):
    trans, psik, norm, pos, kmax = _case(ny, nx, S, P, seed=ny + nx + S)
    k_band = np.float32(BW * float(kmax))
    d_trans = torch.from_numpy(trans if S else np.zeros((1, ny, nx), np.complex64)).to(DEV)
    d_psik = torch.from_numpy(psik).to(DEV)
    d_norm = torch.tensor([norm], dtype=torch.float64, device=DEV)
    d_pos = torch.from_numpy(pos).to(DEV)
    plan = engine.Plan(ny, nx)
    ref = plan.multislice(d_trans[:S], d_psik, d_norm, d_pos, kmax, LAM, SLICE_T, k_band, crop=crop).cpu().numpy()
    plan.close()
    pick = [0, P - 1]
    Pm, _ = O.propagator_gpu(_geom(ny, nx, kmax), SLICE_T, BW)
    fp64 = O.multislice_gpu(trans.astype(np.complex128), psik.astype(np.complex128), Pm, pos[pick], norm,
                            _geom(ny, nx, kmax), crop=crop)
    for _ in range(2):  # the second call starts from the first call's scratch contents
        out = torch.full((P, crop, crop), float('nan'), dtype=torch.float32, device=DEV)
        _noalloc(d_trans, S, d_psik, d_norm, d_pos, kmax, k_band, (crop, crop), out)
        torch.cuda.synchronize()
        got = out.cpu().numpy()
        assert np.isfinite(got).all()
        assert _rel_l2(got, ref) < 2e-5
        assert _rel_l2(got[pick], fp64) < 2e-5


def test_noalloc_rejects_oversized_grid():
    lib = _lib.load()
    rc = lib.msx_multislice_noalloc(None, 1, None, None, None, 1, 2048, 2048, 1.0, 0.025, 1.0, 0.3, None, 1, 1, None)
    assert rc == _lib.MSX_ERR_INVALID
    assert 'static scratch holds 33554432 bytes' in _lib.last_error()
