"""msx_multislice_noalloc, the entry point for callers that cannot allocate
device memory (their memory belongs to their own pool or allocator, their host
forbids allocation in callbacks, or they cannot afford cudaMalloc's implicit
device synchronisation).  It must give the same CBED stack as msx_multislice
with a plan, and keep doing so on back-to-back calls that reuse its static
scratch.  Collected last so a failure here leaves every other test run."""
import ctypes

import numpy as np
import pytest
import torch

from namsa_gb300 import _lib, engine

pytestmark = pytest.mark.gpu
DEV = 'cuda'
_vp = ctypes.c_void_p


def _case(n, S, P, seed):
    rng = np.random.default_rng(seed)
    kmax = np.float32(n / 20.0)
    lam = 0.025
    ky = (np.arange(n) * float(kmax) / (n - 1) - float(kmax) / 2)
    k = np.sqrt(ky[:, None] ** 2 + ky[None, :] ** 2)
    psik = ((k < 1.0) * np.exp(-1j * 3.0 * k ** 2)).astype(np.complex64)
    norm = float(n * n * np.sum(np.abs(psik.astype(np.complex128)) ** 2))
    trans = np.exp(0.3j * rng.standard_normal((S, n, n))).astype(np.complex64)
    pos = rng.uniform(-8, 8, size=(P, 2)).astype(np.float32)
    to = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(DEV)
    return to(trans), to(psik), torch.tensor([norm], dtype=torch.float64, device=DEV), to(pos), kmax, lam


def _noalloc(trans, psik, norm, pos, kmax, lam, slice_t, k_band, crop, out):
    S, ny, nx = trans.shape
    rc = _lib.load().msx_multislice_noalloc(
        _vp(trans.data_ptr()), S, _vp(psik.data_ptr()), _vp(norm.data_ptr()), _vp(pos.data_ptr()), pos.shape[0],
        ny, nx, float(kmax), float(lam), float(slice_t), float(k_band), _vp(out.data_ptr()), crop, crop,
        _vp(torch.cuda.current_stream().cuda_stream))
    _lib.check(rc)
    return out


def _rel_l2(a, b):
    a, b = a.double(), b.double()
    return (torch.linalg.vector_norm(a - b, dim=(1, 2)) / torch.linalg.vector_norm(b, dim=(1, 2))).max().item()


@pytest.mark.parametrize('n,S,P,crop', [(256, 6, 70, 128), (1024, 2, 5, 512)])
def test_noalloc_matches_plan_twice(n, S, P, crop):
    trans, psik, norm, pos, kmax, lam = _case(n, S, P, seed=n)
    k_band = np.float32(float(kmax) / 3)
    plan = engine.Plan(n, n)
    ref = plan.multislice(trans, psik, norm, pos, kmax, lam, 1.5, k_band, crop=crop)
    for _ in range(2):  # the second call starts from the first call's scratch contents
        out = torch.full((P, crop, crop), float('nan'), dtype=torch.float32, device=DEV)
        _noalloc(trans, psik, norm, pos, kmax, lam, 1.5, k_band, crop, out)
        torch.cuda.synchronize()
        assert torch.isfinite(out).all()
        assert _rel_l2(out, ref) < 2e-5
    plan.close()


def test_noalloc_rejects_oversized_grid():
    lib = _lib.load()
    rc = lib.msx_multislice_noalloc(None, 1, None, None, None, 1, 2048, 2048, 1.0, 0.025, 1.0, 0.3, None, 1, 1, None)
    assert rc == _lib.MSX_ERR_INVALID
    assert 'static scratch holds 33554432 bytes' in _lib.last_error()
