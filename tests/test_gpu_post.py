"""Dataset post-processing and the integrated-potential slice source on the
device, against the oracle (which is pinned to the reference's own functions
by tests/golden/postproc.npz and integrated.npz)."""
import os

import numpy as np
import pytest
import torch

from namsa_gb300 import engine
from oracle import msa_oracle as O

pytestmark = pytest.mark.gpu
DEV = 'cuda'
G = os.path.join(os.path.dirname(__file__), 'golden')


def _fp16_close(a, b, ulps=2):
    a = np.asarray(a, np.float32)
    b = np.asarray(b, np.float32)
    tol = ulps * np.maximum(np.abs(b), 1e-3) * 2 ** -10
    assert (np.abs(a - b) <= tol).all(), np.abs(a - b).max()


def test_process_cbed_golden_and_random():
    g = np.load(os.path.join(G, 'postproc.npz'))
    out = engine.process_cbed(torch.from_numpy(g['cbed']).to(DEV)).cpu().numpy()
    _fp16_close(out, g['cbed_out'])
    rng = np.random.default_rng(3)
    x = rng.gamma(0.5, 1e-3, size=(5, 256, 256)).astype(np.float32)
    _fp16_close(engine.process_cbed(torch.from_numpy(x).to(DEV)).cpu().numpy(), O.process_cbed(x))


def test_process_potential_golden_and_random():
    g = np.load(os.path.join(G, 'postproc.npz'))
    out = engine.process_potential(torch.from_numpy(g['trans']).to(DEV)).cpu().numpy()
    _fp16_close(out, g['pot_out'])
    rng = np.random.default_rng(4)
    t = np.exp(1j * rng.uniform(0, 0.7, size=(7, 128, 128))).astype(np.complex64)
    _fp16_close(engine.process_potential(torch.from_numpy(t).to(DEV)).cpu().numpy(), O.process_potential(t))


def test_integrate_potential():
    g = np.load(os.path.join(G, 'integrated.npz'))
    sigma = float(g['sigma'])
    t = engine.integrate_potential(torch.from_numpy(g['pot']).to(DEV), torch.from_numpy(g['z']).to(DEV),
                                   g['slices'].shape[0], np.float32(sigma)).cpu().numpy()
    ref = np.exp(1j * sigma * O.integrate_potential_slices(g['pot'], g['z'], float(g['slice_t'])))
    assert t.shape == ref.shape
    assert np.abs(t - ref).max() < 2e-6
