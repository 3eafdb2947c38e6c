"""The corrector's CUDA forward/backward against the FP64 oracle
(oracle/corrector_oracle.py, itself checked by finite differences)."""
import numpy as np
import pytest
import torch

from namsa_gb300 import engine
from oracle import corrector_oracle as CO

pytestmark = pytest.mark.gpu
DEV = 'cuda'


@pytest.mark.parametrize('C,L,B,H,W', [(8, 2, 2, 32, 32), (32, 4, 2, 64, 48)])
def test_corrector_loss_and_gradients(C, L, B, H, W):
    rng = np.random.default_rng(C + L)
    flat = CO.init_params(C, L, seed=3)
    flat += 0.05 * rng.standard_normal(flat.shape) / np.sqrt(C)
    psi_c = (rng.standard_normal((B, H, W)) + 1j * rng.standard_normal((B, H, W))).astype(np.complex64)
    tc = np.exp(1j * rng.uniform(0, 1, (B, H, W))).astype(np.complex64)
    psi_f = (psi_c + 0.1 * (rng.standard_normal((B, H, W)) + 1j * rng.standard_normal((B, H, W)))).astype(np.complex64)
    denom = float(np.sum(np.abs(psi_f.astype(np.complex128) - psi_c) ** 2))
    net = engine.Corrector(H, W, C, L, max_batch=B)
    assert net.count == flat.size
    net.params.copy_(torch.from_numpy(flat.astype(np.float32)))
    d = lambda a: torch.from_numpy(a).to(DEV)
    pred = net.forward(d(psi_c), d(tc)).cpu().numpy()
    # per-sample weights scale each sample's contribution to the loss
    wts = np.array([0.5, 2.0][:B], np.float32)
    loss_w = net.loss_grad(d(psi_c), d(tc), d(psi_f), denom, weights=d(wts)).item()
    loss = net.loss_grad(d(psi_c), d(tc), d(psi_f), denom).item()
    g = net.grads.cpu().numpy().astype(np.float64)
    ref_pred, _ = CO.forward(flat.astype(np.float32).astype(np.float64), psi_c.astype(np.complex128),
                             tc.astype(np.complex128), C, L)
    ref_loss, ref_g = CO.loss_grad(flat.astype(np.float32).astype(np.float64), psi_c.astype(np.complex128),
                                   tc.astype(np.complex128), psi_f.astype(np.complex128), denom, C, L)
    assert np.abs(pred - ref_pred).max() < 1e-4 * np.abs(ref_pred).max()
    assert abs(loss - ref_loss) < 1e-4 * abs(ref_loss)
    per_sample = np.sum(np.abs(ref_pred - psi_f) ** 2, axis=(1, 2)) / denom
    assert abs(loss_w - float(np.sum(wts * per_sample))) < 1e-4 * abs(loss_w)
    off, _ = CO.layout(C, L)
    for name, (o, s) in off.items():
        err = np.linalg.norm(g[o:o + s] - ref_g[o:o + s]) / max(np.linalg.norm(ref_g[o:o + s]), 1e-12)
        assert err < 1e-3, (name, err)
    # one Adam step moves the parameters against the gradient
    before = net.params.clone()
    net.adam(lr=1e-3)
    step = (net.params - before).cpu().numpy()
    assert (np.sign(step[np.abs(g) > 1e-6]) == -np.sign(g[np.abs(g) > 1e-6])).all()
    net.close()


def test_corrector_training_improves_on_coarse_steps():
    """A small corrector trained on device-generated pairs (Si [001], 64^2,
    fine slices a/4, coarse 4x) lowers the error of single coarse steps on
    held-out probe positions, judged by plain fine-slice multislice.  (Repeated
    application over a full thickness is measured, not asserted, by bench.py
    --workload corrector.)"""
    from namsa_gb300 import corrector as CR, structures
    torch.cuda.set_device(0)
    cr = CR.Crystal(structures.silicon((1, 1, 12)), 64, 5.431 / 4)
    rng = np.random.default_rng(0)
    train_pos = rng.uniform(0, 5.431, size=(24, 2))
    test_pos = rng.uniform(0, 5.431, size=(6, 2))
    c, f, k = cr.pairs(train_pos)
    t = cr.trans_coarse[k].contiguous()
    net = engine.Corrector(64, 64, channels=16, layers=2, max_batch=16)
    net.params.copy_(torch.from_numpy(CR.init_params(16, 2, seed=0)))
    losses = CR.train(net, c, f, t, steps=400, batch=16, lr=2e-3)
    assert np.mean(losses[-50:]) < 0.9 * np.mean(losses[:10])
    hc, hf, hk = cr.pairs(test_pos)
    ht = cr.trans_coarse[hk].contiguous()
    err_c = (hf - hc).abs().pow(2).sum().item()
    pred = torch.cat([net.forward(hc[i:i + 16].contiguous(), ht[i:i + 16].contiguous()) for i in range(0, hc.shape[0], 16)])
    err_p = (hf - pred).abs().pow(2).sum().item()
    assert err_p < 0.95 * err_c, (err_p, err_c)
    net.close()
