"""The learned coarse-slice corrector on the GPU.

* Network: the CUDA forward maps and backward gradients (every contraction a
  bfloat16 tensor-core GEMM with FP32 accumulation) at 32 x 48, 64^2 and 512^2
  against the FP64 oracle
  (oracle/corrector_oracle.py, itself checked by finite differences) run with
  the same bfloat16 operand rounding, and against the plain FP64 oracle.
* Rollout adjoint: the map gradients of a windowed corrected rollout,
  back-propagated through the engine's slice step with the conjugate
  propagator, against a central difference of the loss along a random
  direction, for factors 1 + M and for unit-modulus factors exp(i Im M).
* Training: a corrector trained by rollouts on Si [001] at 256^2 (200 keV,
  fine slices a/4, coarse slices a) lowers the CBED error of 4x-thick slicing
  against plain fine slicing over 200 Angstrom on held-out probe positions, run
  through the production multislice on the effective transmission slices.
"""
import numpy as np
import pytest
import torch

from namsa_gb300 import corrector as CR, engine, structures
from oracle import corrector_oracle as CO

pytestmark = pytest.mark.gpu
DEV = 'cuda'


def _rel(a, b):
    return float(np.linalg.norm(np.ravel(a) - np.ravel(b)) / max(np.linalg.norm(np.ravel(b)), 1e-30))


@pytest.mark.parametrize('H,W,Cin,C,L,MX,MY,S', [(32, 48, 6, 8, 2, 6, 8, 3), (64, 64, 6, 32, 4, 16, 32, 2),
                                                  (512, 512, 6, 8, 1, 16, 32, 1)])
def test_network_forward_backward_match_oracle(H, W, Cin, C, L, MX, MY, S):
    torch.cuda.set_device(0)
    rng = np.random.default_rng(H + C)
    net = engine.Corrector(H, W, Cin, C, L, MX, MY, max_samples=S)
    ref = CO.Net(H, W, Cin, C, L, MX, MY, bf16_gemm=True)
    assert net.count == ref.count()
    flat = CO.init_params(ref, seed=3, out_scale=0.5)
    flat = flat + 0.02 * rng.standard_normal(flat.shape)
    flat = flat.astype(np.float32).astype(np.float64)
    net.params.copy_(torch.from_numpy(flat.astype(np.float32)))
    feats = rng.standard_normal((S, H, W, Cin)).astype(np.float32)
    maps = net.forward(torch.from_numpy(feats).to(DEV)).cpu().numpy()
    want, cache = CO.forward(ref, flat, feats.astype(np.float64))
    assert _rel(maps, want) < 3e-3, _rel(maps, want)
    plain = CO.Net(H, W, Cin, C, L, MX, MY)
    exact, _ = CO.forward(plain, flat, feats.astype(np.float64))
    assert _rel(maps, exact) < 3e-2, _rel(maps, exact)
    dmaps = rng.standard_normal(maps.shape).astype(np.float32)
    net.backward(torch.from_numpy(dmaps).to(DEV))
    net.check()
    g = net.grads.cpu().numpy().astype(np.float64)
    gref = CO.backward(ref, cache, dmaps.astype(np.float64))
    o = 0
    for name, shape in ref.layout():
        n = int(np.prod(shape))
        err = _rel(g[o:o + n], gref[o:o + n])
        assert err < 1e-2, (name, err)
        o += n
    # one Adam step moves every parameter with a clear gradient against it
    before = net.params.clone()
    net.adam(lr=1e-3)
    step = (net.params - before).cpu().numpy()
    big = np.abs(g) > 1e-3 * np.abs(g).max()
    assert (np.sign(step[big]) == -np.sign(g[big])).all()
    net.close()


def test_repeated_slices_share_their_maps():
    """The network runs once per distinct coarse slice; the maps equal those of a run
    over every slice (a periodic crystal repeats its coarse slices)."""
    torch.cuda.set_device(0)
    cr = CR.Crystal(structures.silicon((2, 2, 8)), 64, 5.431 / 4)
    net = engine.Corrector(64, 64, 6, 8, 1, 8, 16, max_samples=4)
    net.params.copy_(torch.from_numpy(CR.init_params(net, seed=0)))
    first, index = CR.distinct_slices(cr.features())
    assert len(index) == cr.coarse_steps and len(first) < cr.coarse_steps, (len(first), cr.coarse_steps)
    f = cr.features()
    for s, j in enumerate(index):
        assert torch.equal(f[s], f[first[j]])
    a = CR.crystal_maps(net, cr)
    b = CR.crystal_maps(net, cr, dedup=False)
    net.check()
    assert torch.equal(a, b)
    net.close()


@pytest.mark.parametrize('n,form', [(256, 1), (512, 1), (256, 0)])
def test_effective_slices_fold_the_corrected_steps(n, form):
    """The production multislice on the effective slices (t'_0 = b_0 t_0, t'_k = a_{k-1} b_k t_k,
    t'_S = a_{S-1}) gives the CBED of the corrected rollout run step by step (b_k t_k, coarse
    step, a_k; a last masked propagation), for random maps."""
    torch.cuda.set_device(0)
    cr = CR.Crystal(structures.silicon((4, 4, 6)), n, 5.431 / 4)
    S = cr.coarse_steps
    maps = (0.05 * torch.randn(S, n, n, 4, generator=torch.Generator().manual_seed(n + form))).to(DEV)
    pos = np.array([[0.3, 1.1], [2.0, 3.0], [4.4, 0.7]], np.float32)
    got = CR.corrected_multislice(None, cr, pos, S, trans=cr.effective_slices(maps, form)).cpu().numpy()
    w = cr.waves(pos)
    tb = torch.empty((n, n), dtype=torch.complex64, device=DEV)
    for k in range(S):
        engine.map_trans(cr.trans_coarse[k], maps[k], 1, out=tb, form=form)
        cr.plan.step_waves(w, tb, cr.ptab_coarse)
        engine.apply_map(w, maps[k], 0, form=form)
    cr.plan.step_waves(w, cr.ones, cr.ptab_coarse)
    want = cr.plan.cbed_waves(w, cr.sim.norm_dev).cpu().numpy()
    assert _rel(got, want) < 2e-5, _rel(got, want)


@pytest.mark.parametrize('form', [0, 1])
def test_rollout_adjoint_matches_central_difference(form):
    torch.cuda.set_device(0)
    cr = CR.Crystal(structures.silicon((1, 1, 6)), 64, 5.431 / 4)
    rng = np.random.default_rng(0)
    tr = cr.trajectory(rng.uniform(0, 5.431, size=(3, 2)), steps=4)
    net = engine.Corrector(64, 64, 6, 8, 1, 8, 16, max_samples=4)
    trainer = CR.RolloutTrainer(net, [cr], [tr], window=3, waves=3, form=form)
    maps = (0.05 * torch.randn(3, 64, 64, 4, generator=torch.Generator().manual_seed(1))).to(DEV)
    dmaps = torch.zeros_like(maps)
    b = torch.arange(3, device=DEV)
    trainer._window(cr, tr, 1, b, maps, dmaps)
    d = torch.randn(maps.shape, generator=torch.Generator().manual_seed(2)).to(DEV)
    eps = 2e-3

    def loss(m):
        return trainer._window(cr, tr, 1, b, m.contiguous(), torch.zeros_like(m))
    num = (loss(maps + eps * d) - loss(maps - eps * d)) / (2 * eps)
    ana = float((dmaps.double() * d.double()).sum().item())
    assert abs(num - ana) <= 2e-2 * abs(ana), (num, ana)
    net.close()


def test_trained_corrector_beats_coarse_slices_over_200A():
    torch.cuda.set_device(0)
    n = 256
    sc = structures.silicon((4, 4, 40))
    cr = CR.Crystal(sc, n, 5.431 / 4)
    steps = 37  # 37 coarse slices of a = 201 Angstrom
    assert cr.coarse_steps >= steps
    rng = np.random.default_rng(5)
    tr = cr.trajectory(rng.uniform(0, 5.431, size=(48, 2)), steps=16)
    net = engine.Corrector(n, n, 6, 32, 4, 32, 64, max_samples=16)
    net.params.copy_(torch.from_numpy(CR.init_params(net, seed=0)))
    trainer = CR.RolloutTrainer(net, [cr], [tr], window=8, waves=8, seed=0)
    losses = [trainer.step(lr=2e-3 * (0.5 * (1 + np.cos(np.pi * i / 300)))) for i in range(300)]
    assert np.mean(losses[-20:]) < 0.5 * np.mean(losses[:5]), (losses[:5], losses[-20:])
    test_pos = np.random.default_rng(9).uniform(0, 5.431, size=(12, 2))
    ref = CR.fine_multislice(cr, test_pos, steps)
    coarse = CR.coarse_multislice(cr, test_pos, steps)
    corr = CR.corrected_multislice(net, cr, test_pos, steps)
    net.check()
    e_coarse = CR.rel_l2(coarse, ref).mean()
    e_corr = CR.rel_l2(corr, ref).mean()
    assert e_corr < 0.8 * e_coarse, (e_corr, e_coarse)
    net.close()
