"""FP64 NumPy restatement of the learned coarse-slice corrector -- TEST INFRASTRUCTURE ONLY.

The corrector has no counterpart in the reference (it is an addition of this
project); this module is the oracle its CUDA forward and backward kernels are
checked against (tests/test_corrector*.py).  The network, parameter layout
and loss are those documented in namsa_gb300/csrc/msx_corrector.cu:

  x0 = [Re psi_c, Im psi_c, Re t_c, Im t_c]
  a0 = W0 x0 + b0
  a_l = gelu(Spec_l(a_{l-1}) + W_l a_{l-1} + b_l)
  Spec(u)[o] = Re(IDFT_K(sum_i R[a, m, o, i] DFT_K(u)[i, a, m])) / (H W)
  h = gelu(P1 a_L + c1);  o = P2 h + c2;  pred = psi_c + o0 + i o1
  loss = sum |pred - psi_f|^2 / denom

with K = 8 retained modes per axis at frequencies -4..3 and the tanh gelu.
"""
from __future__ import annotations

import numpy as np

K = 8


def layout(C, L):
    """Offsets of every parameter block in the flat vector (same order as the C code)."""
    off = {}
    n = 0

    def take(name, size):
        nonlocal n
        off[name] = (n, size)
        n += size
    take('W0', C * 4)
    take('b0', C)
    for l in range(L):
        take(f'Rr{l}', K * K * C * C)
        take(f'Ri{l}', K * K * C * C)
        take(f'W{l + 1}', C * C)
        take(f'b{l + 1}', C)
    take('P1', C * C)
    take('c1', C)
    take('P2', 2 * C)
    take('c2', 2)
    return off, n


def unpack(flat, C, L):
    off, _ = layout(C, L)
    p = {}
    for name, (o, s) in off.items():
        p[name] = flat[o:o + s]
    p['W0'] = p['W0'].reshape(C, 4)
    for l in range(L):
        p[f'R{l}'] = (p[f'Rr{l}'] + 1j * p[f'Ri{l}']).reshape(K, K, C, C)
        p[f'W{l + 1}'] = p[f'W{l + 1}'].reshape(C, C)
    p['P1'] = p['P1'].reshape(C, C)
    p['P2'] = p['P2'].reshape(2, C)
    return p


def init_params(C, L, seed=0):
    """Seeded initial parameters: fan-in scaled linear maps, small spectral
    weights, and a near-zero output layer so the untrained net returns psi_c."""
    rng = np.random.default_rng(seed)
    off, n = layout(C, L)
    flat = np.zeros(n)

    def put(name, arr):
        o, s = off[name]
        flat[o:o + s] = arr.ravel()
    put('W0', rng.standard_normal((C, 4)) / np.sqrt(4))
    for l in range(L):
        put(f'Rr{l}', rng.standard_normal((K, K, C, C)) / C)
        put(f'Ri{l}', rng.standard_normal((K, K, C, C)) / C)
        put(f'W{l + 1}', rng.standard_normal((C, C)) / np.sqrt(C))
    put('P1', rng.standard_normal((C, C)) / np.sqrt(C))
    put('P2', 1e-2 * rng.standard_normal((2, C)) / np.sqrt(C))
    return flat


def freqs(n):
    return np.array([m if m < K // 2 else n - (K - m) for m in range(K)])


def dft_mats(H, W):
    fy, fx = freqs(H), freqs(W)
    Fy = np.exp(-2j * np.pi * np.outer(np.arange(H), fy) / H)   # (H, K)
    Fx = np.exp(-2j * np.pi * np.outer(np.arange(W), fx) / W)   # (W, K)
    return Fy, Fx


def gelu(z):
    k = np.sqrt(2 / np.pi)
    return 0.5 * z * (1 + np.tanh(k * (z + 0.044715 * z ** 3)))


def gelu_d(z):
    k = np.sqrt(2 / np.pi)
    th = np.tanh(k * (z + 0.044715 * z ** 3))
    return 0.5 * (1 + th) + 0.5 * z * (1 - th ** 2) * k * (1 + 3 * 0.044715 * z ** 2)


def lin(Wm, b, x):
    """x (B, Cin, H, W) -> (B, Cout, H, W)."""
    return np.einsum('oi,bihw->bohw', Wm, x) + b[None, :, None, None]


def spec_fwd(R, u, Fy, Fx):
    H, W = u.shape[-2:]
    X = np.einsum('bchw,ha,wm->bcam', u, Fy, Fx)
    Y = np.einsum('amoi,biam->boam', R, X)
    v = np.einsum('boam,ha,wm->bohw', Y, Fy.conj(), Fx.conj()).real / (H * W)
    return v, X


def forward(flat, psi_c, tc, C, L):
    """psi_c, tc: (B, H, W) complex.  Returns (pred, cache)."""
    p = unpack(flat, C, L)
    B, H, W = psi_c.shape
    Fy, Fx = dft_mats(H, W)
    x0 = np.stack([psi_c.real, psi_c.imag, tc.real, tc.imag], 1)
    a = [lin(p['W0'], p['b0'], x0)]
    zs, Xs = [], []
    for l in range(L):
        v, X = spec_fwd(p[f'R{l}'], a[-1], Fy, Fx)
        z = v + lin(p[f'W{l + 1}'], p[f'b{l + 1}'], a[-1])
        zs.append(z)
        Xs.append(X)
        a.append(gelu(z))
    zh = lin(p['P1'], p['c1'], a[-1])
    h = gelu(zh)
    o = lin(p['P2'], p['c2'], h)
    pred = psi_c + o[:, 0] + 1j * o[:, 1]
    return pred, dict(x0=x0, a=a, zs=zs, Xs=Xs, zh=zh, h=h, Fy=Fy, Fx=Fx)


def loss_grad(flat, psi_c, tc, psi_f, denom, C, L):
    """Loss and the gradient w.r.t. the flat parameters (analytic backward)."""
    p = unpack(flat, C, L)
    pred, c = forward(flat, psi_c, tc, C, L)
    B, H, W = psi_c.shape
    r = pred - psi_f
    loss = np.sum(np.abs(r) ** 2) / denom
    off, n = layout(C, L)
    g = np.zeros(n)

    def put(name, arr):
        o_, s = off[name]
        g[o_:o_ + s] = np.asarray(arr).ravel()
    dO = np.stack([2 * r.real / denom, 2 * r.imag / denom], 1)
    put('P2', np.einsum('bohw,bihw->oi', dO, c['h']))
    put('c2', dO.sum((0, 2, 3)))
    dh = np.einsum('oi,bohw->bihw', p['P2'], dO)
    dzh = dh * gelu_d(c['zh'])
    put('P1', np.einsum('bohw,bihw->oi', dzh, c['a'][L]))
    put('c1', dzh.sum((0, 2, 3)))
    da = np.einsum('oi,bohw->bihw', p['P1'], dzh)
    Fy, Fx = c['Fy'], c['Fx']
    for l in range(L - 1, -1, -1):
        dz = da * gelu_d(c['zs'][l])
        ain = c['a'][l]
        put(f'W{l + 1}', np.einsum('bohw,bihw->oi', dz, ain))
        put(f'b{l + 1}', dz.sum((0, 2, 3)))
        da = np.einsum('oi,bohw->bihw', p[f'W{l + 1}'], dz)
        dY = np.einsum('bohw,ha,wm->boam', dz, Fy, Fx) / (H * W)
        dR = np.einsum('boam,biam->amoi', dY, c['Xs'][l].conj())
        put(f'Rr{l}', dR.real)
        put(f'Ri{l}', dR.imag)
        dX = np.einsum('amoi,boam->biam', p[f'R{l}'].conj(), dY)
        da = da + np.einsum('biam,ha,wm->bihw', dX, Fy.conj(), Fx.conj()).real
    put('W0', np.einsum('bohw,bihw->oi', da, c['x0']))
    put('b0', da.sum((0, 2, 3)))
    return loss, g
