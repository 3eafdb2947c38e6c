"""FP64 NumPy restatement of the learned coarse-slice corrector -- TEST INFRASTRUCTURE ONLY.

The corrector has no counterpart in the reference (it is an addition of this
project); this module is the oracle its CUDA forward and backward passes are
checked against (tests/test_corrector_oracle.py, tests/test_gpu_corrector.py).
The network and parameter layout are those of namsa_gb300/csrc/msx_corrector.cu:

  a_0 = x W0^T + b0
  a_l = gelu(Spec_l(a_{l-1}) + a_{l-1} W_l^T + b_l),  l = 1..L
  Spec(u) = IDFT_x(IDFT_y(R . DFT_y(DFT_x(u))))  on modes kx in [0, MX),
            ky in [-MY/2, MY/2), kx >= 1 weighted 2 and 1/(H W) in IDFT_x
  h = gelu(a_L P1^T + c1);  o = h P2^T + c2      (maps: Re A, Im A, Re B, Im B)

Every contraction is written as the GEMM the CUDA code runs, D = A B^T, with
the same operand matrices (the partial DFT matrices included).  With
``bf16=True`` both operands of every GEMM are rounded to bfloat16 (round to
nearest even) as the tensor cores see them; the per-mode mixing stays exact,
as in the CUDA code.  The analytic backward is checked against central finite
differences in float64.
"""
from __future__ import annotations

import math

import numpy as np


def bf16(x):
    """Round to bfloat16 (nearest even) through float32, returned as float64."""
    f = np.ascontiguousarray(np.asarray(x, np.float64).astype(np.float32))
    b = f.view(np.uint32).astype(np.uint64)
    b = (b + 0x7FFF + ((b >> 16) & 1)) & 0xFFFF0000
    return b.astype(np.uint32).view(np.float32).astype(np.float64)


class Net:
    """Sizes, partial DFT matrices and the GEMM rule of one corrector."""

    def __init__(self, H, W, Cin, C, L, MX, MY, bf16_gemm=False):
        self.H, self.W, self.Cin, self.C, self.L, self.MX, self.MY = H, W, Cin, C, L, MX, MY
        self.emulate = bf16_gemm
        f32 = lambda a: np.asarray(a, np.float32).astype(np.float64)
        x = np.arange(W)
        m = np.arange(MX)
        th = 2 * np.pi * ((m[:, None] * x[None, :]) % W) / W
        self.Bdx = f32(np.stack([np.cos(th), -np.sin(th)], 1).reshape(2 * MX, W))
        q = np.arange(MY)
        fq = np.where(q < MY // 2, q, q - MY)
        y = np.arange(H)
        thy = 2 * np.pi * (((fq[:, None] * y[None, :]) % H + H) % H) / H        # (MY, H)
        c, s = np.cos(thy), np.sin(thy)
        Bdy = np.zeros((2 * MY, 2 * H))
        Bdy[0::2, 0::2], Bdy[0::2, 1::2], Bdy[1::2, 0::2], Bdy[1::2, 1::2] = c, s, -s, c
        self.Bdy = f32(Bdy)
        Biy = np.zeros((2 * H, 2 * MY))
        Biy[0::2, 0::2], Biy[0::2, 1::2], Biy[1::2, 0::2], Biy[1::2, 1::2] = c.T, -s.T, s.T, c.T
        self.Biy = f32(Biy)
        wm = np.where(m == 0, 1.0, 2.0) / (H * W)
        thx = 2 * np.pi * ((x[:, None] * m[None, :]) % W) / W                   # (W, MX)
        self.Bix = f32(np.stack([wm * np.cos(thx), -wm * np.sin(thx)], 2).reshape(W, 2 * MX))

    def g(self, A, B):
        """D = A B^T with the operands as the tensor cores see them."""
        if self.emulate:
            A, B = bf16(A), bf16(B)
        return A @ B.T

    # ---------------------------------------------------------------- parameters
    def layout(self):
        C, Ci, L, MX, MY = self.C, self.Cin, self.L, self.MX, self.MY
        shapes = [('W0', (C, Ci)), ('b0', (C,))]
        for l in range(L):
            shapes += [(f'R{l + 1}', (MX, MY, C, C, 2)), (f'W{l + 1}', (C, C)), (f'b{l + 1}', (C,))]
        shapes += [('P1', (C, C)), ('c1', (C,)), ('P2', (4, C)), ('c2', (4,))]
        return shapes

    def count(self):
        return sum(int(np.prod(s)) for _, s in self.layout())

    def unflatten(self, flat):
        out, o = {}, 0
        for name, shape in self.layout():
            n = int(np.prod(shape))
            out[name] = np.asarray(flat[o:o + n], np.float64).reshape(shape)
            o += n
        return out

    def flatten(self, d):
        return np.concatenate([np.asarray(d[name], np.float64).ravel() for name, _ in self.layout()])


def init_params(net, seed=0, out_scale=1e-2, spec_scale=0.5):
    """Initialisation used for training: scaled normal weights, zero biases, a
    small output layer so that the first maps are close to zero."""
    rng = np.random.default_rng(seed)
    C, Ci = net.C, net.Cin
    d = {}
    for name, shape in net.layout():
        if name.startswith('b') or name.startswith('c'):
            d[name] = np.zeros(shape)
        elif name == 'W0':
            d[name] = rng.standard_normal(shape) / math.sqrt(Ci)
        elif name.startswith('R'):
            d[name] = rng.standard_normal(shape) * spec_scale / C
        elif name == 'P2':
            d[name] = rng.standard_normal(shape) * out_scale / math.sqrt(C)
        else:
            d[name] = rng.standard_normal(shape) / math.sqrt(C)
    return net.flatten(d)


def _gelu(z):
    u = 0.7978845608028654 * (z + 0.044715 * z ** 3)
    return 0.5 * z * (1 + np.tanh(u))


def _gelu_d(z):
    k = 0.7978845608028654
    th = np.tanh(k * (z + 0.044715 * z ** 3))
    return 0.5 * (1 + th) + 0.5 * z * (1 - th * th) * k * (1 + 3 * 0.044715 * z * z)


# ------------------------------------------------------------------ forward / backward
def _mix(net, Rr, Ri, Ur, Ui, kind):
    """Per-mode complex channel mixing as the four real GEMMs the CUDA code runs
    (operands rounded to bfloat16 when the net emulates the tensor cores).
    fwd: Y = R X; data: dX = conj(R)^T dY (U = dY); weight: dR = dY X^H summed over
    samples (U = dY, returned with X given as Rr, Ri of shape (S, i, m, q))."""
    b = bf16 if net.emulate else (lambda x: x)
    if kind == 'fwd':
        e = lambda r, u: np.einsum('mqoi,simq->somq', b(r), b(u))
        return (e(Rr, Ur) - e(Ri, Ui)) + 1j * (e(Ri, Ur) + e(Rr, Ui))
    if kind == 'data':
        e = lambda r, u: np.einsum('mqoi,somq->simq', b(r), b(u))
        return (e(Rr, Ur) + e(Ri, Ui)) + 1j * (e(Rr, Ui) - e(Ri, Ur))
    e = lambda u, x: np.einsum('somq,simq->mqoi', b(u), b(x))
    return (e(Ur, Rr) + e(Ui, Ri)) + 1j * (e(Ui, Rr) - e(Ur, Ri))


def _spec(net, p, l, a):
    """Spectral part of layer l for a (S, H, W, C); returns (sp, X) with X the retained modes."""
    S, H, W, C, MX, MY = a.shape[0], net.H, net.W, net.C, net.MX, net.MY
    U1 = net.g(a.transpose(0, 1, 3, 2).reshape(S * H * C, W), net.Bdx).reshape(S, H, C, MX, 2)
    A2 = U1.transpose(0, 2, 3, 1, 4).reshape(S * C * MX, 2 * H)
    Xr = net.g(A2, net.Bdy).reshape(S, C, MX, MY, 2)
    X = Xr[..., 0] + 1j * Xr[..., 1]
    Rr, Ri = p[f'R{l + 1}'][..., 0], p[f'R{l + 1}'][..., 1]                    # (MX, MY, o, i)
    Y = _mix(net, Rr, Ri, X.real, X.imag, 'fwd')
    Yr = np.stack([Y.real, Y.imag], -1).reshape(S * C * MX, 2 * MY)
    U2 = net.g(Yr, net.Biy).reshape(S, C, MX, H, 2).transpose(0, 3, 1, 2, 4)   # (S, H, C, MX, 2)
    sp = net.g(U2.reshape(S * H * C, 2 * MX), net.Bix).reshape(S, H, C, W).transpose(0, 1, 3, 2)
    return sp, X


def forward(net, flat, feats):
    """Maps (S, H, W, 4) of features (S, H, W, Cin); returns (maps, cache)."""
    p = net.unflatten(flat)
    S = feats.shape[0]
    SP, C = S * net.H * net.W, net.C
    x = np.asarray(feats, np.float64)
    a = [(net.g(x.reshape(SP, net.Cin), p['W0']) + p['b0']).reshape(S, net.H, net.W, C)]
    zs, Xs = [], []
    for l in range(net.L):
        sp, X = _spec(net, p, l, a[-1])
        z = sp + (net.g(a[-1].reshape(SP, C), p[f'W{l + 1}']) + p[f'b{l + 1}']).reshape(sp.shape)
        zs.append(z)
        Xs.append(X)
        a.append(_gelu(z))
    zh = net.g(a[-1].reshape(SP, C), p['P1']) + p['c1']
    h = _gelu(zh)
    o = net.g(h, p['P2']) + p['c2']
    return o.reshape(S, net.H, net.W, 4), dict(p=p, x=x, a=a, z=zs, X=Xs, zh=zh, h=h)


def backward(net, cache, dmaps):
    """Parameter gradients (flat) for d loss / d maps (S, H, W, 4)."""
    p, x, a, zs, Xs = cache['p'], cache['x'], cache['a'], cache['z'], cache['X']
    S, H, W, C, MX, MY = x.shape[0], net.H, net.W, net.C, net.MX, net.MY
    SP = S * H * W
    g = {}
    do = np.asarray(dmaps, np.float64).reshape(SP, 4)
    g['P2'] = net.g(do.T, cache['h'].T)
    g['c2'] = do.sum(0)
    dzh = net.g(do, p['P2'].T) * _gelu_d(cache['zh'])
    g['P1'] = net.g(dzh.T, a[-1].reshape(SP, C).T)
    g['c1'] = dzh.sum(0)
    da = net.g(dzh, p['P1'].T).reshape(S, H, W, C)
    for l in range(net.L - 1, -1, -1):
        dz = da * _gelu_d(zs[l])
        dz2 = dz.reshape(SP, C)
        g[f'W{l + 1}'] = net.g(dz2.T, a[l].reshape(SP, C).T)
        g[f'b{l + 1}'] = dz2.sum(0)
        da_new = net.g(dz2, p[f'W{l + 1}'].T).reshape(S, H, W, C)
        # spectral adjoint: every stage D = g(A, B) gives dA = g(dD, B^T)
        dU2 = net.g(dz.transpose(0, 1, 3, 2).reshape(S * H * C, W), net.Bix.T).reshape(S, H, C, MX, 2)
        dYr = net.g(dU2.transpose(0, 2, 3, 1, 4).reshape(S * C * MX, 2 * H), net.Biy.T).reshape(S, C, MX, MY, 2)
        dY = dYr[..., 0] + 1j * dYr[..., 1]
        Rr, Ri = p[f'R{l + 1}'][..., 0], p[f'R{l + 1}'][..., 1]
        dR = _mix(net, Xs[l].real, Xs[l].imag, dY.real, dY.imag, 'weight')
        g[f'R{l + 1}'] = np.stack([dR.real, dR.imag], -1)
        dX = _mix(net, Rr, Ri, dY.real, dY.imag, 'data')
        dXr = np.stack([dX.real, dX.imag], -1).reshape(S * C * MX, 2 * MY)
        dU1 = net.g(dXr, net.Bdy.T).reshape(S, C, MX, H, 2).transpose(0, 3, 1, 2, 4)
        da_sp = net.g(dU1.reshape(S * H * C, 2 * MX), net.Bdx.T).reshape(S, H, C, W).transpose(0, 1, 3, 2)
        da = da_new + da_sp
    da2 = da.reshape(SP, C)
    g['W0'] = net.g(da2.T, x.reshape(SP, net.Cin).T)
    g['b0'] = da2.sum(0)
    return net.flatten(g)


# ------------------------------------------------------------------ corrected coarse step
def corrected_step(psi, tc, Pc, maps):
    """(1 + A) ifft2_u(Pc fft2_u((1 + B) tc psi)) with Pc = P mask / N (as msx_plan_step_waves)."""
    A = maps[..., 0] + 1j * maps[..., 1]
    B = maps[..., 2] + 1j * maps[..., 3]
    u = np.fft.ifft2(Pc * np.fft.fft2((1 + B) * tc * psi)) * (psi.shape[-1] * psi.shape[-2])
    return (1 + A) * u
