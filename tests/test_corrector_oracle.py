"""The corrector oracle's analytic gradient against central finite differences
(CPU, float64), and its bfloat16 rounding rule.  CPU only."""
import numpy as np

from oracle import corrector_oracle as CO


def test_bf16_rounding():
    x = np.array([1.0, 1.0 + 2 ** -8, 1.0 + 3 * 2 ** -8, -2.5, 3.0e-5, 0.0])
    r = CO.bf16(x)
    assert r[0] == 1.0 and r[1] == 1.0            # tie to even
    assert r[2] == 1.0 + 2 ** -6                  # tie to even (upwards)
    assert r[3] == -2.5 and r[5] == 0.0
    assert abs(r[4] - 3.0e-5) < 3.0e-5 * 2 ** -8


def test_layout_count():
    net = CO.Net(256, 256, 6, 32, 4, 32, 64)
    C = 32
    assert net.count() == C * 6 + C + 4 * (32 * 64 * C * C * 2 + C * C + C) + C * C + C + 4 * C + 4


def test_gradient_finite_differences():
    rng = np.random.default_rng(0)
    net = CO.Net(16, 12, 3, 4, 2, 4, 6)
    flat = CO.init_params(net, seed=1, out_scale=0.5)
    flat += 0.05 * rng.standard_normal(flat.shape)
    feats = rng.standard_normal((2, 16, 12, 3))
    target = rng.standard_normal((2, 16, 12, 4))

    def loss(f):
        m, cache = CO.forward(net, f, feats)
        return 0.5 * np.sum((m - target) ** 2), m, cache
    L0, m, cache = loss(flat)
    g = CO.backward(net, cache, m - target)
    idx = rng.choice(flat.size, 80, replace=False)
    eps = 1e-6
    for i in idx:
        fp, fm = flat.copy(), flat.copy()
        fp[i] += eps
        fm[i] -= eps
        num = (loss(fp)[0] - loss(fm)[0]) / (2 * eps)
        assert abs(num - g[i]) <= 1e-6 + 1e-5 * abs(num), (i, num, g[i])


def test_spectral_layer_is_a_low_pass_of_the_fft():
    """With R = identity per mode, Spec(u) is the real-field low-pass of u on the
    retained modes: kx in [0, MX), ky in [-MY/2, MY/2), each kx >= 1 mode together
    with its mirror (-ky, -kx), each kx = 0 mode at half weight with its mirror."""
    rng = np.random.default_rng(2)
    H, W, C, MX, MY = 16, 20, 3, 5, 8
    net = CO.Net(H, W, 1, C, 1, MX, MY)
    p = net.unflatten(np.zeros(net.count()))
    p['R1'][..., 0] = np.eye(C)[None, None]
    u = rng.standard_normal((2, H, W, C))
    sp, _ = CO._spec(net, p, 0, u)
    w = np.zeros((H, W))
    for q in range(MY):
        f = q if q < MY // 2 else q - MY
        w[f % H, 0] += 0.5
        w[(-f) % H, 0] += 0.5
        for m in range(1, MX):
            w[f % H, m] += 1.0
            w[(-f) % H, (-m) % W] += 1.0
    ref = np.fft.ifft2(np.fft.fft2(u, axes=(1, 2)) * w[None, :, :, None], axes=(1, 2)).real
    np.testing.assert_allclose(sp, ref, atol=1e-6 * np.abs(u).max())
