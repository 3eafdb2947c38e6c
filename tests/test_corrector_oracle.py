"""The corrector oracle's analytic gradient against central finite differences
(CPU, float64)."""
import numpy as np

from oracle import corrector_oracle as CO


def test_layout_count():
    C, L = 32, 4
    _, n = CO.layout(C, L)
    assert n == 4 * C + C + L * (2 * CO.K * CO.K * C * C + C * C + C) + C * C + C + 2 * C + 2


def test_gradient_finite_differences():
    rng = np.random.default_rng(0)
    C, L, B, H, W = 4, 2, 2, 16, 12
    flat = CO.init_params(C, L, seed=1)
    flat += 0.05 * rng.standard_normal(flat.shape)      # move off the near-zero output init
    psi_c = rng.standard_normal((B, H, W)) + 1j * rng.standard_normal((B, H, W))
    tc = np.exp(1j * rng.uniform(0, 1, (B, H, W)))
    psi_f = psi_c + 0.1 * (rng.standard_normal((B, H, W)) + 1j * rng.standard_normal((B, H, W)))
    denom = float(np.sum(np.abs(psi_f - psi_c) ** 2))
    loss, g = CO.loss_grad(flat, psi_c, tc, psi_f, denom, C, L)
    idx = rng.choice(flat.size, 60, replace=False)
    eps = 1e-6
    for i in idx:
        fp, fm = flat.copy(), flat.copy()
        fp[i] += eps
        fm[i] -= eps
        num = (CO.loss_grad(fp, psi_c, tc, psi_f, denom, C, L)[0] - CO.loss_grad(fm, psi_c, tc, psi_f, denom, C, L)[0]) / (2 * eps)
        assert abs(num - g[i]) <= 1e-6 + 1e-5 * abs(num), (i, num, g[i])
