"""Split-BF16 tensor-core DFT stages (tcgen05) against NumPy FFTs in float64,
and the tensor-core slice step against the FP32 FFT step."""
import numpy as np
import pytest
import torch

from namsa_gb300 import engine

pytestmark = pytest.mark.gpu
DEV = 'cuda'


@pytest.mark.parametrize('n,lines', [(256, 128), (512, 256)])
def test_tc_dft_matches_fft(n, lines):
    rng = np.random.default_rng(n)
    x = (rng.standard_normal((lines, n)) + 1j * rng.standard_normal((lines, n))).astype(np.complex64)
    xd = torch.from_numpy(x).to(DEV)
    for sign in (-1, 1):
        z = engine.tc_dft(xd, sign).cpu().numpy()
        ref = np.fft.fft(x.astype(np.complex128), axis=1) if sign < 0 else np.fft.ifft(x.astype(np.complex128), axis=1) * n
        err = np.linalg.norm(z - ref) / np.linalg.norm(ref)
        assert err < 5e-5, (sign, err)
    engine.tc_check()


def test_tc_step_matches_fp32_step():
    rng = np.random.default_rng(1)
    n, G = 256, 3
    w = (rng.standard_normal((G, n, n)) + 1j * rng.standard_normal((G, n, n))).astype(np.complex64)
    t = np.exp(0.3j * rng.standard_normal((n, n))).astype(np.complex64)
    ptab = engine.propagator_table(n, n, np.float32(12.0), 0.025, 1.5, np.float32(4.0))
    a = torch.from_numpy(w).to(DEV)
    b = a.clone()
    td = torch.from_numpy(t).to(DEV)
    plan = engine.Plan(n, n)
    plan.step_waves(a, td, ptab)
    engine.step_waves_tc(b, td, ptab)
    torch.cuda.synchronize()
    engine.tc_check()
    err = (torch.linalg.vector_norm(a - b) / torch.linalg.vector_norm(a)).item()
    assert err < 1e-4, err
    plan.close()


def test_tc_multislice_cbed_vs_fp64():
    """A 256^2 SrTiO3 [001] run with every per-slice DFT on the tensor cores
    stays within the 1e-3 CBED bar against the FP64 oracle."""
    from namsa_gb300 import corrector as CR, structures
    from oracle import msa_oracle as O
    torch.cuda.set_device(0)
    sc = structures.srtio3((16, 16, 8))
    cr = CR.Crystal(sc, 256, 3.905 / 2, kv=300, semi_angle=25e-3, ratio=1)
    pos = np.array([[0., 0.], [1.0, 1.9]], np.float32)
    w = cr.waves(pos)
    S = cr.trans_fine.shape[0]
    for s in range(S):
        engine.step_waves_tc(w, cr.trans_fine[s], cr.ptab_fine)
    got = cr.plan.cbed_waves(w, cr.sim.norm_dev).cpu().numpy()
    engine.tc_check()
    xyz = np.column_stack([sc['x'], sc['y'], sc['z']]).astype(np.float32)
    geom = O.Geometry(xyz, sc['atomic_number'], 300., 25e-3, [256, 256])
    P, _ = O.propagator_gpu(geom, 3.905 / 2, 1 / 3)
    psik, _, norm = O.probe_gpu(geom, CR.PROBE)
    ref = O.multislice_gpu(cr.trans_fine.cpu().numpy().astype(np.complex128), psik, P, pos, norm, geom)
    err = O.rel_l2(got, ref)
    assert err.max() < 1e-3, err


def test_tc_dft_norm_compensation_keeps_parseval():
    """With the compensation (default) every output line has |Z|^2 = n |X|^2 to
    float rounding; without it the tensor-core accumulation loses norm."""
    rng = np.random.default_rng(7)
    n, lines = 512, 256
    x = (rng.standard_normal((lines, n)) + 1j * rng.standard_normal((lines, n))).astype(np.complex64)
    xd = torch.from_numpy(x).to(DEV)
    want = n * np.sum(np.abs(x.astype(np.complex128)) ** 2, axis=1)
    try:
        engine.tc_set_compensation(False)
        z0 = engine.tc_dft(xd, -1).cpu().numpy().astype(np.complex128)
    finally:
        engine.tc_set_compensation(True)
    z1 = engine.tc_dft(xd, -1).cpu().numpy().astype(np.complex128)
    engine.tc_check()
    r0 = np.sum(np.abs(z0) ** 2, axis=1) / want
    r1 = np.sum(np.abs(z1) ** 2, axis=1) / want
    assert np.abs(r1 - 1).max() < 2e-6, np.abs(r1 - 1).max()
    assert np.abs(r0 - 1).mean() > np.abs(r1 - 1).mean()
    ref = np.fft.fft(x.astype(np.complex128), axis=1)
    assert np.linalg.norm(z1 - ref) / np.linalg.norm(ref) < 5e-5


@pytest.mark.parametrize('m,n,k', [(128, 32, 64), (300, 64, 100), (1000, 4, 32), (256, 200, 512), (129, 256, 64), (32, 40, 20000),
                                   (64, 640, 192), (200000, 32, 32), (5000, 128, 6), (70000, 256, 40),
                                   (40000, 64, 1000), (32, 32, 50000), (100, 6, 30000), (200, 20, 9000)])
def test_gemm_bf16_matches_fp32_matmul_of_rounded_operands(m, n, k):
    """The general tcgen05 GEMM against a plain PyTorch FP32 matmul of the same
    bfloat16-rounded operands (only the accumulation order differs)."""
    g = torch.Generator().manual_seed(m + n + k)
    a = torch.randn(m, k, generator=g).to(DEV)
    b = torch.randn(n, k, generator=g).to(DEV)
    bias = torch.randn(n, generator=g).to(DEV)
    ref = a.to(torch.bfloat16).float() @ b.to(torch.bfloat16).float().T + bias
    got = engine.gemm_bf16(a, b, bias)
    engine.gemm_check()
    assert torch.allclose(got, ref, rtol=1e-4, atol=1e-4 * k ** 0.5), (got - ref).abs().max().item()
    # accumulate into a strided output view
    big = torch.ones(m, n + 7, device=DEV)
    out = big[:, 3:3 + n]
    engine.gemm_bf16(a, b, None, out=out, accumulate=True)
    torch.cuda.synchronize()
    assert torch.allclose(out, ref - bias + 1, rtol=1e-4, atol=1e-4 * k ** 0.5)
    assert (big[:, :3] == 1).all() and (big[:, 3 + n:] == 1).all()


@pytest.mark.parametrize('m,n,k,pad_a,pad_b', [(5000, 32, 40, 3, 0), (5000, 64, 40, 4, 1), (3000, 200, 100, 8, 3),
                                               (64, 32, 40000, 3, 5), (32, 16, 30000, 4, 0)])
def test_gemm_bf16_padded_operand_rows(m, n, k, pad_a, pad_b):
    """Operands whose rows are padded (leading dimension > k): rows that stay 16-byte
    aligned arrive by one bulk copy each, the others by plain loads; split K included."""
    g = torch.Generator().manual_seed(m + n + k + pad_a)
    a_big = torch.randn(m, k + pad_a, generator=g).to(DEV)
    b_big = torch.randn(n, k + pad_b, generator=g).to(DEV)
    a, b = a_big[:, :k], b_big[:, :k]
    ref = a.to(torch.bfloat16).float() @ b.to(torch.bfloat16).float().T
    got = engine.gemm_bf16(a, b)
    engine.gemm_check()
    assert torch.allclose(got, ref, rtol=1e-4, atol=1e-4 * k ** 0.5), (got - ref).abs().max().item()


def _gemm_cases(seed=11, count=36):
    rng = np.random.default_rng(seed)
    cases = []
    for i in range(count):
        if i % 6 == 5:  # long K, narrow output: split K
            m, n, k = int(rng.integers(1, 129)), int(rng.integers(1, 33)), int(rng.integers(4096, 40000))
        else:
            m, n, k = int(rng.integers(1, 5000)), int(rng.integers(1, 600)), int(rng.integers(1, 3000))
        cases.append((m, n, k, int(rng.integers(0, 6)), int(rng.integers(0, 6)), int(rng.integers(0, 6)),
                      bool(rng.integers(0, 2)), bool(rng.integers(0, 2))))
    return cases


@pytest.mark.parametrize('m,n,k,pad_a,pad_b,pad_c,acc,bias', _gemm_cases())
def test_gemm_bf16_random_shapes(m, n, k, pad_a, pad_b, pad_c, acc, bias):
    """Seeded random sizes, padded rows, accumulation and bias through every loader mode of
    the tensor-core GEMM, against a plain PyTorch FP32 matmul of the bfloat16-rounded
    operands."""
    g = torch.Generator().manual_seed(m * 7 + n * 13 + k)
    a = torch.randn(m, k + pad_a, generator=g).to(DEV)[:, :k]
    b = torch.randn(n, k + pad_b, generator=g).to(DEV)[:, :k]
    c_big = torch.randn(m, n + pad_c, generator=g).to(DEV)
    before = c_big.clone()
    c0 = c_big[:, :n].clone()
    bv = torch.randn(n, generator=g).to(DEV) if bias else None
    ref = a.to(torch.bfloat16).float() @ b.to(torch.bfloat16).float().T
    if bias:
        ref = ref + bv
    if acc:
        ref = ref + c0
    engine.gemm_bf16(a, b, bv, out=c_big[:, :n], accumulate=acc)
    engine.gemm_check()
    got = c_big[:, :n]
    assert torch.allclose(got, ref, rtol=1e-4, atol=1e-4 * (k ** 0.5) + 1e-5), (got - ref).abs().max().item()
    assert torch.equal(c_big[:, n:], before[:, n:])  # the padding of the output rows is untouched
