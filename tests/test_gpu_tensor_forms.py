"""Parity of the tensor-core forms (tf32, bf16x3, tf32x3, bf16x6, fp16x3) against the
oracle, through the C ABI.

Tolerances: the reference's verify rule (every element within 0.05 percent
of its FP32 host loop, polybench/gemm.cpp:96-113) on the polybench inputs,
and a normwise Frobenius error against the FP64 oracle on random inputs of
  tf32    1e-3   (operands rounded to 11 significand bits)
  bf16x3  2e-5   (hi+lo BF16 keep ~16 bits: ~2^-17 per operand)
  tf32x3, bf16x6: the FP32 bound 2e-6*sqrt(K) (the terms keep ~24 bits)
  fp16x3  the same bound (hi+lo FP16 of block-scaled operands keep 22 bits)
"""
import numpy as np
import pytest

import oracle
from gbpoly import Op, Precision

pytestmark = pytest.mark.gpu

P = Precision.BF16X3
FORMS = [Precision.TF32, Precision.BF16X3, Precision.TF32X3, Precision.BF16X6, Precision.FP16X3]
VERIFYING = [Precision.BF16X3, Precision.TF32X3, Precision.BF16X6, Precision.FP16X3]


def frob_bound(prec, K):
    if prec == Precision.TF32:
        return 1e-3
    if prec == Precision.BF16X3:
        return 2e-5
    return 2e-6 * max(1.0, np.sqrt(K))


def run_gemm(ctx, A, B, C, alpha, beta, op_a=Op.N, op_b=Op.N, prec=P):
    M = A.shape[1] if op_a == Op.T else A.shape[0]
    K = A.shape[0] if op_a == Op.T else A.shape[1]
    N = B.shape[0] if op_b == Op.T else B.shape[1]
    dA, dB, dC = ctx.upload(A), ctx.upload(B), ctx.upload(C)
    ctx.gemm(prec, M, N, K, alpha, dA, A.shape[1], dB, B.shape[1], beta, dC, C.shape[1], op_a=op_a, op_b=op_b)
    ctx.synchronize()
    out = ctx.download(dC, C.shape)
    for b in (dA, dB, dC):
        ctx.free(b)
    return out


def assert_verify(host, dev):
    first, max_pd, nfail = oracle.verify(host, dev)
    assert first == -1, f"{nfail} elements over 0.05%, first at {first}, max percentDiff {max_pd}"


@pytest.mark.parametrize("prec", VERIFYING)
@pytest.mark.parametrize("n", [64, 128, 200, 256, 384, 1024])
def test_gemm_polybench_init_passes_reference_verify(ctx, prec, n):
    A, B, C = oracle.init_gemm(n)
    dev = run_gemm(ctx, A, B, C, 32412.0, 2123.0, prec=prec)
    assert_verify(oracle.host_gemm(n), dev)
    ref = oracle.gemm_f64(A, B, C, 32412.0, 2123.0)
    max_rel, frob, _ = oracle.error_norms(dev, ref)
    assert frob < frob_bound(prec, n), (max_rel, frob)


@pytest.mark.parametrize("prec", FORMS)
@pytest.mark.parametrize("op_a", [Op.N, Op.T])
@pytest.mark.parametrize("op_b", [Op.N, Op.T])
@pytest.mark.parametrize("mnk", [(128, 256, 64), (200, 300, 100), (256, 512, 1024), (33, 65, 17), (129, 1, 40)])
def test_gemm_random_ops_vs_fp64(ctx, prec, op_a, op_b, mnk):
    M, N, K = mnk
    rng = np.random.default_rng(M * 7 + N * 3 + K + 11 * int(op_a) + 13 * int(op_b))
    A = rng.uniform(-1, 1, (K, M) if op_a == Op.T else (M, K)).astype(np.float32)
    B = rng.uniform(-1, 1, (N, K) if op_b == Op.T else (K, N)).astype(np.float32)
    C = rng.uniform(-1, 1, (M, N)).astype(np.float32)
    dev = run_gemm(ctx, A, B, C, 1.5, -0.5, op_a=op_a, op_b=op_b, prec=prec)
    ref = oracle.gemm_f64(A, B, C, 1.5, -0.5, op_a=int(op_a), op_b=int(op_b))
    max_rel, frob, _ = oracle.error_norms(dev, ref)
    assert frob < frob_bound(prec, K), (max_rel, frob)


BF16X3_ERR, BF16X3_RATIO = 4.44e-6, 21.3


def test_error_relative_to_fp32(ctx):
    """Error against the FP64 oracle relative to plain FP32's, normal(0,1) inputs.

    tf32x3 and bf16x6 keep ~24 significand bits per operand and match FP32,
    fp16x3 keeps 22 (2^-23 relative per operand) and matches it too;
    bf16x3 keeps ~16, so its error is set by its operands' representation
    (about 2^-17 relative), not by K: at K = 512, where FP32's accumulation
    error is still small (2.1e-7), it is 4.4e-6, BF16X3_RATIO times FP32's, as
    measured on a GB300 (still 100x inside the 0.05 percent verify
    threshold).  The test allows 1.5 times the measured error and ratio."""
    n = 512
    rng = np.random.default_rng(3)
    A = rng.standard_normal((n, n)).astype(np.float32)
    B = rng.standard_normal((n, n)).astype(np.float32)
    C = rng.standard_normal((n, n)).astype(np.float32)
    ref = oracle.gemm_f64(A, B, C, 1.0, 1.0)
    err = {p: oracle.error_norms(run_gemm(ctx, A, B, C, 1.0, 1.0, prec=p), ref)[1]
           for p in [Precision.FP32] + FORMS}
    print({p.name: f"{e:.3e}" for p, e in err.items()})
    f32 = err[Precision.FP32]
    assert err[Precision.TF32X3] < 1.5 * f32
    assert err[Precision.BF16X6] < 1.5 * f32
    assert err[Precision.FP16X3] < 1.5 * f32
    assert err[Precision.BF16X3] < 1.5 * BF16X3_RATIO * f32
    assert err[Precision.BF16X3] < 1.5 * BF16X3_ERR


@pytest.mark.parametrize("prec", [Precision.TF32X3, Precision.BF16X6, Precision.FP16X3])
def test_long_k_error_no_worse_than_fp32(ctx, prec):
    """K = 8192 on the polybench gemm inputs (all positive: truncation bias
    would add up): the 24-bit forms stay within FP32's error."""
    M, N, K = 256, 256, 8192
    i = np.arange(M, dtype=np.float32)[:, None] * np.float32(32)
    k = np.arange(K, dtype=np.float32)
    A = (i * k[None, :]) / np.float32(K)
    B = (k[:, None] * (np.arange(N, dtype=np.float32)[None, :] * np.float32(32)) + np.float32(1)) / np.float32(K)
    C = np.ones((M, N), np.float32)
    ref = oracle.gemm_f64(A, B, C, 32412.0, 2123.0)
    f32 = oracle.error_norms(run_gemm(ctx, A, B, C, 32412.0, 2123.0, prec=Precision.FP32), ref)
    x = oracle.error_norms(run_gemm(ctx, A, B, C, 32412.0, 2123.0, prec=prec), ref)
    print(prec.name, "max/frob", x[:2], "fp32", f32[:2])
    assert x[1] < 1.5 * f32[1] and x[0] < 1.5 * f32[0]


def test_beta_zero_does_not_read_c(ctx):
    rng = np.random.default_rng(1)
    A = rng.uniform(-1, 1, (130, 70)).astype(np.float32)
    B = rng.uniform(-1, 1, (70, 260)).astype(np.float32)
    C = np.full((130, 260), np.nan, np.float32)
    dev = run_gemm(ctx, A, B, C, 2.0, 0.0)
    assert np.isfinite(dev).all()
    assert oracle.error_norms(dev, oracle.gemm_f64(A, B, None, 2.0, 0.0))[1] < 2e-5


@pytest.mark.parametrize("prec", VERIFYING)
@pytest.mark.parametrize("n", [64, 257, 512])
def test_syrk_polybench_init_passes_reference_verify(ctx, prec, n):
    A, C = oracle.init_syrk(n)
    dA, dC = ctx.upload(A), ctx.upload(C)
    ctx.syrk(prec, n, n, 123.0, dA, n, 14512.0, dC, n)
    ctx.synchronize()
    assert_verify(oracle.host_syrk(n), ctx.download(dC, C.shape))


@pytest.mark.parametrize("prec", VERIFYING)
@pytest.mark.parametrize("n", [64, 257, 512])
def test_syr2k_polybench_init_passes_reference_verify(ctx, prec, n):
    A, B, C = oracle.init_syr2k(n)
    dA, dB, dC = ctx.upload(A), ctx.upload(B), ctx.upload(C)
    ctx.syr2k(prec, n, n, 1.0, dA, n, dB, n, 1.0, dC, n)
    ctx.synchronize()
    assert_verify(oracle.host_syr2k(n), ctx.download(dC, C.shape))


@pytest.mark.parametrize("prec", FORMS)
@pytest.mark.parametrize("nk", [(128, 64), (300, 200)])
def test_syr2k_random_vs_fp64(ctx, prec, nk):
    n, k = nk
    rng = np.random.default_rng(n + k)
    A = rng.standard_normal((n, k)).astype(np.float32)
    B = rng.standard_normal((n, k)).astype(np.float32)
    C = rng.standard_normal((n, n)).astype(np.float32)
    dA, dB, dC = ctx.upload(A), ctx.upload(B), ctx.upload(C)
    ctx.syr2k(prec, n, k, 0.75, dA, k, dB, k, 1.25, dC, n)
    ctx.synchronize()
    ref = oracle.gemm_f64(A, B, C, 0.75, 1.25, op_b=1, A2=B, B2=A)
    assert oracle.error_norms(ctx.download(dC, C.shape), ref)[1] < frob_bound(prec, 2 * k)


@pytest.mark.parametrize("prec", VERIFYING)
def test_2mm_chain_passes_reference_verify(ctx, prec):
    P = prec
    n = 256
    A, B, C, D = oracle.init_mm2(n)
    dA, dB, dC, dD = (ctx.upload(x) for x in (A, B, C, D))
    dE = ctx.alloc(n * n * 4)
    ctx.gemm(P, n, n, n, 1.0, dA, n, dB, n, 1.0, dC, n)
    ctx.gemm(P, n, n, n, 1.0, dC, n, dD, n, 0.0, dE, n)
    ctx.synchronize()
    assert_verify(oracle.host_mm2(n), ctx.download(dE, (n, n)))


def _block_scaled(rng, rows, cols, lo=1e-3, hi=1e3):
    x = rng.uniform(-1, 1, (rows, cols))
    for r in range(0, rows, 128):
        for c in range(0, cols, 128):
            x[r:r + 128, c:c + 128] *= np.exp(rng.uniform(np.log(lo), np.log(hi)))
    return x.astype(np.float32)


@pytest.mark.parametrize("op_b", [Op.N, Op.T])
@pytest.mark.parametrize("mnk", [(256, 384, 512), (200, 130, 300), (128, 256, 128)])
def test_fp8_block_scaled_vs_fp64(ctx, op_b, mnk):
    """e4m3 with one scale per 128 x 128 block: 3 mantissa bits, so a few
    percent normwise; block-wise magnitudes spanning 1e-3..1e3 stay resolved."""
    M, N, K = mnk
    rng = np.random.default_rng(M + N + K)
    A = _block_scaled(rng, M, K)
    B = _block_scaled(rng, N, K) if op_b == Op.T else _block_scaled(rng, K, N)
    A[:128, :128] = 0.0  # an all-zero block (scale 1)
    C = rng.uniform(-1, 1, (M, N)).astype(np.float32)
    dev = run_gemm(ctx, A, B, C, 1.0, 0.25, op_b=op_b, prec=Precision.FP8)
    ref = oracle.gemm_f64(A, B, C, 1.0, 0.25, op_b=int(op_b))
    max_rel, frob, _ = oracle.error_norms(dev, ref)
    assert frob < 6e-2, (max_rel, frob)


def test_fp8_syrk_and_syr2k(ctx):
    rng = np.random.default_rng(4)
    n, k = 256, 384
    A = rng.standard_normal((n, k)).astype(np.float32)
    B = rng.standard_normal((n, k)).astype(np.float32)
    C = rng.standard_normal((n, n)).astype(np.float32)
    dA, dB, dC = ctx.upload(A), ctx.upload(B), ctx.upload(C)
    ctx.syrk(Precision.FP8, n, k, 1.0, dA, k, 1.0, dC, n)
    ctx.synchronize()
    ref = oracle.gemm_f64(A, A, C, 1.0, 1.0, op_b=1)
    assert oracle.error_norms(ctx.download(dC, C.shape), ref)[1] < 6e-2
    ctx.h2d(dC, C)
    ctx.syr2k(Precision.FP8, n, k, 1.0, dA, k, dB, k, 1.0, dC, n)
    ctx.synchronize()
    ref2 = oracle.gemm_f64(A, B, C, 1.0, 1.0, op_b=1, A2=B, B2=A)
    assert oracle.error_norms(ctx.download(dC, C.shape), ref2)[1] < 6e-2


@pytest.mark.parametrize("op_b", [Op.N, Op.T])
@pytest.mark.parametrize("mnk", [(256, 512, 512), (200, 300, 300), (384, 256, 128)])
def test_fp8_wide_tiles_are_bitwise_the_square_ones(ctx, op_b, mnk):
    """fp8 configuration 1 (128 x 256 tiles) computes every element as
    configuration 0 (128 x 128): the same scaled chunk sums in the same order;
    symmetric products set to configuration 1 run configuration 0."""
    M, N, K = mnk
    rng = np.random.default_rng(M * N + K)
    A = _block_scaled(rng, M, K)
    B = _block_scaled(rng, N, K) if op_b == Op.T else _block_scaled(rng, K, N)
    C = rng.uniform(-1, 1, (M, N)).astype(np.float32)
    outs = []
    for cfg in (0, 1):
        ctx.config_set(Precision.FP8, M, N, K, cfg)
        outs.append(run_gemm(ctx, A, B, C, 1.0, 0.25, op_b=op_b, prec=Precision.FP8))
    ctx.config_set(Precision.FP8, M, N, K, 0)
    np.testing.assert_array_equal(outs[1].view(np.uint32), outs[0].view(np.uint32))
    n, k = 300, 200
    X = rng.standard_normal((n, k)).astype(np.float32)
    C2 = rng.standard_normal((n, n)).astype(np.float32)
    dX, dC = ctx.upload(X), ctx.upload(C2)
    ctx.config_set(Precision.FP8, n, n, k, 1)
    ctx.syrk(Precision.FP8, n, k, 1.0, dX, k, 1.0, dC, n)
    ctx.synchronize()
    ctx.config_set(Precision.FP8, n, n, k, 0)
    ref = oracle.gemm_f64(X, X, C2, 1.0, 1.0, op_b=1)
    assert oracle.error_norms(ctx.download(dC, C2.shape), ref)[1] < 6e-2
    ctx.free(dX)
    ctx.free(dC)
