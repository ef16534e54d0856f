"""Parity of the plain FP32 SIMT path against the oracle, through the C ABI.

Tolerance: the reference's own verify rule (percentDiff <= 0.05 percent for
every element against its FP32 host loop, polybench/gemm.cpp:96-113) and, for
seeded random inputs, a normwise relative error against the FP64 oracle of
at most 2e-6 * sqrt(K)-scaled bound written in each test.
"""
import numpy as np
import pytest

import gbpoly
import oracle
from gbpoly import Op, Precision

pytestmark = pytest.mark.gpu

P = Precision.FP32
SIZES = [1, 2, 17, 64, 100, 128, 255, 256, 257, 512, 1024]


def run_gemm(ctx, A, B, C, alpha, beta, op_a=Op.N, op_b=Op.N, prec=P, lda=None, ldb=None, ldc=None):
    M = A.shape[1] if op_a == Op.T else A.shape[0]
    K = A.shape[0] if op_a == Op.T else A.shape[1]
    N = B.shape[0] if op_b == Op.T else B.shape[1]
    dA, dB, dC = ctx.upload(A), ctx.upload(B), ctx.upload(C)
    ctx.gemm(prec, M, N, K, alpha, dA, lda or A.shape[1], dB, ldb or B.shape[1], beta, dC, ldc or C.shape[1],
             op_a=op_a, op_b=op_b)
    ctx.synchronize()
    out = ctx.download(dC, C.shape)
    for b in (dA, dB, dC):
        ctx.free(b)
    return out


def assert_verify(host, dev):
    first, max_pd, nfail = oracle.verify(host, dev)
    assert first == -1, f"{nfail} elements over 0.05%, first at {first}, max percentDiff {max_pd}"


@pytest.mark.parametrize("n", SIZES)
def test_gemm_polybench_init_passes_reference_verify(ctx, n):
    A, B, C = oracle.init_gemm(n)
    dev = run_gemm(ctx, A, B, C, 32412.0, 2123.0)
    assert_verify(oracle.host_gemm(n), dev)
    ref = oracle.gemm_f64(A, B, C, 32412.0, 2123.0)
    max_rel, frob, _ = oracle.error_norms(dev, ref)
    assert max_rel < 1e-5 and frob < 1e-5, (max_rel, frob)


@pytest.mark.parametrize("op_a", [Op.N, Op.T])
@pytest.mark.parametrize("op_b", [Op.N, Op.T])
@pytest.mark.parametrize("mnk", [(128, 128, 32), (200, 136, 96), (256, 384, 512), (33, 65, 17), (129, 1, 40)])
def test_gemm_random_ops_vs_fp64(ctx, op_a, op_b, mnk):
    M, N, K = mnk
    rng = np.random.default_rng(M * 7 + N * 3 + K + 11 * int(op_a) + 13 * int(op_b))
    A = rng.uniform(-1, 1, (K, M) if op_a == Op.T else (M, K)).astype(np.float32)
    B = rng.uniform(-1, 1, (N, K) if op_b == Op.T else (K, N)).astype(np.float32)
    C = rng.uniform(-1, 1, (M, N)).astype(np.float32)
    dev = run_gemm(ctx, A, B, C, 1.5, -0.5, op_a=op_a, op_b=op_b)
    ref = oracle.gemm_f64(A, B, C, 1.5, -0.5, op_a=int(op_a), op_b=int(op_b))
    max_rel, frob, _ = oracle.error_norms(dev, ref)
    # FP32 accumulation over K terms: ~sqrt(K) * 2^-24 relative, generous margin
    assert frob < 2e-6 * max(1.0, np.sqrt(K)), (max_rel, frob)


def test_gemm_beta_zero_does_not_read_c(ctx):
    rng = np.random.default_rng(1)
    A = rng.uniform(-1, 1, (130, 70)).astype(np.float32)
    B = rng.uniform(-1, 1, (70, 260)).astype(np.float32)
    C = np.full((130, 260), np.nan, np.float32)
    dev = run_gemm(ctx, A, B, C, 2.0, 0.0)
    assert np.isfinite(dev).all()
    ref = oracle.gemm_f64(A, B, None, 2.0, 0.0)
    assert oracle.error_norms(dev, ref)[1] < 1e-5


def test_gemm_k_zero_scales_c(ctx):
    C = np.arange(12 * 8, dtype=np.float32).reshape(12, 8)
    A = np.zeros((12, 0), np.float32)
    B = np.zeros((0, 8), np.float32)
    dA = ctx.alloc(16)
    dB = ctx.alloc(16)
    dC = ctx.upload(C)
    ctx.gemm(P, 12, 8, 0, 3.0, dA, 1, dB, 8, 0.5, dC, 8)
    ctx.synchronize()
    np.testing.assert_array_equal(ctx.download(dC, C.shape), C * 0.5)


def test_gemm_padded_leading_dimensions(ctx):
    rng = np.random.default_rng(5)
    M, N, K = 150, 90, 70
    Ap = rng.uniform(-1, 1, (M, 80)).astype(np.float32)   # lda = 80 > K
    Bp = rng.uniform(-1, 1, (K, 96)).astype(np.float32)   # ldb = 96 > N
    Cp = rng.uniform(-1, 1, (M, 100)).astype(np.float32)  # ldc = 100 > N
    dA, dB, dC = ctx.upload(Ap), ctx.upload(Bp), ctx.upload(Cp)
    ctx.gemm(P, M, N, K, 1.0, dA, 80, dB, 96, 1.0, dC, 100)
    ctx.synchronize()
    out = ctx.download(dC, Cp.shape)
    ref = oracle.gemm_f64(Ap[:, :K], Bp[:, :N], Cp[:, :N], 1.0, 1.0)
    assert oracle.error_norms(np.ascontiguousarray(out[:, :N]), ref)[1] < 1e-5
    np.testing.assert_array_equal(out[:, N:], Cp[:, N:])  # padding untouched


@pytest.mark.parametrize("n", [1, 17, 64, 100, 128, 257, 512])
def test_syrk_polybench_init_passes_reference_verify(ctx, n):
    A, C = oracle.init_syrk(n)
    dA, dC = ctx.upload(A), ctx.upload(C)
    ctx.syrk(P, n, n, 123.0, dA, n, 14512.0, dC, n)
    ctx.synchronize()
    dev = ctx.download(dC, C.shape)
    assert_verify(oracle.host_syrk(n), dev)


@pytest.mark.parametrize("n", [1, 17, 64, 100, 128, 257, 512])
def test_syr2k_polybench_init_passes_reference_verify(ctx, n):
    A, B, C = oracle.init_syr2k(n)
    dA, dB, dC = ctx.upload(A), ctx.upload(B), ctx.upload(C)
    ctx.syr2k(P, n, n, 1.0, dA, n, dB, n, 1.0, dC, n)
    ctx.synchronize()
    dev = ctx.download(dC, C.shape)
    assert_verify(oracle.host_syr2k(n), dev)


@pytest.mark.parametrize("nk", [(128, 64), (200, 333), (64, 1000)])
def test_syr2k_random_vs_fp64(ctx, nk):
    n, k = nk
    rng = np.random.default_rng(n + k)
    A = rng.standard_normal((n, k)).astype(np.float32)
    B = rng.standard_normal((n, k)).astype(np.float32)
    C = rng.standard_normal((n, n)).astype(np.float32)
    dA, dB, dC = ctx.upload(A), ctx.upload(B), ctx.upload(C)
    ctx.syr2k(P, n, k, 0.75, dA, k, dB, k, 1.25, dC, n)
    ctx.synchronize()
    dev = ctx.download(dC, C.shape)
    ref = oracle.gemm_f64(A, B, C, 0.75, 1.25, op_b=1, A2=B, B2=A)
    assert oracle.error_norms(dev, ref)[1] < 2e-6 * np.sqrt(2 * k)
    # exact symmetry of the update: C_out - beta*C is symmetric up to rounding of the beta term
    upd = dev.astype(np.float64) - 1.25 * C
    assert np.allclose(upd, upd.T, rtol=1e-5, atol=1e-4)


@pytest.mark.parametrize("n", [17, 128, 256])
def test_2mm_chain_passes_reference_verify(ctx, n):
    A, B, C, D = oracle.init_mm2(n)
    dA, dB, dC, dD = (ctx.upload(x) for x in (A, B, C, D))
    dE = ctx.alloc(n * n * 4)
    ctx.gemm(P, n, n, n, 1.0, dA, n, dB, n, 1.0, dC, n)   # C += A.B   (2mm.cpp:99-106)
    ctx.gemm(P, n, n, n, 1.0, dC, n, dD, n, 0.0, dE, n)   # E = C.D    (2mm.cpp:114-122)
    ctx.synchronize()
    assert_verify(oracle.host_mm2(n), ctx.download(dE, (n, n)))


@pytest.mark.parametrize("n", [17, 128, 256])
def test_3mm_chain_passes_reference_verify(ctx, n):
    A, B, C, D = oracle.init_mm3(n)
    dA, dB, dC, dD = (ctx.upload(x) for x in (A, B, C, D))
    dE, dF, dG = (ctx.alloc(n * n * 4) for _ in range(3))
    ctx.gemm(P, n, n, n, 1.0, dA, n, dB, n, 0.0, dE, n)
    ctx.gemm(P, n, n, n, 1.0, dC, n, dD, n, 0.0, dF, n)
    ctx.gemm(P, n, n, n, 1.0, dE, n, dF, n, 0.0, dG, n)
    ctx.synchronize()
    assert_verify(oracle.host_mm3(n), ctx.download(dG, (n, n)))


def test_invalid_arguments_are_rejected(ctx):
    with pytest.raises(gbpoly.GbpolyError) as e:
        ctx.gemm(P, 4, 4, 4, 1.0, 0, 4, 0, 4, 0.0, 0, 4)
    assert e.value.status == gbpoly.Status.INVALID
    with pytest.raises(gbpoly.GbpolyError) as e:
        ctx.gemm(P, -1, 4, 4, 1.0, 0, 4, 0, 4, 0.0, 0, 4)
    assert e.value.status == gbpoly.Status.INVALID
    buf = ctx.alloc(64)
    with pytest.raises(gbpoly.GbpolyError) as e:
        ctx.gemm(P, 4, 4, 4, 1.0, buf, 2, buf, 4, 0.0, buf, 4)  # lda < K
    assert e.value.status == gbpoly.Status.INVALID
    ctx.synchronize()


@pytest.mark.parametrize("N,ldc", [(96, 104), (90, 100), (128, 132)])
def test_gemm_leaves_the_padding_of_ldc(ctx, N, ldc):
    # row ends on and off 16-byte boundaries: the padding keeps its values
    rng = np.random.default_rng(N * ldc)
    M, K = 150, 70
    A = rng.uniform(-1, 1, (M, K)).astype(np.float32)
    B = rng.uniform(-1, 1, (K, N)).astype(np.float32)
    Cp = rng.uniform(-1, 1, (M, ldc)).astype(np.float32)
    out = run_gemm(ctx, A, B, Cp, 1.0, 1.0, ldc=ldc)
    np.testing.assert_array_equal(out[:, N:], Cp[:, N:])
    ref = oracle.gemm_f64(A, B, np.ascontiguousarray(Cp[:, :N]), 1.0, 1.0)
    assert oracle.error_norms(np.ascontiguousarray(out[:, :N]), ref)[1] < 1e-5
