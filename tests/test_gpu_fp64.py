"""FP64 on the GPU through the C ABI: the oracle DGEMM and the double
variants' syrk/syr2k (gbpoly_gemm_f64, gbpoly_syrk_f64, gbpoly_syr2k_f64).

Tolerance: relative Frobenius 1e-13 against numpy's float64 products (both
are FP64 sums in different orders).  Symmetric products compute the lower
triangle of 64 x 64 tiles and mirror it: bit-identical to the full square
computed from a distinct copy of the operand.
"""
import numpy as np
import pytest

from gbpoly import Op

pytestmark = pytest.mark.gpu


def rel(got, ref):
    return float(np.linalg.norm(got - ref) / max(np.linalg.norm(ref), 1e-300))


@pytest.mark.parametrize("ops", [(Op.N, Op.N), (Op.N, Op.T), (Op.T, Op.N), (Op.T, Op.T)])
@pytest.mark.parametrize("M,N,K", [(1, 1, 1), (65, 130, 33), (300, 200, 257)])
def test_dgemm_against_numpy(ctx, ops, M, N, K):
    rng = np.random.default_rng(M * N + K)
    A = rng.standard_normal((K, M) if ops[0] == Op.T else (M, K))
    B = rng.standard_normal((N, K) if ops[1] == Op.T else (K, N))
    C = rng.standard_normal((M, N))
    dA, dB, dC = ctx.upload(A), ctx.upload(B), ctx.upload(C)
    ctx.gemm_f64(M, N, K, 1.5, dA, A.shape[1], dB, B.shape[1], -0.25, dC, N, op_a=ops[0], op_b=ops[1])
    ctx.synchronize()
    a = A.T if ops[0] == Op.T else A
    b = B.T if ops[1] == Op.T else B
    assert rel(ctx.download(dC, C.shape, np.float64), 1.5 * a @ b - 0.25 * C) < 1e-13
    for x in (dA, dB, dC):
        ctx.free(x)


@pytest.mark.parametrize("n,k", [(64, 64), (200, 90), (517, 300)])
def test_syrk_syr2k_f64_against_numpy(ctx, n, k):
    rng = np.random.default_rng(n + k)
    A = rng.standard_normal((n, k))
    B = rng.standard_normal((n, k))
    C = rng.standard_normal((n, n))  # not symmetric: the mirrored tiles read their own C
    dA, dB = ctx.upload(A), ctx.upload(B)
    dC = ctx.upload(C)
    ctx.syrk_f64(n, k, 2.0, dA, k, 0.5, dC, n)
    ctx.synchronize()
    assert rel(ctx.download(dC, C.shape, np.float64), 2.0 * A @ A.T + 0.5 * C) < 1e-13
    ctx.free(dC)
    dC = ctx.upload(C)
    ctx.syr2k_f64(n, k, -1.0, dA, k, dB, k, 1.0, dC, n)
    ctx.synchronize()
    assert rel(ctx.download(dC, C.shape, np.float64), -(A @ B.T + B @ A.T) + C) < 1e-13
    for x in (dA, dB, dC):
        ctx.free(x)


def test_symmetric_dgemm_is_bitwise_the_full_square(ctx):
    n, k = 333, 129
    rng = np.random.default_rng(5)
    A = rng.standard_normal((n, k))
    C = rng.standard_normal((n, n))
    dA, dA2 = ctx.upload(A), ctx.upload(A)
    d1, d2 = ctx.upload(C), ctx.upload(C)
    ctx.gemm_f64(n, n, k, 1.25, dA, k, dA, k, -0.5, d1, n, op_a=Op.N, op_b=Op.T)   # triangle + mirror
    ctx.gemm_f64(n, n, k, 1.25, dA, k, dA2, k, -0.5, d2, n, op_a=Op.N, op_b=Op.T)  # every tile
    ctx.synchronize()
    tri, full = ctx.download(d1, C.shape, np.float64), ctx.download(d2, C.shape, np.float64)
    np.testing.assert_array_equal(tri.view(np.uint64), full.view(np.uint64))
    for x in (dA, dA2, d1, d2):
        ctx.free(x)
