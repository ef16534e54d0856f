"""Covariance and correlation on the GPU, through the C ABI, against the oracle.

The column passes (gbpoly_column_mean_f32, gbpoly_column_stddev_f32,
gbpoly_center_columns_f32, gbpoly_set_diagonal_f32) and the symmetric X^T.X
contraction (gbpoly_gemm_f32 with op_a = T, op_b = N, A == B) are chained as
polybench/covariance.cpp:80-127 and polybench/correlation.cpp:107-187 chain
their kernels, on the reference's own (n + 1) x (n + 1) arrays.

Tolerances:
  * whole benchmarks: the reference's verify rule, percentDiff <= 0.05 percent
    for every interior element against its FP32 host loop (covariance.cpp:
    129-152, correlation.cpp:189-214), for the plain form and the split forms;
  * column means and standard deviations: relative 1e-6 against FP64 sums of
    the same FP32 data (the device sums in a fixed two-level order, the
    reference sequentially);
  * centring: bit-exact against the same FP32 operations in numpy, given the
    device's means and standard deviations;
  * the FP32 symmetric contraction (lower triangle of tiles, mirrored):
    bit-exact against the full-square contraction of the same data.
"""
import numpy as np
import pytest

import gbpoly
import oracle
from gbpoly import Op, Precision

pytestmark = pytest.mark.gpu

COV_FLOAT_N = np.float32(3214212.01)          # covariance.cpp:18
CORR_FLOAT_N = 3214212.01                     # correlation.cpp:12 (double)
CORR_EPS = 0.005
SIZES = [1, 2, 7, 16, 37, 64, 100, 255, 256, 257, 640, 1024]
FORMS = [Precision.FP32, Precision.BF16X3, Precision.TF32X3, Precision.BF16X6, Precision.FP16X3]


def ldp_of(n):
    return (n + 31) // 32 * 32


def covariance_gpu(ctx, prec, data, n):
    ld, ldp = n + 1, ldp_of(n)
    d = ctx.upload(data)
    mean = ctx.upload(np.zeros(ld, np.float32))
    S = ctx.upload(np.zeros((ld, ld), np.float32))
    Y = ctx.alloc(max(n * ldp, 1) * 4)
    X, mu, Sint = d.ptr + (ld + 1) * 4, mean.ptr + 4, S.ptr + (ld + 1) * 4
    ctx.column_mean(n, n, X, ld, COV_FLOAT_N, mu)
    ctx.center_columns(n, n, X, ld, mu, None, 1.0, Y, ldp)
    ctx.gemm(prec, n, n, n, 1.0, Y, ldp, Y, ldp, 0.0, Sint, ld, op_a=Op.T, op_b=Op.N)
    ctx.synchronize()
    out = ctx.download(S, (ld, ld))
    for b in (d, mean, S, Y):
        ctx.free(b)
    return out


def correlation_gpu(ctx, prec, data, n):
    ld, ldp = n + 1, ldp_of(n)
    d = ctx.upload(data)
    mean = ctx.upload(np.zeros(ld, np.float32))
    sd = ctx.upload(np.zeros(ld, np.float32))
    S = ctx.upload(np.zeros((ld, ld), np.float32))
    Y = ctx.alloc(max(n * ldp, 1) * 4)
    X, mu, sdp, Sint = d.ptr + (ld + 1) * 4, mean.ptr + 4, sd.ptr + 4, S.ptr + (ld + 1) * 4
    ctx.column_mean(n, n, X, ld, np.float32(CORR_FLOAT_N), mu)
    ctx.column_stddev(n, n, X, ld, mu, np.float32(CORR_FLOAT_N), np.float32(CORR_EPS), sdp)
    ctx.center_columns(n, n, X, ld, mu, sdp, np.float32(np.sqrt(CORR_FLOAT_N)), Y, ldp)
    ctx.gemm(prec, n, n, n, 1.0, Y, ldp, Y, ldp, 0.0, Sint, ld, op_a=Op.T, op_b=Op.N)
    ctx.set_diagonal(n, 1.0, Sint, ld)
    ctx.synchronize()
    out = ctx.download(S, (ld, ld))
    for b in (d, mean, sd, S, Y):
        ctx.free(b)
    return out


def assert_interior_verifies(host, dev):
    first, max_pd, nfail = oracle.verify(host[1:, 1:], dev[1:, 1:])
    assert first == -1, f"{nfail} elements over 0.05%, first at {first}, max percentDiff {max_pd}"


@pytest.mark.parametrize("prec", FORMS, ids=lambda p: p.name.lower())
@pytest.mark.parametrize("n", SIZES)
def test_covariance_verifies_against_host_loop(ctx, prec, n):
    got = covariance_gpu(ctx, prec, oracle.init_covariance(n), n)
    assert_interior_verifies(oracle.host_covariance(n), got)
    assert not got[0].any() and not got[:, 0].any()  # row and column 0 untouched


@pytest.mark.parametrize("prec", FORMS, ids=lambda p: p.name.lower())
@pytest.mark.parametrize("n", SIZES)
def test_correlation_verifies_against_host_loop(ctx, prec, n):
    got = correlation_gpu(ctx, prec, oracle.init_correlation(n), n)
    host = oracle.host_correlation(n)
    assert_interior_verifies(host, got)
    assert (np.diag(got)[1:] == 1.0).all()


def test_covariance_fp32_seeded_error_vs_fp64(ctx):
    n = 700
    rng = np.random.default_rng(5)
    data = rng.standard_normal((n + 1, n + 1)).astype(np.float32)
    got = covariance_gpu(ctx, Precision.FP32, data, n)[1:, 1:]
    x = data[1:, 1:].astype(np.float64)
    x = x - x.sum(axis=0) / float(COV_FLOAT_N)
    ref = x.T @ x
    frob = np.linalg.norm(got - ref) / np.linalg.norm(ref)
    assert frob < 2e-6, frob


def test_column_statistics_against_fp64(ctx):
    rows, cols, ldx = 3001, 777, 801
    rng = np.random.default_rng(9)
    X = rng.uniform(-2, 5, (rows, ldx)).astype(np.float32)
    dX = ctx.upload(X)
    dm, ds = ctx.alloc(cols * 4), ctx.alloc(cols * 4)
    ctx.column_mean(rows, cols, dX, ldx, np.float32(rows), dm)
    ctx.column_stddev(rows, cols, dX, ldx, dm, np.float32(rows), np.float32(0.0), ds)
    ctx.synchronize()
    m = ctx.download(dm, (cols,))
    s = ctx.download(ds, (cols,))
    x = X[:, :cols].astype(np.float64)
    np.testing.assert_allclose(m, x.mean(axis=0), rtol=1e-6)
    ref_s = np.sqrt(((x - m.astype(np.float64)) ** 2).sum(axis=0) / rows)
    np.testing.assert_allclose(s, ref_s, rtol=1e-6)
    # eps clamp: a constant column has deviation 0 -> 1
    Z = np.full((64, 32), 3.0, np.float32)
    dZ = ctx.upload(Z)
    ctx.column_mean(64, 32, dZ, 32, np.float32(64), dm)
    ctx.column_stddev(64, 32, dZ, 32, dm, np.float32(64), np.float32(0.005), ds)
    ctx.synchronize()
    assert (ctx.download(ds, (32,)) == 1.0).all()
    for b in (dX, dm, ds, dZ):
        ctx.free(b)


def test_centering_is_bitwise_and_in_place(ctx):
    rows, cols, ld = 517, 300, 301
    rng = np.random.default_rng(2)
    X = rng.uniform(0, 100, (rows, ld)).astype(np.float32)
    mu = rng.uniform(0, 1, cols).astype(np.float32)
    sd = rng.uniform(0.5, 2, cols).astype(np.float32)
    c = np.float32(np.sqrt(CORR_FLOAT_N))
    dX, dm, ds = ctx.upload(X), ctx.upload(mu), ctx.upload(sd)
    dY = ctx.alloc(rows * 320 * 4)
    ctx.center_columns(rows, cols, dX, ld, dm, ds, c, dY, 320)
    ctx.center_columns(rows, cols, dX, ld, dm, None, 1.0, dX, ld)  # in place
    ctx.synchronize()
    Y = ctx.download(dY, (rows, 320))[:, :cols]
    Xc = ctx.download(dX, (rows, ld))
    ref_scaled = ((X[:, :cols] - mu) / c) / sd
    np.testing.assert_array_equal(Y.view(np.uint32), ref_scaled.astype(np.float32).view(np.uint32))
    np.testing.assert_array_equal(Xc[:, :cols].view(np.uint32), (X[:, :cols] - mu).view(np.uint32))
    np.testing.assert_array_equal(Xc[:, cols:], X[:, cols:])  # padding column untouched
    with pytest.raises(gbpoly.GbpolyError):
        ctx.center_columns(rows, cols, dX, ld, dm, None, 1.0, dX, ld + 1)
    for b in (dX, dm, ds, dY):
        ctx.free(b)


@pytest.mark.parametrize("n", [100, 300, 513])
@pytest.mark.parametrize("ops", [(Op.N, Op.T), (Op.T, Op.N)], ids=["AAt", "AtA"])
def test_fp32_symmetric_triangle_is_bitwise_the_full_square(ctx, n, ops):
    # same stored matrix for both operands -> lower triangle of tiles + mirror;
    # a distinct copy -> every tile computed.  beta != 0 on a non-symmetric C.
    rng = np.random.default_rng(n)
    # op_a = N: A stored M x K; op_a = T: A stored K x M.  Leading dimension a
    # multiple of 4 floats, so the TMA-fed kernel (not the unaligned fallback) runs.
    M, K = (n, n + 3) if ops[0] == Op.N else (n + 8, n)
    rows, cols = (M, K) if ops[0] == Op.N else (K, M)
    lda = (cols + 3) // 4 * 4
    A = rng.uniform(-1, 1, (rows, lda)).astype(np.float32)
    C = rng.uniform(-1, 1, (M, M)).astype(np.float32)
    dA, dA2 = ctx.upload(A), ctx.upload(A)
    d1, d2 = ctx.upload(C), ctx.upload(C)
    ctx.gemm(Precision.FP32, M, M, K, 1.25, dA, lda, dA, lda, -0.5, d1, M, op_a=ops[0], op_b=ops[1])
    ctx.gemm(Precision.FP32, M, M, K, 1.25, dA, lda, dA2, lda, -0.5, d2, M, op_a=ops[0], op_b=ops[1])
    ctx.synchronize()
    tri, full = ctx.download(d1, C.shape), ctx.download(d2, C.shape)
    np.testing.assert_array_equal(tri.view(np.uint32), full.view(np.uint32))
    for b in (dA, dA2, d1, d2):
        ctx.free(b)


def test_fp32_syr2k_triangle_against_fp64(ctx):
    n, k = 389, 211
    rng = np.random.default_rng(4)
    A = rng.uniform(-1, 1, (n, k)).astype(np.float32)
    B = rng.uniform(-1, 1, (n, k)).astype(np.float32)
    C = rng.uniform(-1, 1, (n, n)).astype(np.float32)  # not symmetric
    dA, dB, dC = ctx.upload(A), ctx.upload(B), ctx.upload(C)
    ctx.syr2k(Precision.FP32, n, k, 2.0, dA, k, dB, k, 0.75, dC, n)
    ctx.synchronize()
    got = ctx.download(dC, C.shape)
    a, b = A.astype(np.float64), B.astype(np.float64)
    ref = 2.0 * (a @ b.T + b @ a.T) + 0.75 * C.astype(np.float64)
    assert np.linalg.norm(got - ref) / np.linalg.norm(ref) < 2e-6
    for x in (dA, dB, dC):
        ctx.free(x)


@pytest.mark.parametrize("prec", FORMS + [Precision.TF32, Precision.FP8], ids=lambda p: p.name.lower())
@pytest.mark.parametrize("n", [100, 257, 640])
@pytest.mark.parametrize("scaled", [False, True], ids=["covariance", "correlation"])
def test_covariance_call_is_bitwise_the_chain(ctx, prec, n, scaled):
    # gbpoly_covariance_f32 (the split forms centre inside their split pass)
    # gives the bits of centring into a copy and contracting the copy
    ld, ldp = n + 1, ldp_of(n)
    data = oracle.init_correlation(n) if scaled else oracle.init_covariance(n)
    d = ctx.upload(data)
    mean, sd = ctx.upload(np.zeros(ld, np.float32)), ctx.upload(np.zeros(ld, np.float32))
    S1, S2 = ctx.upload(np.zeros((ld, ld), np.float32)), ctx.upload(np.zeros((ld, ld), np.float32))
    Y = ctx.alloc(max(n * ldp, 1) * 4)
    X, mu, sdp = d.ptr + (ld + 1) * 4, mean.ptr + 4, sd.ptr + 4
    fn = np.float32(CORR_FLOAT_N) if scaled else COV_FLOAT_N
    ctx.column_mean(n, n, X, ld, fn, mu)
    if scaled:
        ctx.column_stddev(n, n, X, ld, mu, fn, np.float32(CORR_EPS), sdp)
    div = np.float32(np.sqrt(CORR_FLOAT_N)) if scaled else np.float32(1.0)
    ctx.center_columns(n, n, X, ld, mu, sdp if scaled else None, div, Y, ldp)
    ctx.gemm(prec, n, n, n, 1.0, Y, ldp, Y, ldp, 0.0, S1.ptr + (ld + 1) * 4, ld, op_a=Op.T, op_b=Op.N)
    ctx.covariance(prec, n, n, X, ld, mu, sdp if scaled else None, div, S2.ptr + (ld + 1) * 4, ld)
    ctx.synchronize()
    a, b = ctx.download(S1, (ld, ld)), ctx.download(S2, (ld, ld))
    np.testing.assert_array_equal(b.view(np.uint32), a.view(np.uint32))
    for buf in (d, mean, sd, S1, S2, Y):
        ctx.free(buf)
