"""The matrix-vector entry points on the GPU, through the C ABI, against the
oracle and FP64.

Tolerances:
  * the four benchmarks on their own inputs: the reference's verify rule,
    percentDiff <= 0.05 percent per output element against its FP32 host
    loop (atax.cpp:100-120, bicg.cpp:102-124, mvt.cpp:100-124,
    gesummv.cpp:100-117);
  * seeded inputs: relative error of each output vector against FP64 at most
    1e-5 in the Frobenius norm (FP32 sums of up to 5000 terms);
  * beta/alpha handling and empty shapes: exact.
"""
import numpy as np
import pytest

import gbpoly
import oracle
from gbpoly import Op

pytestmark = pytest.mark.gpu

SIZES = [1, 2, 7, 16, 37, 64, 100, 255, 256, 1023, 1024, 1025, 2048, 3000]


def rel(got, ref):
    return float(np.linalg.norm(got.astype(np.float64) - ref) / max(np.linalg.norm(ref), 1e-300))


def assert_verifies(host, dev):
    first, max_pd, nfail = oracle.verify(host, dev)
    assert first == -1, f"{nfail} elements over 0.05%, first at {first}, max percentDiff {max_pd}"


@pytest.mark.parametrize("n", SIZES)
def test_atax_verifies(ctx, n):
    A, x = oracle.init_atax(n)
    dA, dx = ctx.upload(A), ctx.upload(x)
    dt, dy = ctx.upload(np.zeros(n, np.float32)), ctx.upload(np.zeros(n, np.float32))
    ctx.gemv(Op.N, n, n, 1.0, dA, n, dx, 1.0, dt)
    ctx.gemv(Op.T, n, n, 1.0, dA, n, dt, 1.0, dy)
    ctx.synchronize()
    assert_verifies(oracle.host_atax(n), ctx.download(dy, (n,)))
    for b in (dA, dx, dt, dy):
        ctx.free(b)


@pytest.mark.parametrize("n", SIZES + [4096, 4100, 5000, 8192, 8196])
def test_atax_one_call_verifies(ctx, n):
    # gbpoly_atax_f32: one kernel up to 8192 aligned columns, two passes beyond or unaligned
    A, x = oracle.init_atax(n)
    dA, dx = ctx.upload(A), ctx.upload(x)
    dt, dy = ctx.upload(np.zeros(n, np.float32)), ctx.upload(np.zeros(n, np.float32))
    ctx.atax(n, n, dA, n, dx, dt, dy)
    ctx.synchronize()
    assert_verifies(oracle.host_atax(n), ctx.download(dy, (n,)))
    for b in (dA, dx, dt, dy):
        ctx.free(b)


@pytest.mark.parametrize("rows,cols", [(3001, 4096), (17, 1024), (4096, 3072), (1000, 2052)])
def test_atax_seeded_against_fp64(ctx, rows, cols):
    rng = np.random.default_rng(rows + cols)
    A = rng.standard_normal((rows, cols)).astype(np.float32)
    x = rng.standard_normal(cols).astype(np.float32)
    t0 = rng.standard_normal(rows).astype(np.float32)
    y0 = rng.standard_normal(cols).astype(np.float32)
    dA, dx, dt, dy = ctx.upload(A), ctx.upload(x), ctx.upload(t0), ctx.upload(y0)
    ctx.atax(rows, cols, dA, cols, dx, dt, dy)
    ctx.synchronize()
    a = A.astype(np.float64)
    t = t0 + a @ x.astype(np.float64)
    y = y0 + a.T @ t
    assert rel(ctx.download(dt, (rows,)), t) < 1e-5
    assert rel(ctx.download(dy, (cols,)), y) < 1e-5
    for b in (dA, dx, dt, dy):
        ctx.free(b)


@pytest.mark.parametrize("n", SIZES)
def test_bicg_verifies(ctx, n):
    A, p, r = oracle.init_bicg(n)
    dA, dp, dr = ctx.upload(A), ctx.upload(p), ctx.upload(r)
    ds, dq = ctx.upload(np.zeros(n, np.float32)), ctx.upload(np.zeros(n, np.float32))
    ctx.gemv_pair(n, n, dA, n, [(Op.T, 1.0, 1.0, dr, ds), (Op.N, 1.0, 1.0, dp, dq)])
    ctx.synchronize()
    got = np.concatenate([ctx.download(ds, (n,)), ctx.download(dq, (n,))])
    assert_verifies(oracle.host_bicg(n), got)
    for b in (dA, dp, dr, ds, dq):
        ctx.free(b)


@pytest.mark.parametrize("n", SIZES)
def test_mvt_verifies(ctx, n):
    a, x1, x2, y1, y2 = oracle.init_mvt(n)
    da, d1, d2, e1, e2 = (ctx.upload(v) for v in (a, x1, x2, y1, y2))
    ctx.gemv_pair(n, n, da, n, [(Op.N, 1.0, 1.0, e1, d1), (Op.N, 1.0, 1.0, e2, d2)])
    ctx.synchronize()
    got = np.concatenate([ctx.download(d1, (n,)), ctx.download(d2, (n,))])
    assert_verifies(oracle.host_mvt(n), got)
    for b in (da, d1, d2, e1, e2):
        ctx.free(b)


@pytest.mark.parametrize("n", SIZES)
def test_gesummv_verifies(ctx, n):
    A, B, x = oracle.init_gesummv(n)
    dA, dB, dx = ctx.upload(A), ctx.upload(B), ctx.upload(x)
    dt, dy = ctx.upload(np.zeros(n, np.float32)), ctx.upload(np.zeros(n, np.float32))
    ctx.gesummv(n, n, 1.0, dA, n, dB, n, dx, 1.0, dt, dy)
    ctx.synchronize()
    assert_verifies(oracle.host_gesummv(n), ctx.download(dy, (n,)))
    np.testing.assert_array_equal(ctx.download(dt, (n,)), np.full(n, 2.0 * n, np.float32))
    for b in (dA, dB, dx, dt, dy):
        ctx.free(b)


# rows x cols with a padded leading dimension; ragged and unaligned shapes take the scalar path
@pytest.mark.parametrize("rows,cols,ld", [(5000, 300, 300), (300, 5000, 5003), (1, 1, 1), (33, 1030, 1032),
                                          (4097, 4099, 4099), (2048, 2048, 2056)])
def test_seeded_products_against_fp64(ctx, rows, cols, ld):
    rng = np.random.default_rng(rows * 7 + cols)
    A = rng.standard_normal((rows, ld)).astype(np.float32)
    xr = rng.standard_normal(cols).astype(np.float32)
    xc = rng.standard_normal(rows).astype(np.float32)
    y0r = rng.standard_normal(rows).astype(np.float32)
    y0c = rng.standard_normal(cols).astype(np.float32)
    dA, dxr, dxc = ctx.upload(A), ctx.upload(xr), ctx.upload(xc)
    dyr, dyc = ctx.upload(y0r), ctx.upload(y0c)
    ctx.gemv_pair(rows, cols, dA, ld, [(Op.N, 1.5, -0.5, dxr, dyr), (Op.T, -2.0, 0.25, dxc, dyc)])
    ctx.synchronize()
    a = A[:, :cols].astype(np.float64)
    ref_r = 1.5 * (a @ xr.astype(np.float64)) - 0.5 * y0r
    ref_c = -2.0 * (a.T @ xc.astype(np.float64)) + 0.25 * y0c
    assert rel(ctx.download(dyr, (rows,)), ref_r) < 1e-5
    assert rel(ctx.download(dyc, (cols,)), ref_c) < 1e-5
    # the padding columns beyond cols are never read: poison them and recompute the row product
    A2 = A.copy()
    A2[:, cols:] = np.nan
    dA2 = ctx.upload(A2)
    dyr2 = ctx.upload(np.zeros(rows, np.float32))
    ctx.gemv(Op.N, rows, cols, 1.0, dA2, ld, dxr, 0.0, dyr2)
    ctx.synchronize()
    assert np.isfinite(ctx.download(dyr2, (rows,))).all()
    for b in (dA, dxr, dxc, dyr, dyc, dA2, dyr2):
        ctx.free(b)


def test_deterministic_and_beta_zero_ignores_nan(ctx):
    n = 3001
    rng = np.random.default_rng(3)
    A = rng.standard_normal((n, n)).astype(np.float32)
    x = rng.standard_normal(n).astype(np.float32)
    dA, dx = ctx.upload(A), ctx.upload(x)
    outs = []
    for _ in range(2):
        dy = ctx.upload(np.full(n, np.nan, np.float32))
        ctx.gemv(Op.T, n, n, 1.0, dA, n, dx, 0.0, dy)  # beta = 0: y is not read
        ctx.synchronize()
        outs.append(ctx.download(dy, (n,)))
        ctx.free(dy)
    assert np.isfinite(outs[0]).all()
    np.testing.assert_array_equal(outs[0].view(np.uint32), outs[1].view(np.uint32))
    ctx.free(dA)
    ctx.free(dx)


def test_empty_shapes_scale_y(ctx):
    y = np.arange(1, 6, dtype=np.float32)
    dy = ctx.upload(y)
    dx = ctx.upload(np.zeros(1, np.float32))
    ctx.gemv(Op.N, 5, 0, 1.0, None, 1, dx, 2.0, dy)  # no columns: y = 2 y
    ctx.synchronize()
    np.testing.assert_array_equal(ctx.download(dy, (5,)), 2 * y)
    with pytest.raises(gbpoly.GbpolyError):
        ctx.gemv_pair(4, 4, dy, 4, [(Op.T, 1.0, 1.0, dx, dy), (Op.T, 1.0, 1.0, dx, dy)])
    ctx.free(dy)
    ctx.free(dx)
