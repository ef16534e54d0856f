"""gbpoly_stream_hold / gbpoly_stream_release through the C ABI: work queued
behind a hold starts once the host releases it, and a hold nobody releases
ends by itself after its timeout (the waiting kernel is bounded), leaving the
context usable."""
import time

import numpy as np
import pytest

from gbpoly import Op, Precision

pytestmark = pytest.mark.gpu


def small_gemm(ctx, dA, dC, n):
    ctx.gemm(Precision.FP32, n, n, n, 1.0, dA, n, dA, n, 0.0, dC, n, op_a=Op.N, op_b=Op.N)


def test_hold_then_release_runs_the_queued_work(ctx):
    n = 256
    A = np.eye(n, dtype=np.float32)
    dA, dC = ctx.upload(A), ctx.alloc(n * n * 4)
    ctx.stream_hold(20000)
    e0, e1 = ctx.event(), ctx.event()
    e0.record()
    small_gemm(ctx, dA, dC, n)
    e1.record()
    ctx.stream_release()
    ctx.synchronize()
    assert e0.elapsed_ms(e1) < 20.0  # started on release, not on the timeout
    np.testing.assert_array_equal(ctx.download(dC, (n, n)), A)
    for x in (dA, dC):
        ctx.free(x)


def test_unreleased_hold_ends_after_its_timeout(ctx):
    n = 128
    dA, dC = ctx.upload(np.eye(n, dtype=np.float32)), ctx.alloc(n * n * 4)
    e0, e1 = ctx.event(), ctx.event()
    e0.record()
    ctx.stream_hold(30000)  # 30 ms, never released in time
    small_gemm(ctx, dA, dC, n)
    e1.record()
    t0 = time.time()
    ctx.synchronize()  # returns once the hold has timed out
    waited = time.time() - t0
    assert 0.02 <= e0.elapsed_ms(e1) / 1e3 < 5.0 and waited < 5.0
    ctx.stream_release()
    # the context stays usable: a held-and-released round trip afterwards
    ctx.stream_hold(20000)
    small_gemm(ctx, dA, dC, n)
    ctx.stream_release()
    ctx.synchronize()
    np.testing.assert_array_equal(ctx.download(dC, (n, n)), np.eye(n, dtype=np.float32))
    for x in (dA, dC):
        ctx.free(x)
