"""Stage chains captured into one CUDA graph replay the eager result
(2mm: C += A.B then E = C.D, 2mm.cpp:94-123) for the plain and split forms."""
import numpy as np
import pytest

import gbpoly
import oracle
from gbpoly import Precision

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("prec", [Precision.FP32, Precision.BF16X3, Precision.BF16X6])
def test_2mm_graph_replay_matches_eager(ctx, prec):
    n = 384
    A, B, C, D = oracle.init_mm2(n)
    dA, dB, dD = ctx.upload(A), ctx.upload(B), ctx.upload(D)
    dC, dE = ctx.upload(C), ctx.alloc(n * n * 4)

    def stages():
        ctx.gemm(prec, n, n, n, 1.0, dA, n, dB, n, 1.0, dC, n)
        ctx.gemm(prec, n, n, n, 1.0, dC, n, dD, n, 0.0, dE, n)

    stages()
    ctx.synchronize()
    eager = ctx.download(dE, (n, n))
    ctx.workspace_reserve(ctx.workspace_query(prec, n, n, n))
    ctx.graph_begin()
    try:
        stages()
    finally:
        g = ctx.graph_end()  # a failed call must not leave the stream capturing
    for _ in range(2):  # replay twice, C reset in between (stage 1 accumulates into C)
        ctx.h2d(dC, C)
        ctx.graph_launch(g)
        ctx.synchronize()
        np.testing.assert_array_equal(ctx.download(dE, (n, n)), eager)
    ctx.graph_destroy(g)
    assert oracle.verify(oracle.host_mm2(n), eager)[0] == -1


def test_workspace_growth_during_capture_is_refused():
    n = 2048 + 64
    with gbpoly.Context(0) as fresh:  # its workspace is empty: any tensor-core call must grow it
        d = fresh.alloc(n * n * 4)
        fresh.graph_begin()
        try:
            with pytest.raises(gbpoly.GbpolyError) as e:
                fresh.gemm(Precision.BF16X6, n, n, n, 1.0, d, n, d, n, 0.0, d, n)
        finally:
            g = fresh.graph_end()  # nothing was enqueued: an empty graph
            fresh.graph_destroy(g)
        assert e.value.status == gbpoly.Status.STATE
        fresh.synchronize()
