"""Stage chains captured into one CUDA graph replay the eager result
(2mm: C += A.B then E = C.D, 2mm.cpp:94-123) for the plain and split forms."""
import numpy as np
import pytest

import gbpoly
import oracle
from gbpoly import Precision

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("prec", [Precision.FP32, Precision.BF16X3, Precision.BF16X6, Precision.FP16X3])
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


@pytest.mark.parametrize("prec", [Precision.BF16X3, Precision.TF32X3, Precision.BF16X6, Precision.FP16X3, Precision.TF32])
@pytest.mark.parametrize("mnk", [(1000, 700, 333), (2304, 2048, 512), (130, 4100, 70)])
def test_workspace_query_covers_every_configuration(prec, mnk):
    """A fresh context reserved with gbpoly_workspace_query's bytes captures the
    call in every tile configuration without growing its workspace (fp16x3's
    block-scale tables and the K-split tail's partial sums included)."""
    M, N, K = mnk
    rng = np.random.default_rng(M + N + K)
    A = rng.uniform(-1, 1, (M, K)).astype(np.float32)
    B = rng.uniform(-1, 1, (K, N)).astype(np.float32)
    ref = oracle.gemm_f64(A, B, None, 1.0, 0.0)
    with gbpoly.Context(0) as fresh:
        dA, dB, dC = fresh.upload(A), fresh.upload(B), fresh.alloc(M * N * 4)
        fresh.workspace_reserve(fresh.workspace_query(prec, M, N, K))
        for cfg in range(fresh.config_count(prec)):
            fresh.config_set(prec, M, N, K, cfg)
            fresh.graph_begin()
            try:
                fresh.gemm(prec, M, N, K, 1.0, dA, K, dB, N, 0.0, dC, N)
            finally:
                g = fresh.graph_end()
            fresh.graph_launch(g)
            fresh.synchronize()
            fresh.graph_destroy(g)
            bound = 1e-3 if prec == Precision.TF32 else 2e-5
            assert oracle.error_norms(fresh.download(dC, (M, N)), ref)[1] < bound, cfg
