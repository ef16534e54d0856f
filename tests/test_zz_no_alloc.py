"""The allocation-free split-BF16 entry point, through the C ABI.

gbpoly_gemm_f32_bf16x3_noalloc serves callers that may not allocate device
memory at call time: it keeps its split panels in a fixed device array
inside the library instead of the context workspace.  Two calls in a row, of
different shapes (the second must not see the first one's panels), must give
what the existing entry point gbpoly_gemm_f32(..., GBPOLY_PREC_BF16X3, ...)
gives, within the split-BF16 tolerance of the other tests (Frobenius 2e-5);
a shape whose panels do not fit is refused with a message.

The file name sorts last so that a run stopping at its first failure has
already run every other test.
"""
import ctypes as ct

import numpy as np
import pytest

import gbpoly
from gbpoly import Op, Precision

pytestmark = pytest.mark.gpu

TOL = 2e-5


def frob_rel(x, ref):
    return float(np.linalg.norm(x.astype(np.float64) - ref) / max(np.linalg.norm(ref.astype(np.float64)), 1e-300))


def call_noalloc(ctx, op_a, op_b, M, N, K, alpha, dA, lda, dB, ldb, beta, dC, ldc) -> int:
    fn = ctx.lib.gbpoly_gemm_f32_bf16x3_noalloc
    return fn(ctx.handle, int(op_a), int(op_b), M, N, K, ct.c_float(alpha), ct.c_void_p(dA.ptr), lda,
              ct.c_void_p(dB.ptr), ldb, ct.c_float(beta), ct.c_void_p(dC.ptr), ldc)


def both_paths(ctx, A, B, C, alpha, beta, op_a, op_b):
    M = A.shape[1] if op_a == Op.T else A.shape[0]
    K = A.shape[0] if op_a == Op.T else A.shape[1]
    N = B.shape[0] if op_b == Op.T else B.shape[1]
    dA, dB = ctx.upload(A), ctx.upload(B)
    d_ref, d_new = ctx.upload(C), ctx.upload(C)
    ctx.gemm(Precision.BF16X3, M, N, K, alpha, dA, A.shape[1], dB, B.shape[1], beta, d_ref, N, op_a=op_a, op_b=op_b)
    status = call_noalloc(ctx, op_a, op_b, M, N, K, alpha, dA, A.shape[1], dB, B.shape[1], beta, d_new, N)
    assert status == 0, ctx.lib.gbpoly_last_error()
    ctx.synchronize()
    ref = ctx.download(d_ref, C.shape)
    new = ctx.download(d_new, C.shape)
    for b in (dA, dB, d_ref, d_new):
        ctx.free(b)
    return ref, new


def test_two_calls_match_the_workspace_entry_point(ctx):
    rng = np.random.default_rng(11)
    # call 1: 1024 x 1024 x 1024, both operands as stored
    A = rng.standard_normal((1024, 1024)).astype(np.float32)
    B = rng.standard_normal((1024, 1024)).astype(np.float32)
    C = rng.standard_normal((1024, 1024)).astype(np.float32)
    ref, new = both_paths(ctx, A, B, C, 1.5, -0.5, Op.N, Op.N)
    assert frob_rel(new, ref) < TOL
    # call 2: a smaller, ragged shape with B transposed; stale panels of call 1 must not leak in
    A2 = rng.uniform(-1, 1, (300, 1000)).astype(np.float32)
    B2 = rng.uniform(-1, 1, (200, 1000)).astype(np.float32)
    C2 = rng.uniform(-1, 1, (300, 200)).astype(np.float32)
    ref2, new2 = both_paths(ctx, A2, B2, C2, 2.0, 0.25, Op.N, Op.T)
    assert frob_rel(new2, ref2) < TOL


def test_oversized_shape_is_refused(ctx):
    n = 4096  # (4096 + 4096) x 4096 x 4 bytes = 128 MiB of panels
    d = ctx.alloc(4)
    status = call_noalloc(ctx, Op.N, Op.N, n, n, n, 1.0, d, n, d, n, 0.0, d, n)
    assert status == int(gbpoly.Status.INVALID)
    assert b"bytes" in ctx.lib.gbpoly_last_error()
    ctx.free(d)
    ctx.synchronize()
