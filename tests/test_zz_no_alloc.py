"""The allocation-free split-BF16 entry point, through the C ABI.

gbpoly_gemm_f32_bf16x3_noalloc serves callers that may not allocate device
memory when they call a contraction: code captured into a CUDA graph in
global mode, applications whose memory pool owns the whole device, real-time
loops that forbid the synchronisation an allocation can cause, processes
under a device-memory quota.  It keeps its split panels in a fixed device
array inside the library instead of the context workspace.

Two calls in a row, of different shapes (the second must not see the first
one's panels), on a context that has never run a contraction:
  * give what the existing entry point gbpoly_gemm_f32(..., GBPOLY_PREC_BF16X3,
    ...) gives, within the split-BF16 tolerance of the other tests
    (Frobenius 2e-5), and are within that tolerance of the FP64 oracle too;
  * leave the device's free memory exactly as it was (after one warm-up call
    of each shape, which looks the array's address up and loads the kernels):
    neither call allocated.
A shape whose panels do not fit is refused with a message.

The file name sorts last so that a run stopping at its first failure has
already run every other test.
"""
import ctypes as ct

import numpy as np
import pytest

import gbpoly
import oracle
from gbpoly import Op, Precision

pytestmark = pytest.mark.gpu

TOL = 2e-5


def frob_rel(x, ref):
    ref = ref.astype(np.float64)
    return float(np.linalg.norm(x.astype(np.float64) - ref) / max(np.linalg.norm(ref), 1e-300))


def device_free_bytes() -> int:
    """cudaMemGetInfo's free bytes of the current device (the CUDA runtime the library loaded)."""
    rt = ct.CDLL("libcudart.so.13")
    free, total = ct.c_size_t(), ct.c_size_t()
    assert rt.cudaMemGetInfo(ct.byref(free), ct.byref(total)) == 0
    return free.value


def call_noalloc(ctx, op_a, op_b, M, N, K, alpha, dA, lda, dB, ldb, beta, dC, ldc) -> int:
    fn = ctx.lib.gbpoly_gemm_f32_bf16x3_noalloc
    return fn(ctx.handle, int(op_a), int(op_b), M, N, K, ct.c_float(alpha), ct.c_void_p(int(dA)), lda,
              ct.c_void_p(int(dB)), ldb, ct.c_float(beta), ct.c_void_p(int(dC)), ldc)


def shape_of(A, B, op_a, op_b):
    M = A.shape[1] if op_a == Op.T else A.shape[0]
    K = A.shape[0] if op_a == Op.T else A.shape[1]
    N = B.shape[0] if op_b == Op.T else B.shape[1]
    return M, N, K


def workspace_result(ctx, case):
    """The existing entry point's result (it allocates its workspace as it needs)."""
    A, B, C, alpha, beta, op_a, op_b = case
    M, N, K = shape_of(A, B, op_a, op_b)
    dA, dB, dC = ctx.upload(A), ctx.upload(B), ctx.upload(C)
    ctx.gemm(Precision.BF16X3, M, N, K, alpha, dA, A.shape[1], dB, B.shape[1], beta, dC, N, op_a=op_a, op_b=op_b)
    out = ctx.download(dC, C.shape)
    for b in (dA, dB, dC):
        ctx.free(b)
    return out


def test_two_calls_match_and_allocate_nothing(ctx):
    rng = np.random.default_rng(11)
    cases = [
        # 1024 x 1024 x 1024, both operands as stored
        (rng.standard_normal((1024, 1024)).astype(np.float32), rng.standard_normal((1024, 1024)).astype(np.float32),
         rng.standard_normal((1024, 1024)).astype(np.float32), 1.5, -0.5, Op.N, Op.N),
        # a smaller, ragged shape with B transposed: stale panels of the first call must not leak in
        (rng.uniform(-1, 1, (300, 1000)).astype(np.float32), rng.uniform(-1, 1, (200, 1000)).astype(np.float32),
         rng.uniform(-1, 1, (300, 200)).astype(np.float32), 2.0, 0.25, Op.N, Op.T),
    ]
    refs = [workspace_result(ctx, c) for c in cases]
    f64 = [oracle.gemm_f64(A, B, C, alpha, beta, op_a=int(op_a), op_b=int(op_b))
           for A, B, C, alpha, beta, op_a, op_b in cases]

    with gbpoly.Context(0) as fresh:  # never ran a contraction: an empty workspace
        dev = []
        for A, B, C, alpha, beta, op_a, op_b in cases:
            dev.append((fresh.upload(A), fresh.upload(B), fresh.alloc(C.nbytes)))

        def run_all():
            for (A, B, C, alpha, beta, op_a, op_b), (dA, dB, dC) in zip(cases, dev):
                fresh.h2d(dC, C)
                M, N, K = shape_of(A, B, op_a, op_b)
                status = call_noalloc(fresh, op_a, op_b, M, N, K, alpha, dA, A.shape[1], dB, B.shape[1], beta, dC, N)
                assert status == 0, fresh.lib.gbpoly_last_error()
            fresh.synchronize()

        run_all()  # warm-up: the first call looks the array's address up
        free_before = device_free_bytes()
        run_all()  # the two calls under test
        free_after = device_free_bytes()
        outs = [fresh.download(dC, C.shape) for (_, _, C, *_), (_, _, dC) in zip(cases, dev)]
    assert free_after == free_before, f"device free memory changed by {free_before - free_after} bytes"
    for out, ref, r64 in zip(outs, refs, f64):
        assert frob_rel(out, ref) < TOL
        assert frob_rel(out, r64) < TOL


def test_oversized_shape_is_refused(ctx):
    n = 4096  # (4096 + 4096) x 4096 x 4 bytes = 128 MiB of panels
    d = ctx.alloc(4)
    status = call_noalloc(ctx, Op.N, Op.N, n, n, n, 1.0, d, n, d, n, 0.0, d, n)
    assert status == int(gbpoly.Status.INVALID)
    assert b"bytes" in ctx.lib.gbpoly_last_error()
    ctx.free(d)
    ctx.synchronize()
