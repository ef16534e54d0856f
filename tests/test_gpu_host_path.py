"""Host-buffer contraction (gbpoly_gemm_f32_host): operands in host memory,
copies pipelined over row panels inside the call.  Results must equal the
device-buffer entry point's for the same form, bit for bit (same kernels on
the same data), including ragged panel edges and padded leading dimensions."""
import ctypes as ct

import numpy as np
import pytest

from gbpoly import Op, Precision

pytestmark = pytest.mark.gpu


def pinned(ctx, arr):
    p = ct.c_void_p()
    assert ctx.lib.gbpoly_host_alloc(ctx.handle, ct.byref(p), arr.nbytes) == 0
    view = np.ctypeslib.as_array((ct.c_float * arr.size).from_address(p.value)).reshape(arr.shape)
    view[...] = arr
    return p, view


@pytest.mark.parametrize("prec", [Precision.FP32, Precision.BF16X3, Precision.BF16X6, Precision.TF32X3])
@pytest.mark.parametrize("shape", [(4500, 700, 300), (2048, 512, 1024), (100, 60, 40)])
def test_host_path_equals_device_path(ctx, prec, shape):
    M, N, K = shape
    rng = np.random.default_rng(M + N)
    A = rng.uniform(-1, 1, (M, K + 3)).astype(np.float32)   # lda = K + 3
    B = rng.uniform(-1, 1, (K, N)).astype(np.float32)
    C = rng.uniform(-1, 1, (M, N + 5)).astype(np.float32)   # ldc = N + 5
    dA, dB, dC = ctx.upload(A), ctx.upload(B), ctx.upload(C)
    ctx.gemm(prec, M, N, K, 1.5, dA, K + 3, dB, N, -0.5, dC, N + 5)
    ctx.synchronize()
    ref = ctx.download(dC, C.shape)
    pa, hA = pinned(ctx, A)
    pb, hB = pinned(ctx, B)
    pc, hC = pinned(ctx, C)
    ctx.gemm_host(prec, M, N, K, 1.5, pa.value, K + 3, pb.value, N, -0.5, pc.value, N + 5)
    ctx.synchronize()
    np.testing.assert_array_equal(hC[:, :N], ref[:, :N])
    np.testing.assert_array_equal(hC[:, N:], C[:, N:])  # padding untouched
    for p in (pa, pb, pc):
        ctx.lib.gbpoly_host_free(ctx.handle, p)


def test_host_path_transposed_and_pageable(ctx):
    M, N, K = 700, 300, 200
    rng = np.random.default_rng(9)
    A = rng.uniform(-1, 1, (K, M)).astype(np.float32)
    B = rng.uniform(-1, 1, (N, K)).astype(np.float32)
    C = np.zeros((M, N), np.float32)
    out = C.copy()
    ctx.gemm_host(Precision.BF16X3, M, N, K, 1.0, A, M, B, K, 0.0, out, N, op_a=Op.T, op_b=Op.T)  # pageable numpy memory
    ctx.synchronize()
    ref = A.T.astype(np.float64) @ B.T.astype(np.float64)
    assert np.linalg.norm(out - ref) / np.linalg.norm(ref) < 2e-5
