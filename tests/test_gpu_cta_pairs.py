"""CTA-pair (cluster of two, cta_group::2) configurations of the tensor-core
forms, through the C ABI: configurations 3 (128-byte rows), 4 (64-byte
rows, deeper pipeline) and 5 (C tile in shared memory, TMA loads and stores
of C) of tf32, bf16x3, tf32x3 and bf16x6 compute 256 x 256
tiles with each CTA holding half of the A and B tiles.  Results against FP64 within each form's bound (the same bounds as
the other configurations), on shapes that leave the second CTA of a pair
beyond the last row, walk several tiles per cluster, and use one or many
pipeline stages.
"""
import numpy as np
import pytest

import oracle
from gbpoly import Op, Precision

pytestmark = pytest.mark.gpu

PAIR_CONFIGS = (3, 4)
BOUND = {Precision.TF32: 1e-3, Precision.BF16X3: 2e-5, Precision.TF32X3: 5e-6, Precision.BF16X6: 5e-6}
FORMS = list(BOUND)


def run_pair(ctx, prec, A, B, C, alpha, beta, op_a=Op.N, op_b=Op.N, config=3):
    M = A.shape[1] if op_a == Op.T else A.shape[0]
    K = A.shape[0] if op_a == Op.T else A.shape[1]
    N = B.shape[0] if op_b == Op.T else B.shape[1]
    assert ctx.config_count(prec) > max(PAIR_CONFIGS)
    ctx.config_set(prec, M, N, K, config)
    dA, dB, dC = ctx.upload(A), ctx.upload(B), ctx.upload(C)
    ctx.gemm(prec, M, N, K, alpha, dA, A.shape[1], dB, B.shape[1], beta, dC, N, op_a=op_a, op_b=op_b)
    ctx.synchronize()
    out = ctx.download(dC, C.shape)
    for b in (dA, dB, dC):
        ctx.free(b)
    ctx.config_set(prec, M, N, K, 0)
    return out


@pytest.mark.parametrize("M,N,K", [(256, 256, 64), (200, 130, 70), (520, 300, 333), (1024, 768, 1024),
                                   (2304, 2048, 512)])
@pytest.mark.parametrize("prec", FORMS, ids=lambda p: p.name.lower())
@pytest.mark.parametrize("config", PAIR_CONFIGS)
def test_pair_configuration_against_fp64(ctx, prec, M, N, K, config):
    rng = np.random.default_rng(M + 7 * N + 13 * K)
    A = rng.standard_normal((M, K)).astype(np.float32)
    B = rng.standard_normal((K, N)).astype(np.float32)
    C = rng.standard_normal((M, N)).astype(np.float32)
    got = run_pair(ctx, prec, A, B, C, 1.25, -0.5, config=config)
    ref = oracle.gemm_f64(A, B, C, 1.25, -0.5)
    frob = oracle.error_norms(got, ref)[1]
    assert frob < BOUND[prec], frob


@pytest.mark.parametrize("ops", [(Op.T, Op.N), (Op.N, Op.T), (Op.T, Op.T)], ids=["TN", "NT", "TT"])
@pytest.mark.parametrize("config", PAIR_CONFIGS)
def test_pair_configuration_transposed_operands(ctx, ops, config):
    M, N, K = 700, 600, 500
    rng = np.random.default_rng(3)
    A = rng.uniform(-1, 1, (K, M) if ops[0] == Op.T else (M, K)).astype(np.float32)
    B = rng.uniform(-1, 1, (N, K) if ops[1] == Op.T else (K, N)).astype(np.float32)
    C = rng.uniform(-1, 1, (M, N)).astype(np.float32)
    got = run_pair(ctx, Precision.BF16X3, A, B, C, 2.0, 0.25, op_a=ops[0], op_b=ops[1], config=config)
    ref = oracle.gemm_f64(A, B, C, 2.0, 0.25, op_a=int(ops[0]), op_b=int(ops[1]))
    assert oracle.error_norms(got, ref)[1] < BOUND[Precision.BF16X3]


def test_pair_configuration_polybench_gemm_verifies(ctx):
    n = 1024
    A, B, C = oracle.init_gemm(n)
    got = run_pair(ctx, Precision.BF16X3, A, B, C, 32412.0, 2123.0)
    first, max_pd, nfail = oracle.verify(oracle.host_gemm(n), got)
    assert first == -1, f"{nfail} elements over 0.05%, max {max_pd}"


@pytest.mark.parametrize("config", PAIR_CONFIGS)
@pytest.mark.parametrize("prec", [Precision.BF16X3, Precision.BF16X6], ids=lambda p: p.name.lower())
def test_pair_configuration_symmetric_updates(ctx, prec, config):
    # syrk and syr2k on 256 x 256 pair tiles: lower triangle of tiles, the
    # tiles below the diagonal also store their transpose (beta on a
    # non-symmetric C, so a wrong mirror shows)
    n, k = 1000, 300
    rng = np.random.default_rng(config)
    A = rng.uniform(-1, 1, (n, k)).astype(np.float32)
    B = rng.uniform(-1, 1, (n, k)).astype(np.float32)
    C = rng.uniform(-1, 1, (n, n)).astype(np.float32)
    dA, dB = ctx.upload(A), ctx.upload(B)
    ctx.config_set(prec, n, n, k, config)
    for name in ("syrk", "syr2k"):
        dC = ctx.upload(C)
        if name == "syrk":
            ctx.syrk(prec, n, k, 1.5, dA, k, -0.5, dC, n)
            ref = oracle.gemm_f64(A, A, C, 1.5, -0.5, op_b=1)
        else:
            ctx.syr2k(prec, n, k, 1.5, dA, k, dB, k, -0.5, dC, n)
            ref = oracle.gemm_f64(A, B, C, 1.5, -0.5, op_b=1, A2=B, B2=A)
        ctx.synchronize()
        assert oracle.error_norms(ctx.download(dC, C.shape), ref)[1] < BOUND[prec], name
        ctx.free(dC)
    ctx.config_set(prec, n, n, k, 0)
    ctx.free(dA)
    ctx.free(dB)



def run_split_and_whole(ctx, fn):
    """fn() twice with the K-split tail enabled, once without: (split, split again, whole)."""
    out = [fn(), fn()]
    ctx.tail_split(False)
    try:
        out.append(fn())
    finally:
        ctx.tail_split(True)
    return out


@pytest.mark.parametrize("M,N,K", [(520, 300, 333), (1024, 768, 1024), (2560, 2560, 256)])
@pytest.mark.parametrize("prec", FORMS, ids=lambda p: p.name.lower())
@pytest.mark.parametrize("config", PAIR_CONFIGS)
def test_tail_split_against_fp64_and_deterministic(ctx, prec, M, N, K, config):
    # 6 and 12 tiles (every tile split in two K halves on two CTA pairs; a
    # ragged edge) and 100 tiles (only the last round's tiles split): within
    # the form's bound, the same bits on every run, and close to the result
    # of whole tiles (only the order of two partial sums differs)
    rng = np.random.default_rng(M + N + K + config)
    A = rng.standard_normal((M, K)).astype(np.float32)
    B = rng.standard_normal((K, N)).astype(np.float32)
    C = rng.standard_normal((M, N)).astype(np.float32)
    split, again, whole = run_split_and_whole(ctx, lambda: run_pair(ctx, prec, A, B, C, 1.25, -0.5, config=config))
    np.testing.assert_array_equal(split.view(np.uint32), again.view(np.uint32))
    ref = oracle.gemm_f64(A, B, C, 1.25, -0.5)
    assert oracle.error_norms(split, ref)[1] < BOUND[prec]
    assert oracle.error_norms(whole, ref)[1] < BOUND[prec]
    assert np.linalg.norm(split - whole) / np.linalg.norm(whole) < 1e-6


@pytest.mark.parametrize("config", PAIR_CONFIGS)
def test_tail_split_symmetric_updates(ctx, config):
    # lower triangle of 4 x 4 pair tiles (10 tiles, all K-split): the first
    # half of a tile below the diagonal also writes its mirror
    n, k = 1000, 300
    rng = np.random.default_rng(11)
    A = rng.uniform(-1, 1, (n, k)).astype(np.float32)
    B = rng.uniform(-1, 1, (n, k)).astype(np.float32)
    C = rng.uniform(-1, 1, (n, n)).astype(np.float32)
    dA, dB = ctx.upload(A), ctx.upload(B)
    ctx.config_set(Precision.BF16X3, n, n, k, config)

    def run(name):
        dC = ctx.upload(C)
        if name == "syrk":
            ctx.syrk(Precision.BF16X3, n, k, 1.5, dA, k, -0.5, dC, n)
        else:
            ctx.syr2k(Precision.BF16X3, n, k, 1.5, dA, k, dB, k, -0.5, dC, n)
        ctx.synchronize()
        out = ctx.download(dC, C.shape)
        ctx.free(dC)
        return out

    refs = {"syrk": oracle.gemm_f64(A, A, C, 1.5, -0.5, op_b=1),
            "syr2k": oracle.gemm_f64(A, B, C, 1.5, -0.5, op_b=1, A2=B, B2=A)}
    for name in ("syrk", "syr2k"):
        split, again, whole = run_split_and_whole(ctx, lambda: run(name))
        np.testing.assert_array_equal(split.view(np.uint32), again.view(np.uint32), err_msg=name)
        assert oracle.error_norms(split, refs[name])[1] < BOUND[Precision.BF16X3], name
        assert np.linalg.norm(split - whole) / np.linalg.norm(whole) < 1e-6, name
    ctx.config_set(Precision.BF16X3, n, n, k, 0)
    ctx.free(dA)
    ctx.free(dB)


@pytest.mark.parametrize("M,N,K", [(256, 256, 64), (300, 520, 70), (1024, 768, 32), (1000, 1000, 512)])
@pytest.mark.parametrize("prec", FORMS, ids=lambda p: p.name.lower())
@pytest.mark.parametrize("beta", [0.0, -0.5])
def test_c_tile_epilogue_is_bitwise_the_staged_one(ctx, prec, M, N, K, beta):
    # configuration 5 (C tile in shared memory, TMA loads and stores of C)
    # computes every element as configuration 3 does: alpha acc + beta C,
    # the same chunk sums; ragged edges are clipped by the TMA stores
    rng = np.random.default_rng(M * 3 + N + K)
    A = rng.standard_normal((M, K)).astype(np.float32)
    B = rng.standard_normal((K, N)).astype(np.float32)
    C = rng.standard_normal((M, N)).astype(np.float32)
    ctx.tail_split(False)  # configuration 5 has no K-split tail: compare whole tiles
    try:
        staged = run_pair(ctx, prec, A, B, C, 1.25, beta, config=3)
        tiled = run_pair(ctx, prec, A, B, C, 1.25, beta, config=5)
    finally:
        ctx.tail_split(True)
    np.testing.assert_array_equal(tiled.view(np.uint32), staged.view(np.uint32))
    assert oracle.error_norms(tiled, oracle.gemm_f64(A, B, C, 1.25, beta))[1] < BOUND[prec]


def test_c_tile_epilogue_falls_back_for_unaligned_c_and_symmetric_products(ctx):
    # C rows TMA cannot address (ldc not a multiple of 4 floats) and syrk run
    # the staged epilogue when configuration 5 is set for their shape
    M, N, K = 520, 301, 96
    rng = np.random.default_rng(17)
    A = rng.uniform(-1, 1, (M, K)).astype(np.float32)
    B = rng.uniform(-1, 1, (K, N)).astype(np.float32)
    C = rng.uniform(-1, 1, (M, N)).astype(np.float32)  # ldc = 301
    got = run_pair(ctx, Precision.BF16X3, A, B, C, 1.0, 0.5, config=5)
    assert oracle.error_norms(got, oracle.gemm_f64(A, B, C, 1.0, 0.5))[1] < BOUND[Precision.BF16X3]
    n, k = 1000, 96
    X = rng.uniform(-1, 1, (n, k)).astype(np.float32)
    C2 = rng.uniform(-1, 1, (n, n)).astype(np.float32)
    dX, dC = ctx.upload(X), ctx.upload(C2)
    ctx.config_set(Precision.BF16X3, n, n, k, 5)
    ctx.syrk(Precision.BF16X3, n, k, 1.5, dX, k, -0.5, dC, n)
    ctx.synchronize()
    ctx.config_set(Precision.BF16X3, n, n, k, 0)
    ref = oracle.gemm_f64(X, X, C2, 1.5, -0.5, op_b=1)
    assert oracle.error_norms(ctx.download(dC, C2.shape), ref)[1] < BOUND[Precision.BF16X3]
    ctx.free(dX)
    ctx.free(dC)


def test_default_configuration_by_k(ctx):
    # pair-filling shapes: the C-tile configuration while K is short, the
    # staged one beyond; small grids keep a 128 x 128 configuration
    assert ctx.config_get(Precision.BF16X3, 8192, 8192, 64) == 5
    assert ctx.config_get(Precision.BF16X3, 8192, 8192, 8192) == 3
    assert ctx.config_get(Precision.TF32, 8192, 8192, 512) == 5
    assert ctx.config_get(Precision.BF16X3, 512, 512, 64) not in (3, 4, 5)
    assert ctx.config_get(Precision.FP8, 8192, 8192, 8192) == 1  # 128 x 256 tiles
    assert ctx.config_get(Precision.FP8, 512, 512, 512) == 0


@pytest.mark.parametrize("N,ldc", [(90, 96), (300, 304), (256, 260)])
def test_c_tile_epilogue_leaves_the_padding_of_ldc(ctx, N, ldc):
    # configuration 5 set for the shape: rows that end inside a 16-byte chunk
    # (N not a multiple of 4) take the staged epilogue; the padding columns
    # of C keep their values either way
    M, K = 300, 64
    rng = np.random.default_rng(N + ldc)
    A = rng.uniform(-1, 1, (M, K)).astype(np.float32)
    B = rng.uniform(-1, 1, (K, N)).astype(np.float32)
    Cp = rng.uniform(-1, 1, (M, ldc)).astype(np.float32)
    dA, dB, dC = ctx.upload(A), ctx.upload(B), ctx.upload(Cp)
    ctx.config_set(Precision.BF16X3, M, N, K, 5)
    ctx.gemm(Precision.BF16X3, M, N, K, 1.0, dA, K, dB, N, 0.5, dC, ldc)
    ctx.synchronize()
    ctx.config_set(Precision.BF16X3, M, N, K, 0)
    out = ctx.download(dC, Cp.shape)
    np.testing.assert_array_equal(out[:, N:], Cp[:, N:])
    ref = oracle.gemm_f64(A, B, np.ascontiguousarray(Cp[:, :N]), 1.0, 0.5)
    assert oracle.error_norms(np.ascontiguousarray(out[:, :N]), ref)[1] < BOUND[Precision.BF16X3]
    for b in (dA, dB, dC):
        ctx.free(b)
