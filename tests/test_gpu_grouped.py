"""Grouped contractions (one split pass + one persistent tensor-core launch
over all problems) against the FP64 oracle, problem by problem.

Workload shape of the grouped benchmark: M, N, K log-uniform, entries
uniform[-1, 1] times a per-matrix scale log-uniform in [1e-3, 1e3],
C = A.B + 0.5 C; here with smaller sizes so the oracle finishes quickly,
plus degenerate problems (K = 0, 1 x 1, transposed operands)."""
import numpy as np
import pytest

import gbpoly
import oracle
from gbpoly import Op, Precision

pytestmark = pytest.mark.gpu

BOUND = {Precision.FP32: 2e-5, Precision.TF32: 2e-3, Precision.BF16X3: 3e-5, Precision.TF32X3: 5e-6,
         Precision.BF16X6: 5e-6, Precision.FP16X3: 5e-6}


def make_problems(rng, count, lo, hi):
    probs = []
    for i in range(count):
        M, N, K = (int(np.exp(rng.uniform(np.log(lo), np.log(hi)))) for _ in range(3))
        op_a = Op.T if i % 5 == 3 else Op.N
        op_b = Op.T if i % 3 == 1 else Op.N
        scale = float(np.exp(rng.uniform(np.log(1e-3), np.log(1e3))))
        A = (rng.uniform(-1, 1, (K, M) if op_a == Op.T else (M, K)) * scale).astype(np.float32)
        B = rng.uniform(-1, 1, (N, K) if op_b == Op.T else (K, N)).astype(np.float32)
        C = rng.uniform(-1, 1, (M, N)).astype(np.float32)
        probs.append((op_a, op_b, M, N, K, A, B, C))
    probs.append((Op.N, Op.N, 70, 90, 0, np.zeros((70, 0), np.float32), np.zeros((0, 90), np.float32),
                  rng.uniform(-1, 1, (70, 90)).astype(np.float32)))  # K = 0: C = 0.5 C
    probs.append((Op.N, Op.N, 1, 1, 1, np.full((1, 1), 3, np.float32), np.full((1, 1), 5, np.float32),
                  np.ones((1, 1), np.float32)))
    return probs


def run_group(ctx, prec, probs):
    items, bufs = [], []
    for op_a, op_b, M, N, K, A, B, C in probs:
        dA = ctx.upload(A) if A.size else ctx.alloc(16)
        dB = ctx.upload(B) if B.size else ctx.alloc(16)
        dC = ctx.upload(C)
        bufs.append((dA, dB, dC))
        items.append(dict(op_a=op_a, op_b=op_b, M=M, N=N, K=K, alpha=1.0, beta=0.5, A=dA, lda=max(A.shape[1], 1),
                          B=dB, ldb=max(B.shape[1], 1), C=dC, ldc=N))
    descs = ctx.descs(items)
    plan = ctx.grouped_plan(prec, descs)
    return plan, bufs


@pytest.mark.parametrize("prec", list(BOUND))
def test_grouped_matches_fp64_per_problem(ctx, prec):
    rng = np.random.default_rng(21)
    probs = make_problems(rng, 40, 16, 700)
    plan, bufs = run_group(ctx, prec, probs)
    info = ctx.grouped_info(plan)
    assert info["flops"] == sum(2 * p[2] * p[3] * p[4] for p in probs)
    ctx.grouped_run(plan)
    ctx.synchronize()
    for (op_a, op_b, M, N, K, A, B, C), (_, _, dC) in zip(probs, bufs):
        out = ctx.download(dC, (M, N))
        if K == 0:
            np.testing.assert_allclose(out, 0.5 * C, rtol=1e-7)
            continue
        ref = oracle.gemm_f64(A, B, C, 1.0, 0.5, op_a=int(op_a), op_b=int(op_b))
        frob = oracle.error_norms(out, ref)[1]
        assert frob < BOUND[prec], (prec.name, M, N, K, frob)
    ctx.grouped_destroy(plan)
    for b in bufs:
        for x in b:
            ctx.free(x)


def test_grouped_run_in_a_graph(ctx):
    rng = np.random.default_rng(5)
    probs = make_problems(rng, 12, 64, 400)
    plan, bufs = run_group(ctx, Precision.BF16X3, probs)
    ctx.grouped_run(plan)
    ctx.synchronize()
    eager = [ctx.download(b[2], (p[2], p[3])) for p, b in zip(probs, bufs)]
    ctx.graph_begin()
    try:
        ctx.grouped_run(plan)
    finally:
        g = ctx.graph_end()  # a failed call must not leave the stream capturing
    for p, b in zip(probs, bufs):
        ctx.h2d(b[2], p[7])  # restore C (beta = 0.5 reads it)
    ctx.graph_launch(g)
    ctx.synchronize()
    for e, p, b in zip(eager, probs, bufs):
        np.testing.assert_array_equal(ctx.download(b[2], (p[2], p[3])), e)
    ctx.graph_destroy(g)
    ctx.grouped_destroy(plan)


@pytest.mark.parametrize("prec", [Precision.FP32, Precision.BF16X3, Precision.TF32X3, Precision.TF32])
def test_grouped_empty_group(ctx, prec):
    # an empty group plans without device memory and runs as nothing
    plan = ctx.grouped_plan(prec, ctx.descs([]))
    assert ctx.grouped_info(plan) == {"flops": 0, "tiles": 0, "device_bytes": 0}
    ctx.grouped_run(plan)
    ctx.synchronize()
    ctx.grouped_destroy(plan)
    with pytest.raises(gbpoly.GbpolyError) as e:  # fp8 has no grouped form, empty or not
        ctx.grouped_plan(Precision.FP8, ctx.descs([]))
    assert e.value.status == gbpoly.Status.UNSUPPORTED


def test_grouped_rejects_bad_descriptor(ctx):
    d = ctx.alloc(64)
    descs = ctx.descs([dict(M=4, N=4, K=4, alpha=1.0, beta=0.0, A=d, lda=2, B=d, ldb=4, C=d, ldc=4)])
    with pytest.raises(gbpoly.GbpolyError) as e:
        ctx.grouped_plan(Precision.BF16X3, descs)
    assert e.value.status == gbpoly.Status.INVALID and b"problem 0" in ctx.lib.gbpoly_last_error()


@pytest.mark.parametrize("prec", [Precision.BF16X3, Precision.TF32X3])
def test_grouped_large_problems_run_on_cta_pairs(ctx, prec):
    # a few large products (256 x 256 tiles pad them no more than 128 x 128
    # ones, and they fill two rounds of pairs) run on CTA-pair tiles: each
    # result is bitwise the single-call result of the pair configuration
    rng = np.random.default_rng(31)
    probs = []
    for i, (M, N, K) in enumerate([(2048, 2048, 512), (2048, 1792, 384), (1536, 2048, 640)]):
        op_b = Op.T if i == 1 else Op.N
        A = rng.uniform(-1, 1, (M, K)).astype(np.float32)
        B = rng.uniform(-1, 1, (N, K) if op_b == Op.T else (K, N)).astype(np.float32)
        C = rng.uniform(-1, 1, (M, N)).astype(np.float32)
        probs.append((Op.N, op_b, M, N, K, A, B, C))
    plan, bufs = run_group(ctx, prec, probs)
    ctx.grouped_run(plan)
    ctx.synchronize()
    for (op_a, op_b, M, N, K, A, B, C), (_, _, dC) in zip(probs, bufs):
        got = ctx.download(dC, (M, N))
        dA, dB, dS = ctx.upload(A), ctx.upload(B), ctx.upload(C)
        ctx.config_set(prec, M, N, K, 3)
        ctx.tail_split(False)
        ctx.gemm(prec, M, N, K, 1.0, dA, K, dB, B.shape[1], 0.5, dS, N, op_a=op_a, op_b=op_b)
        ctx.synchronize()
        ctx.tail_split(True)
        ctx.config_set(prec, M, N, K, 0)
        single = ctx.download(dS, (M, N))
        np.testing.assert_array_equal(got.view(np.uint32), single.view(np.uint32))
        for b in (dA, dB, dS):
            ctx.free(b)
    ctx.grouped_destroy(plan)
    for b in bufs:
        for x in b:
            ctx.free(x)


# fp16x3 grouped tile configuration -> the single-call configuration with the same tiles
FP16X3_SINGLE_OF_GROUPED = {0: 1, 1: 2, 2: 0}


@pytest.mark.parametrize("cfg", [0, 1, 2])
def test_grouped_fp16x3_is_bitwise_the_single_calls(ctx, cfg):
    # the grouped split pass writes the same FP16 terms and block scales as a
    # single call's, and the tiles sum the same chunks in the same order
    rng = np.random.default_rng(41 + cfg)
    prec = Precision.FP16X3
    probs = []
    for i, (M, N, K) in enumerate([(700, 520, 333), (256, 384, 64), (130, 1000, 450), (1024, 512, 700)]):
        op_a = Op.T if i == 2 else Op.N
        op_b = Op.T if i == 1 else Op.N
        A = (rng.uniform(-1, 1, (K, M) if op_a == Op.T else (M, K)) * 10.0 ** (i - 2)).astype(np.float32)
        B = rng.uniform(-1, 1, (N, K) if op_b == Op.T else (K, N)).astype(np.float32)
        C = rng.uniform(-1, 1, (M, N)).astype(np.float32)
        probs.append((op_a, op_b, M, N, K, A, B, C))
    descs, bufs = group_descs(ctx, probs)
    ctx.grouped_config_set(prec, descs, cfg)
    plan = ctx.grouped_plan(prec, descs)
    assert ctx.grouped_config_of(plan) == cfg
    ctx.grouped_run(plan)
    ctx.synchronize()
    ctx.tail_split(False)
    try:
        for (op_a, op_b, M, N, K, A, B, C), (_, _, dC) in zip(probs, bufs):
            got = ctx.download(dC, (M, N))
            dA, dB, dS = ctx.upload(A), ctx.upload(B), ctx.upload(C)
            ctx.config_set(prec, M, N, K, FP16X3_SINGLE_OF_GROUPED[cfg])
            ctx.gemm(prec, M, N, K, 1.0, dA, A.shape[1], dB, B.shape[1], 0.5, dS, N, op_a=op_a, op_b=op_b)
            ctx.synchronize()
            ctx.config_set(prec, M, N, K, 0)
            np.testing.assert_array_equal(got.view(np.uint32), ctx.download(dS, (M, N)).view(np.uint32))
            for b in (dA, dB, dS):
                ctx.free(b)
    finally:
        ctx.tail_split(True)
    ctx.grouped_destroy(plan)
    for b in bufs:
        for x in b:
            ctx.free(x)


def group_descs(ctx, probs):
    items, bufs = [], []
    for op_a, op_b, M, N, K, A, B, C in probs:
        dA = ctx.upload(A) if A.size else ctx.alloc(16)
        dB = ctx.upload(B) if B.size else ctx.alloc(16)
        dC = ctx.upload(C)
        bufs.append((dA, dB, dC))
        items.append(dict(op_a=op_a, op_b=op_b, M=M, N=N, K=K, alpha=1.0, beta=0.5, A=dA, lda=max(A.shape[1], 1),
                          B=dB, ldb=max(B.shape[1], 1), C=dC, ldc=N))
    return ctx.descs(items), bufs


@pytest.mark.parametrize("prec", list(BOUND))
def test_every_grouped_configuration_is_correct(ctx, prec):
    """Each grouped tile configuration (forced per problem class) matches FP64 per problem."""
    rng = np.random.default_rng(33)
    probs = make_problems(rng, 20, 40, 600)
    descs, bufs = group_descs(ctx, probs)
    for cfg in range(ctx.grouped_config_count(prec)):
        ctx.grouped_config_set(prec, descs, cfg)
        assert ctx.grouped_config_get(prec, descs) == cfg
        for (_, _, _, _, _, _, _, C), (_, _, dC) in zip(probs, bufs):
            ctx.h2d(dC, C)
        plan = ctx.grouped_plan(prec, descs)
        assert ctx.grouped_config_of(plan) == cfg
        ctx.grouped_run(plan)
        ctx.synchronize()
        for (op_a, op_b, M, N, K, A, B, C), (_, _, dC) in zip(probs, bufs):
            out = ctx.download(dC, (M, N))
            ref = oracle.gemm_f64(A, B, C, 1.0, 0.5, op_a=int(op_a), op_b=int(op_b)) if K else 0.5 * C.astype(
                np.float64)
            assert oracle.error_norms(out, ref)[1] < BOUND[prec], (cfg, M, N, K)
        ctx.grouped_destroy(plan)
    for b in bufs:
        for x in b:
            ctx.free(x)


def test_grouped_autotune_records_and_persists(ctx, tmp_path):
    """The grouped autotuner times every configuration on the group, keeps the
    fastest for the group's class (the next plan of that class uses it), and
    the entry survives save / load into a new context."""
    import gbpoly
    prec = Precision.BF16X3
    rng = np.random.default_rng(34)
    probs = make_problems(rng, 24, 64, 900)
    descs, bufs = group_descs(ctx, probs)
    best, ms = ctx.autotune_grouped(prec, descs, reps=2)
    assert 0 <= best < ctx.grouped_config_count(prec) and ms > 0
    assert ctx.grouped_config_get(prec, descs) == best
    plan = ctx.grouped_plan(prec, descs)
    assert ctx.grouped_config_of(plan) == best
    ctx.grouped_destroy(plan)
    other = (best + 1) % ctx.grouped_config_count(prec)
    ctx.grouped_config_set(prec, descs, other)
    path = tmp_path / "tuned.txt"
    ctx.autotune_save(path)
    assert "\tG\t" in path.read_text()
    with gbpoly.Context(0) as fresh:
        assert fresh.autotune_load(path) >= 1
        assert fresh.grouped_config_get(prec, descs) == other
    for b in bufs:
        for x in b:
            ctx.free(x)
