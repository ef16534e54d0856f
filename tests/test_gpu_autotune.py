"""Every compiled tile configuration of every tensor-core form is correct
(forced through gbpoly_gemm_config_set), and the autotuner picks, records,
saves and restores a configuration per shape bucket."""
import numpy as np
import pytest

import oracle
from gbpoly import Op, Precision

pytestmark = pytest.mark.gpu

FORMS = [Precision.TF32, Precision.BF16X3, Precision.TF32X3, Precision.BF16X6, Precision.FP16X3]
BOUND = {Precision.TF32: 1e-3, Precision.BF16X3: 2e-5, Precision.TF32X3: 5e-6, Precision.BF16X6: 5e-6,
         Precision.FP16X3: 5e-6}


@pytest.mark.parametrize("prec", FORMS)
@pytest.mark.parametrize("op_b", [Op.N, Op.T])
def test_every_configuration_is_correct(ctx, prec, op_b):
    M, N, K = 300, 520, 333
    rng = np.random.default_rng(7)
    A = rng.standard_normal((M, K)).astype(np.float32)
    B = rng.standard_normal((N, K) if op_b == Op.T else (K, N)).astype(np.float32)
    C = rng.standard_normal((M, N)).astype(np.float32)
    ref = oracle.gemm_f64(A, B, C, 1.25, 0.5, op_b=int(op_b))
    dA, dB = ctx.upload(A), ctx.upload(B)
    for cfg in range(ctx.config_count(prec)):
        ctx.config_set(prec, M, N, K, cfg)
        assert ctx.config_get(prec, M, N, K) == cfg
        dC = ctx.upload(C)
        ctx.gemm(prec, M, N, K, 1.25, dA, K, dB, B.shape[1], 0.5, dC, N, op_b=op_b)
        ctx.synchronize()
        frob = oracle.error_norms(ctx.download(dC, C.shape), ref)[1]
        assert frob < BOUND[prec], (cfg, frob)
        ctx.free(dC)
    ctx.config_set(prec, M, N, K, 0)


@pytest.mark.parametrize("prec", [Precision.BF16X3, Precision.BF16X6, Precision.FP16X3])
def test_every_configuration_runs_syr2k(ctx, prec):
    n, k = 264, 200
    rng = np.random.default_rng(8)
    A = rng.standard_normal((n, k)).astype(np.float32)
    B = rng.standard_normal((n, k)).astype(np.float32)
    C = rng.standard_normal((n, n)).astype(np.float32)
    ref = oracle.gemm_f64(A, B, C, 1.0, 1.0, op_b=1, A2=B, B2=A)
    dA, dB = ctx.upload(A), ctx.upload(B)
    for cfg in range(ctx.config_count(prec)):
        ctx.config_set(prec, n, n, k, cfg)
        dC = ctx.upload(C)
        ctx.syr2k(prec, n, k, 1.0, dA, k, dB, k, 1.0, dC, n)
        ctx.synchronize()
        assert oracle.error_norms(ctx.download(dC, C.shape), ref)[1] < BOUND[prec]
        ctx.free(dC)
    ctx.config_set(prec, n, n, k, 0)


def test_autotune_records_and_persists(ctx, tmp_path):
    prec = Precision.BF16X3
    best, ms = ctx.autotune(prec, 1024, 1024, 1024, reps=2)
    assert 0 <= best < ctx.config_count(prec) and ms > 0
    assert ctx.config_get(prec, 1024, 1024, 1024) == best
    assert ctx.config_get(prec, 1000, 1000, 1000) == best  # same log2 bucket
    path = tmp_path / "tune.txt"
    ctx.autotune_save(path)
    other = 2 if best != 2 else 1
    ctx.config_set(prec, 1024, 1024, 1024, other)
    assert ctx.autotune_load(path) >= 1
    assert ctx.config_get(prec, 1024, 1024, 1024) == best
