"""The split-FP16 form (fp16x3), through the C ABI: what its block scales add.

FP16 keeps 11 significand bits but only the exponents -14..15; the split
pass scales every 64 x 64 operand block by a power of two 2^e chosen from the
block's largest finite magnitude (so that it lands in [2^14, 2^15)) before
it writes hi = fp16(x 2^e) and lo = fp16(x 2^e - hi), and the epilogue
multiplies each chunk of the product by 2^-(ea + eb).  So:

  * scaling an operand by a power of two scales the result by the same power,
    bit for bit (the same FP16 terms, the same sums), for every tile
    configuration, across magnitudes far outside FP16's range;
  * operands whose 64 x 64 blocks span 2^-40 .. 2^40 give every element of
    the product within a componentwise bound of 2^-18 (|alpha| |A||B| +
    |beta| |C|) against FP64 (plain FP32 arithmetic stays within it too);
  * an infinity or NaN is left out of its block's scale: the other rows of
    its 64-row block give the bits they give without it;
  * K = 0 leaves beta C.
"""
import numpy as np
import pytest

import oracle
from gbpoly import Op, Precision

pytestmark = pytest.mark.gpu

P = Precision.FP16X3


def run(ctx, A, B, C, alpha, beta, op_b=Op.N, config=None, prec=P):
    M, K = A.shape
    N = B.shape[0] if op_b == Op.T else B.shape[1]
    if config is not None:
        ctx.config_set(prec, M, N, K, config)
    dA, dB, dC = ctx.upload(A), ctx.upload(B), ctx.upload(C)
    ctx.gemm(prec, M, N, K, alpha, dA, max(K, 1), dB, B.shape[1], beta, dC, N, op_b=op_b)
    ctx.synchronize()
    out = ctx.download(dC, C.shape)
    for b in (dA, dB, dC):
        ctx.free(b)
    if config is not None:
        ctx.config_set(prec, M, N, K, 0)
    return out


def block_magnitudes(rng, rows, cols, lo_exp, hi_exp, block=64):
    x = rng.uniform(-1, 1, (rows, cols))
    for r in range(0, rows, block):
        for c in range(0, cols, block):
            x[r:r + block, c:c + block] *= 2.0 ** int(rng.integers(lo_exp, hi_exp + 1))
    return x.astype(np.float32)


@pytest.mark.parametrize("config", [0, 1, 2])
@pytest.mark.parametrize("op_b", [Op.N, Op.T])
def test_power_of_two_scaling_is_exact(ctx, config, op_b):
    M, N, K = 300, 520, 333
    rng = np.random.default_rng(21)
    A = rng.standard_normal((M, K)).astype(np.float32)
    B = rng.standard_normal((N, K) if op_b == Op.T else (K, N)).astype(np.float32)
    C = np.zeros((M, N), np.float32)
    base = run(ctx, A, B, C, 1.0, 0.0, op_b=op_b, config=config)
    for ea, eb in ((37, -29), (-60, -40), (50, 20)):
        got = run(ctx, A * np.float32(2.0 ** ea), B * np.float32(2.0 ** eb), C, 1.0, 0.0, op_b=op_b, config=config)
        want = base * np.float32(2.0 ** (ea + eb))
        np.testing.assert_array_equal(got.view(np.uint32), want.view(np.uint32), err_msg=f"2^{ea} x 2^{eb}")


@pytest.mark.parametrize("config", [0, 1, 2])
@pytest.mark.parametrize("mnk", [(256, 384, 512), (200, 130, 300), (520, 300, 333)])
def test_block_magnitudes_far_outside_fp16_range(ctx, config, mnk):
    M, N, K = mnk
    rng = np.random.default_rng(M + 3 * N + 7 * K)
    A = block_magnitudes(rng, M, K, -40, 40)
    B = block_magnitudes(rng, K, N, -40, 40)
    C = rng.uniform(-1, 1, (M, N)).astype(np.float32)
    alpha, beta = 1.5, 0.25
    got = run(ctx, A, B, C, alpha, beta, config=config).astype(np.float64)
    ref = oracle.gemm_f64(A, B, C, alpha, beta)
    bound = 2.0 ** -18 * (abs(alpha) * (np.abs(A.astype(np.float64)) @ np.abs(B.astype(np.float64)))
                          + abs(beta) * np.abs(C.astype(np.float64)))
    excess = np.abs(got - ref) / np.maximum(bound, 1e-300)
    assert np.isfinite(got).all()
    assert excess.max() <= 1.0, (float(excess.max()), np.unravel_index(int(np.argmax(excess)), excess.shape))
    # plain FP32 meets the same bound on the same data
    f32 = run(ctx, A, B, C, alpha, beta, prec=Precision.FP32).astype(np.float64)
    assert (np.abs(f32 - ref) <= bound).all()


@pytest.mark.parametrize("bad", [np.inf, -np.inf, np.nan])
def test_nonfinite_element_leaves_its_block_scale_alone(ctx, bad):
    M, N, K = 192, 256, 200
    rng = np.random.default_rng(5)
    A = rng.uniform(-1, 1, (M, K)).astype(np.float32) * np.float32(1e6)  # beyond FP16's largest finite value
    B = rng.uniform(-1, 1, (K, N)).astype(np.float32)
    C = rng.uniform(-1, 1, (M, N)).astype(np.float32)
    A[70, 90] = 0.0
    base = run(ctx, A, B, C, 1.0, 1.0)
    A[70, 90] = bad
    got = run(ctx, A, B, C, 1.0, 1.0)
    assert not np.isfinite(got[70]).any()
    rows = np.arange(M) != 70
    np.testing.assert_array_equal(got[rows].view(np.uint32), base[rows].view(np.uint32))
    assert oracle.error_norms(base, oracle.gemm_f64(np.where(np.isfinite(A), A, 0), B, C, 1.0, 1.0))[1] < 5e-6


@pytest.mark.parametrize("config", [0, 1, 2])
def test_k_zero_leaves_beta_c(ctx, config):
    rng = np.random.default_rng(9)
    M, N = 300, 260
    C = rng.standard_normal((M, N)).astype(np.float32)
    dA, dB, dC = ctx.alloc(16), ctx.alloc(16), ctx.upload(C)
    ctx.config_set(P, M, N, 0, config)
    ctx.gemm(P, M, N, 0, 2.0, dA, 1, dB, N, 0.75, dC, N)
    ctx.synchronize()
    ctx.config_set(P, M, N, 0, 0)
    np.testing.assert_array_equal(ctx.download(dC, C.shape), C * np.float32(0.75))
    for b in (dA, dB, dC):
        ctx.free(b)
