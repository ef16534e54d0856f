"""Correctness of every arithmetic form at the full workload sizes, through the C ABI.

The other GPU tests stop at N = 1024, where the host loops of the oracle
finish in seconds.  This file runs the contractions at the sizes the
throughput figures are quoted on:

  gemm    N = 4096 and 8192, alpha = 32412, beta = 2123, polybench inputs
          (gemm.cpp:18-40) and seeded uniform[-1, 1] inputs
  2mm     N = 4096, C += A.B then E = C.D (2mm.cpp:94-123), stages of the
          tensor-core forms captured in one CUDA graph
  3mm     N = 4096, E = A.B, F = C.D, G = E.F (3mm.cpp:115-158), E and F as
          one grouped launch and G after it, in one CUDA graph
  syrk    N = 4096 (syrk.cpp:74-83), alpha/beta 123/14512 and 32412/2123
  syr2k   N = 4096 (syr2k.cpp:78-87), alpha/beta 1/1 and 32412/2123
  (2mm, 3mm, syrk, syr2k: polybench inputs and seeded normal(0, 1) inputs)

The oracle at these sizes is an FP64 contraction on the GPU
(gbpoly_gemm_f64; the host loops would take hours), itself checked against
numpy's FP64 product at N = 2048 below.  Every form's result is compared
with it:

  * the reference's verify rule, every element within 0.05 percent
    (polybench/gemm.cpp:95-113 with polybenchUtilFuncts.h:36-42), applied to
    the FP64 result on the polybench inputs, for fp32, bf16x3, tf32x3, bf16x6,
    fp16x3;
  * fp32: normwise (max |C-R| / max |R|) and Frobenius error below 1e-5;
  * tf32x3, bf16x6 and fp16x3: both norms at most 1.5 x plain FP32's on the
    same inputs;
  * bf16x3 and tf32: both norms at most 1.5 x the figure this test measured
    on a GB300 (table MEASURED below), so an accuracy regression of half
    again fails;
  * fp8: reported, bounded only against garbage (Frobenius below 0.1).
"""
import json

import numpy as np
import pytest

import gbpoly
import oracle
from gbpoly import Op, Precision

pytestmark = pytest.mark.gpu

ALL = [Precision.FP32, Precision.BF16X3, Precision.TF32, Precision.TF32X3, Precision.BF16X6, Precision.FP16X3,
       Precision.FP8]
VERIFYING = {Precision.FP32, Precision.BF16X3, Precision.TF32X3, Precision.BF16X6, Precision.FP16X3}
MATCHED = {Precision.TF32X3, Precision.BF16X6, Precision.FP16X3}

# (case, inputs, form) -> (normwise, Frobenius) relative error against FP64 measured
# by this file on a GB300; bf16x3 and tf32 are bounded at 1.5 x these.
MEASURED: dict[tuple[str, str, str], tuple[float, float]] = {
    ('2mm_end_to_end_E', 'normal01', 'bf16x3'): (6.13e-06, 6.28e-06),
    ('2mm_end_to_end_E', 'normal01', 'tf32'): (0.000445, 0.000415),
    ('2mm_end_to_end_E', 'polybench', 'bf16x3'): (2.3e-06, 2.11e-07),
    ('2mm_end_to_end_E', 'polybench', 'tf32'): (0.000179, 7.05e-06),
    ('2mm_stage1_C', 'normal01', 'bf16x3'): (4.43e-06, 4.44e-06),
    ('2mm_stage1_C', 'normal01', 'tf32'): (0.000274, 0.000294),
    ('2mm_stage1_C', 'polybench', 'bf16x3'): (2.95e-06, 2.05e-07),
    ('2mm_stage1_C', 'polybench', 'tf32'): (0.000214, 5.85e-06),
    ('3mm_end_to_end_G', 'normal01', 'bf16x3'): (7.75e-06, 7.69e-06),
    ('3mm_end_to_end_G', 'normal01', 'tf32'): (0.000509, 0.000509),
    ('3mm_end_to_end_G', 'polybench', 'bf16x3'): (3.25e-06, 2.89e-07),
    ('3mm_end_to_end_G', 'polybench', 'tf32'): (0.00016, 7.56e-06),
    ('3mm_stage1_E', 'normal01', 'bf16x3'): (4.41e-06, 4.44e-06),
    ('3mm_stage1_E', 'normal01', 'tf32'): (0.000273, 0.000294),
    ('3mm_stage1_E', 'polybench', 'bf16x3'): (2.95e-06, 2.07e-07),
    ('3mm_stage1_E', 'polybench', 'tf32'): (0.000214, 5.85e-06),
    ('3mm_stage2_F', 'normal01', 'bf16x3'): (4.38e-06, 4.44e-06),
    ('3mm_stage2_F', 'normal01', 'tf32'): (0.000292, 0.000294),
    ('3mm_stage2_F', 'polybench', 'bf16x3'): (2.03e-06, 1.95e-07),
    ('3mm_stage2_F', 'polybench', 'tf32'): (0.000213, 6.51e-06),
    ('gemm4096', 'polybench', 'bf16x3'): (3.07e-06, 2.76e-07),
    ('gemm4096', 'polybench', 'tf32'): (0.000214, 6.54e-06),
    ('gemm4096', 'uniform', 'bf16x3'): (3.62e-06, 3.78e-06),
    ('gemm4096', 'uniform', 'tf32'): (0.000281, 0.000261),
    ('gemm8192', 'polybench', 'bf16x3'): (3.07e-06, 2.21e-07),
    ('gemm8192', 'polybench', 'tf32'): (7.21e-05, 2.78e-06),
    ('gemm8192', 'uniform', 'bf16x3'): (3.84e-06, 3.78e-06),
    ('gemm8192', 'uniform', 'tf32'): (0.000261, 0.000261),
    ('syr2k_ab32412_2123', 'normal01', 'bf16x3'): (5.03e-06, 4.44e-06),
    ('syr2k_ab32412_2123', 'normal01', 'tf32'): (0.000316, 0.000294),
    ('syr2k_ab32412_2123', 'polybench', 'bf16x3'): (2.87e-06, 2.69e-07),
    ('syr2k_ab32412_2123', 'polybench', 'tf32'): (0.000214, 6.21e-06),
    ('syr2k_abreference', 'normal01', 'bf16x3'): (5.03e-06, 4.44e-06),
    ('syr2k_abreference', 'normal01', 'tf32'): (0.000316, 0.000294),
    ('syr2k_abreference', 'polybench', 'bf16x3'): (2.83e-06, 2.69e-07),
    ('syr2k_abreference', 'polybench', 'tf32'): (0.000214, 6.21e-06),
    ('syrk_ab32412_2123', 'normal01', 'bf16x3'): (3.34e-06, 3.73e-06),
    ('syrk_ab32412_2123', 'normal01', 'tf32'): (3.63e-05, 0.000208),
    ('syrk_ab32412_2123', 'polybench', 'bf16x3'): (2.98e-06, 2.11e-07),
    ('syrk_ab32412_2123', 'polybench', 'tf32'): (0.000214, 5.85e-06),
    ('syrk_abreference', 'normal01', 'bf16x3'): (3.22e-06, 2.27e-06),
    ('syrk_abreference', 'normal01', 'tf32'): (3.42e-05, 0.000126),
    ('syrk_abreference', 'polybench', 'bf16x3'): (2.94e-06, 2.1e-07),
    ('syrk_abreference', 'polybench', 'tf32'): (0.000214, 5.85e-06),
}


def _bound_measured(case, inputs, prec, got):
    key = (case, inputs, prec.name.lower())
    mx, fr = MEASURED[key]
    assert got[0] <= 1.5 * mx and got[1] <= 1.5 * fr, (key, got, MEASURED[key])


def check_form(case, inputs, prec, got, fp32):
    """got, fp32: (normwise, Frobenius, max elementwise) of this form and of plain FP32."""
    print("ERRLINE " + json.dumps({"case": case, "inputs": inputs, "form": prec.name.lower(),
                                   "max_rel": got[0], "frob_rel": got[1], "max_elem_rel": got[2]}))
    assert np.isfinite(got[0]) and np.isfinite(got[1]), (case, inputs, prec, got)
    if prec == Precision.FP32:
        assert got[0] < 1e-5 and got[1] < 1e-5, (case, inputs, got)
    elif prec in MATCHED:
        assert got[0] <= 1.5 * fp32[0] and got[1] <= 1.5 * fp32[1], (case, inputs, prec.name, got, fp32)
    elif prec == Precision.FP8:
        assert got[1] < 0.1, (case, inputs, got)
    else:
        _bound_measured(case, inputs, prec, got)


class Ref64:
    """FP64 copies of device operands and FP64 contractions of them (the oracle at these sizes)."""

    def __init__(self, ctx, n):
        self.ctx, self.n = ctx, n
        self.bufs = []

    def alloc(self):
        b = self.ctx.alloc(self.n * self.n * 8)
        self.bufs.append(b)
        return b

    def of(self, d32):
        b = self.alloc()
        self.ctx.convert_f32_f64(d32, b, self.n * self.n)
        return b

    def gemm(self, a, b, c, alpha, beta, op_b=Op.N):
        n = self.n
        self.ctx.gemm_f64(n, n, n, alpha, a, n, b, n, beta, c, n, op_b=op_b)

    def free(self):
        for b in self.bufs:
            self.ctx.free(b)
        self.bufs.clear()


def errors(ctx, d32, r64, n):
    return ctx.error_norms(d32, n, r64, n, n, n)


def assert_reference_verify(ctx, d32, r64, n, what):
    """Every element within 0.05 percent of the FP64 result (the reference's rule)."""
    dev = ctx.download(d32, (n, n))
    ref = ctx.download(r64, (n, n), np.float64).astype(np.float32)
    first, max_pd, nfail = oracle.verify(ref, dev)
    assert first == -1, f"{what}: {nfail} elements over 0.05%, first at {first}, max percentDiff {max_pd}"


def copy(ctx, dst, src, nbytes):
    gbpoly._check(ctx.lib.gbpoly_memcpy_d2d(ctx.handle, gbpoly._ptr(dst), gbpoly._ptr(src), nbytes))


def test_gpu_fp64_oracle_matches_numpy(ctx):
    """The FP64 contraction used as the oracle here agrees with numpy's FP64
    product (both operand orders the tests use) to FP64 rounding."""
    n = 2048
    rng = np.random.default_rng(2048)
    A = rng.standard_normal((n, n)).astype(np.float32)
    B = rng.standard_normal((n, n)).astype(np.float32)
    C = rng.standard_normal((n, n)).astype(np.float32)
    r = Ref64(ctx, n)
    dA, dB, dC = ctx.upload(A), ctx.upload(B), ctx.upload(C)
    a, b = r.of(dA), r.of(dB)
    A64, B64, C64 = (x.astype(np.float64) for x in (A, B, C))
    for op_b, want in ((Op.N, 3.5 * (A64 @ B64) - 0.5 * C64), (Op.T, 3.5 * (A64 @ B64.T) - 0.5 * C64)):
        c = r.of(dC)
        r.gemm(a, b, c, 3.5, -0.5, op_b=op_b)
        got = ctx.download(c, (n, n), np.float64)
        rel = np.abs(got - want).max() / np.abs(want).max()
        assert rel < 1e-13, (op_b, rel)
    r.free()
    for x in (dA, dB, dC):
        ctx.free(x)


def gemm_inputs(kind, n):
    if kind == "polybench":
        return oracle.init_gemm(n)
    rng = np.random.default_rng(n + 7)
    return tuple(rng.uniform(-1, 1, (n, n)).astype(np.float32) for _ in range(3))


@pytest.mark.parametrize("n", [4096, 8192])
@pytest.mark.parametrize("inputs", ["polybench", "uniform"])
def test_gemm_every_form_vs_fp64(ctx, n, inputs):
    alpha, beta = 32412.0, 2123.0
    A, B, C = gemm_inputs(inputs, n)
    nb = n * n * 4
    dA, dB, dC0 = ctx.upload(A), ctx.upload(B), ctx.upload(C)
    del A, B, C
    dC = ctx.alloc(nb)
    r = Ref64(ctx, n)
    R = r.of(dC0)
    r.gemm(r.of(dA), r.of(dB), R, alpha, beta)
    ctx.synchronize()
    fp32 = None
    for prec in ALL:
        copy(ctx, dC, dC0, nb)
        ctx.gemm(prec, n, n, n, alpha, dA, n, dB, n, beta, dC, n)
        ctx.synchronize()
        got = errors(ctx, dC, R, n)
        if prec == Precision.FP32:
            fp32 = got
        check_form(f"gemm{n}", inputs, prec, got, fp32)
        if inputs == "polybench" and prec in VERIFYING:
            assert_reference_verify(ctx, dC, R, n, f"gemm {n} {prec.name}")
    r.free()
    for x in (dA, dB, dC0, dC):
        ctx.free(x)


def family_inputs(kind, n, count):
    if kind == "polybench":
        return oracle.init_mm2(n)[:count]
    rng = np.random.default_rng(4096 + count)
    return tuple(rng.standard_normal((n, n)).astype(np.float32) for _ in range(count))


def run_captured(ctx, prec, n, stages):
    """Eager for fp32 and fp8; one CUDA graph of all stages for the split forms."""
    if prec in (Precision.FP32, Precision.FP8):
        stages()
        ctx.synchronize()
        return
    ctx.workspace_reserve(ctx.workspace_query(prec, n, n, n))
    ctx.graph_begin()
    try:
        stages()
    finally:
        g = ctx.graph_end()  # a failed call must not leave the stream capturing
    ctx.graph_launch(g)
    ctx.synchronize()
    ctx.graph_destroy(g)


@pytest.mark.parametrize("inputs", ["polybench", "normal01"])
def test_2mm_every_form_vs_fp64(ctx, inputs):
    n = 4096
    nb = n * n * 4
    A, B, C, D = family_inputs(inputs, n, 4)
    dA, dB, dC0, dD = (ctx.upload(x) for x in (A, B, C, D))
    del A, B, C, D
    dC, dE = ctx.alloc(nb), ctx.alloc(nb)
    r = Ref64(ctx, n)
    C64 = r.of(dC0)
    r.gemm(r.of(dA), r.of(dB), C64, 1.0, 1.0)           # stage 1 in FP64
    E64 = r.alloc()
    r.gemm(C64, r.of(dD), E64, 1.0, 0.0)                # stage 2 in FP64
    fp32 = {}
    for prec in ALL:
        def stages(prec=prec):
            ctx.gemm(prec, n, n, n, 1.0, dA, n, dB, n, 1.0, dC, n)
            ctx.gemm(prec, n, n, n, 1.0, dC, n, dD, n, 0.0, dE, n)
        copy(ctx, dC, dC0, nb)
        run_captured(ctx, prec, n, stages)
        for stage, d, R in (("stage1_C", dC, C64), ("end_to_end_E", dE, E64)):
            got = errors(ctx, d, R, n)
            if prec == Precision.FP32:
                fp32[stage] = got
            check_form(f"2mm_{stage}", inputs, prec, got, fp32[stage])
        if inputs == "polybench" and prec in VERIFYING:
            assert_reference_verify(ctx, dE, E64, n, f"2mm {prec.name}")
    r.free()
    for x in (dA, dB, dC0, dD, dC, dE):
        ctx.free(x)


@pytest.mark.parametrize("inputs", ["polybench", "normal01"])
def test_3mm_every_form_vs_fp64(ctx, inputs):
    n = 4096
    nb = n * n * 4
    A, B, C, D = family_inputs(inputs, n, 4)
    dA, dB, dC, dD = (ctx.upload(x) for x in (A, B, C, D))
    del A, B, C, D
    dE, dF, dG = ctx.alloc(nb), ctx.alloc(nb), ctx.alloc(nb)
    r = Ref64(ctx, n)
    E64, F64, G64 = r.alloc(), r.alloc(), r.alloc()
    r.gemm(r.of(dA), r.of(dB), E64, 1.0, 0.0)
    r.gemm(r.of(dC), r.of(dD), F64, 1.0, 0.0)
    r.gemm(E64, F64, G64, 1.0, 0.0)
    fp32 = {}
    for prec in ALL:
        plan = None
        if prec not in (Precision.FP32, Precision.FP8):
            plan = ctx.grouped_plan(prec, ctx.descs([
                {"M": n, "N": n, "K": n, "alpha": 1.0, "beta": 0.0, "A": dA, "lda": n, "B": dB, "ldb": n, "C": dE,
                 "ldc": n},
                {"M": n, "N": n, "K": n, "alpha": 1.0, "beta": 0.0, "A": dC, "lda": n, "B": dD, "ldb": n, "C": dF,
                 "ldc": n}]))

        def stages(prec=prec, plan=plan):
            if plan is None:
                ctx.gemm(prec, n, n, n, 1.0, dA, n, dB, n, 0.0, dE, n)
                ctx.gemm(prec, n, n, n, 1.0, dC, n, dD, n, 0.0, dF, n)
            else:
                ctx.grouped_run(plan)
            ctx.gemm(prec, n, n, n, 1.0, dE, n, dF, n, 0.0, dG, n)
        run_captured(ctx, prec, n, stages)
        if plan is not None:
            ctx.grouped_destroy(plan)
        for stage, d, R in (("stage1_E", dE, E64), ("stage2_F", dF, F64), ("end_to_end_G", dG, G64)):
            got = errors(ctx, d, R, n)
            if prec == Precision.FP32:
                fp32[stage] = got
            check_form(f"3mm_{stage}", inputs, prec, got, fp32[stage])
        if inputs == "polybench" and prec in VERIFYING:
            assert_reference_verify(ctx, dG, G64, n, f"3mm {prec.name}")
    r.free()
    for x in (dA, dB, dC, dD, dE, dF, dG):
        ctx.free(x)


@pytest.mark.parametrize("name", ["syrk", "syr2k"])
@pytest.mark.parametrize("inputs", ["polybench", "normal01"])
@pytest.mark.parametrize("alpha_beta", ["reference", "32412_2123"])
def test_symmetric_every_form_vs_fp64(ctx, name, inputs, alpha_beta):
    n = 4096
    nb = n * n * 4
    if alpha_beta == "reference":
        alpha, beta = (123.0, 14512.0) if name == "syrk" else (1.0, 1.0)
    else:
        alpha, beta = 32412.0, 2123.0
    if inputs == "polybench":
        A, B, C = oracle.init_syr2k(n)  # A = ij/N, C = (ij+2)/N: syrk.cpp:18-31's A and C too
    else:
        rng = np.random.default_rng(4099)
        A, B, C = (rng.standard_normal((n, n)).astype(np.float32) for _ in range(3))
    dA, dB, dC0 = ctx.upload(A), ctx.upload(B), ctx.upload(C)
    del A, B, C
    dC = ctx.alloc(nb)
    r = Ref64(ctx, n)
    a64, b64 = r.of(dA), r.of(dB)
    R = r.of(dC0)
    if name == "syrk":
        r.gemm(a64, a64, R, alpha, beta, op_b=Op.T)
    else:
        r.gemm(a64, b64, R, alpha, beta, op_b=Op.T)
        r.gemm(b64, a64, R, alpha, 1.0, op_b=Op.T)
    fp32 = None
    for prec in ALL:
        copy(ctx, dC, dC0, nb)
        if name == "syrk":
            ctx.syrk(prec, n, n, alpha, dA, n, beta, dC, n)
        else:
            ctx.syr2k(prec, n, n, alpha, dA, n, dB, n, beta, dC, n)
        ctx.synchronize()
        got = errors(ctx, dC, R, n)
        if prec == Precision.FP32:
            fp32 = got
        check_form(f"{name}_ab{alpha_beta}", inputs, prec, got, fp32)
        if inputs == "polybench" and prec in VERIFYING:
            assert_reference_verify(ctx, dC, R, n, f"{name} {prec.name}")
    r.free()
    for x in (dA, dB, dC0, dC):
        ctx.free(x)
