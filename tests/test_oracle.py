"""The CPU oracle, pinned against the reference's own outputs (no GPU).

tests/golden/reference_outputs.npz was produced by the reference's unmodified
PolyBench sources (tests/golden/make_golden.py); the oracle must reproduce its
host verification loops and its kernel bodies bit for bit.
"""
from pathlib import Path

import numpy as np
import pytest

import oracle

GOLDEN = np.load(Path(__file__).resolve().parent / "golden" / "reference_outputs.npz")
SIZES = sorted({int(k.split("_")[1]) for k in GOLDEN.files})
HOST = {"gemm": oracle.host_gemm, "2mm": oracle.host_mm2, "3mm": oracle.host_mm3, "syrk": oracle.host_syrk,
        "syr2k": oracle.host_syr2k, "covariance": oracle.host_covariance, "correlation": oracle.host_correlation,
        "atax": oracle.host_atax, "bicg": oracle.host_bicg, "mvt": oracle.host_mvt, "gesummv": oracle.host_gesummv}


def bits(x):
    return np.ascontiguousarray(x, np.float32).view(np.uint32)


@pytest.mark.parametrize("bench", list(HOST))
@pytest.mark.parametrize("n", SIZES)
def test_host_loops_match_reference_bitwise(bench, n):
    np.testing.assert_array_equal(bits(HOST[bench](n)), bits(GOLDEN[f"{bench}_{n}_host"]))


@pytest.mark.parametrize("n", SIZES)
def test_kernel_bodies_match_reference_bitwise(n):
    lib = oracle.lib()
    A, B, C = oracle.init_gemm(n)
    lib.orc_gemm_body(A, B, C, n, 0, n, 32412.0, 2123.0)
    np.testing.assert_array_equal(bits(C), bits(GOLDEN[f"gemm_{n}_device"]))
    A, C = oracle.init_syrk(n)
    lib.orc_syrk_body(A, C, n, 0, n, 123.0, 14512.0)
    np.testing.assert_array_equal(bits(C), bits(GOLDEN[f"syrk_{n}_device"]))
    A, B, C = oracle.init_syr2k(n)
    lib.orc_syr2k_body(A, B, C, n, 0, n, 1.0, 1.0)
    np.testing.assert_array_equal(bits(C), bits(GOLDEN[f"syr2k_{n}_device"]))
    # 2mm: C += A.B then E = C.D, each stage the gemm body with alpha 1
    A, B, C, D = oracle.init_mm2(n)
    E = np.zeros((n, n), np.float32)
    lib.orc_gemm_body(A, B, C, n, 0, n, 1.0, 1.0)
    lib.orc_gemm_body(C, D, E, n, 0, n, 1.0, 0.0)
    np.testing.assert_array_equal(bits(E), bits(GOLDEN[f"2mm_{n}_device"]))


@pytest.mark.parametrize("bench", ["covariance", "correlation"])
@pytest.mark.parametrize("n", SIZES)
def test_statistics_kernels_match_reference_bitwise(bench, n):
    # the run() kernels (mean, [stddev,] reduce, contraction) perform the host
    # loop's per-element operations in the same order: same bits on the
    # (n + 1) x (n + 1) arrays, read from index 1
    got = HOST[bench](n)
    np.testing.assert_array_equal(bits(got[1:, 1:]), bits(GOLDEN[f"{bench}_{n}_device"][1:, 1:]))


@pytest.mark.parametrize("bench", ["atax", "bicg", "mvt", "gesummv"])
@pytest.mark.parametrize("n", SIZES)
def test_matrix_vector_kernels_match_reference_bitwise(bench, n):
    # each run() kernel walks its row or column in the host loop's order
    np.testing.assert_array_equal(bits(HOST[bench](n)), bits(GOLDEN[f"{bench}_{n}_device"]))


def test_correlation_init_keeps_row_stride_of_n():
    n = 5
    d = oracle.init_correlation(n).ravel()
    # flat index i*n + j holds i*j/(n+1); row i's j = n slot is row i+1's j = 0 (zero) except after the last row
    assert d[2 * n + 3] == np.float32(np.float32(2 * 3) / np.float32(n + 1))
    assert d[3 * n] == 0.0 and d[n * n + n] == np.float32(np.float32(n * n) / np.float32(n + 1))
    assert not d[(n + 1) * n + 1:].any()


@pytest.mark.parametrize("n", SIZES)
def test_matmulchain_matches_reference_on_identities(n):
    eye = np.eye(n, dtype=np.float32)
    p = oracle.matmulchain_product(eye, eye)
    q = oracle.matmulchain_product(eye, eye)
    r = oracle.matmulchain_product(p, q)
    np.testing.assert_array_equal(bits(r), bits(GOLDEN[f"matmulchain_{n}_device"]))
    np.testing.assert_array_equal(bits(r), bits(GOLDEN[f"matmulchain_{n}_host"]))


def test_matmulchain_int_accumulator_truncates():
    # matmulchain.cpp:21 accumulates into an int: 0 + 0.75 -> 0, (0 + 0.75) + 0.75 -> 0 ... for halves
    # and quarters, while the true product (a float sum) is 1.5; only identity inputs hide it
    a = np.full((2, 2), 0.75, np.float32)
    b = np.full((2, 2), 1.0, np.float32)
    assert (oracle.matmulchain_product(a, b) == 0.0).all()
    c = np.full((2, 2), 1.5, np.float32)
    assert (oracle.matmulchain_product(c, b) == 2.0).all()   # 0 + 1.5 -> 1, 1 + 1.5 -> 2


def test_kernel_body_row_sample_is_a_prefix():
    n = 37
    A, B, C = oracle.init_gemm(n)
    C2 = C.copy()
    oracle.lib().orc_gemm_body(A, B, C2, n, 0, 5, 32412.0, 2123.0)
    ref = GOLDEN[f"gemm_{n}_device"]
    np.testing.assert_array_equal(bits(C2[:5]), bits(ref[:5]))
    np.testing.assert_array_equal(bits(C2[5:]), bits(C[5:]))


# percentDiff (polybench/common/polybenchUtilFuncts.h:36-42): known answers
@pytest.mark.parametrize("v1,v2,expect", [
    (0.005, 0.009, 0.0),          # both below 0.01: no difference
    (0.005, 0.02, 300.0),         # one above: relative to v1
    (100.0, 0.0, 100.0),
    (-2.0, 2.0, 200.0),
    (1.0, 1.0, 0.0),
    (4.0, 5.0, 25.0),
])
def test_percent_diff_known_answers(v1, v2, expect):
    assert oracle.percent_diff(v1, v2) == pytest.approx(expect, rel=1e-5)


def test_percent_diff_narrows_to_float():
    # absVal takes a float: 0.01 narrows to 0.0099999998 < 0.01, so it counts as "small"
    assert oracle.percent_diff(0.01, 0.0) == 0.0
    assert oracle.percent_diff(0.0100001, 0.0) == pytest.approx(100.0, rel=1e-5)


def test_percent_diff_threshold_boundary():
    assert oracle.percent_diff(1000.0, 1000.5) == pytest.approx(0.05, rel=1e-4)
    assert oracle.percent_diff(1000.0, 1000.49) < 0.05
    assert oracle.percent_diff(1000.0, 1000.51) > 0.05


def test_verify_reports_first_failure_in_row_major_order():
    host = np.ones((4, 4), np.float32) * 10
    dev = host.copy()
    dev[2, 1] = 10.1   # 1 percent
    dev[3, 3] = 20.0
    first, max_pd, nfail = oracle.verify(host, dev)
    assert first == 2 * 4 + 1 and nfail == 2 and max_pd == pytest.approx(100.0)
    assert oracle.verify(host, host)[0] == -1


def test_verify_flags_nan():
    host = np.ones((2, 2), np.float32)
    dev = host.copy()
    dev[0, 1] = np.nan
    # percentDiff(1, NaN) is NaN and NaN > 0.05 is false: the reference's loop passes NaN
    assert oracle.verify(host, dev)[0] == -1
    assert np.isnan(oracle.verify(host, dev)[1])


def test_fp64_reference_and_error_norms():
    rng = np.random.default_rng(0)
    A = rng.standard_normal((20, 30)).astype(np.float32)
    B = rng.standard_normal((30, 25)).astype(np.float32)
    C = rng.standard_normal((20, 25)).astype(np.float32)
    R = oracle.gemm_f64(A, B, C, 2.0, -1.0)
    np.testing.assert_allclose(R, 2.0 * A.astype(np.float64) @ B - C, rtol=1e-12, atol=1e-12)
    RT = oracle.gemm_f64(np.ascontiguousarray(A.T), np.ascontiguousarray(B.T), None, 1.0, 0.0, op_a=1, op_b=1)
    np.testing.assert_allclose(RT, A.astype(np.float64) @ B, rtol=1e-12, atol=1e-12)
    mr, fr, er = oracle.error_norms(R.astype(np.float32), R)
    assert mr < 1e-7 and fr < 1e-7 and er < 1e-6
    bad = R.astype(np.float32)
    bad[0, 0] += 1.0
    assert oracle.error_norms(bad, R)[0] == pytest.approx(1.0 / np.abs(R).max(), rel=1e-3)


def test_oracle_is_thread_count_independent():
    import subprocess
    import sys
    code = ("import sys; sys.path.insert(0, 'oracle'); import oracle, numpy as np; "
            "print(oracle.host_gemm(50).view(np.uint32).sum(dtype=np.uint64))")
    root = Path(__file__).resolve().parent.parent
    outs = {subprocess.run([sys.executable, "-c", code], cwd=root, capture_output=True, text=True, check=True,
                           env={"OMP_NUM_THREADS": t, "PATH": "/usr/bin:/bin"}).stdout for t in ("1", "3")}
    assert len(outs) == 1
