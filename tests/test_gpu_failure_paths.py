"""Failure paths, exercised without any fault on the GPU.

The reference reports device errors by throwing from
queue::wait_and_throw() and catches them per benchmark: the partial results
are discarded, the error goes to stderr and the process still exits 0
(include/common.h:123-126, :208-212); a wrong result only turns the CSV's
Verification column to FAIL.  Here:

  * a bounded device-side wait that runs out (gbpoly_wait_probe: the kernels'
    own wait routine on an mbarrier nothing completes) makes the next
    gbpoly_synchronize return GBPOLY_ERR_TIMEOUT, and the same context then
    computes a contraction correctly;
  * GBPOLY_FAULT_INJECT=alloc:N fails an allocation on the host (NOMEM) and
    corrupt:N changes a copied-back element on the host, through the C ABI and
    through a drop-in executable, which must behave as the reference does.
"""
import os
import subprocess
from pathlib import Path

import numpy as np
import pytest

import gbpoly
import oracle
from gbpoly import Precision

pytestmark = pytest.mark.gpu

BIN = Path(__file__).resolve().parent.parent / "sycl-bench_gb300" / "bin"


def small_gemm_ok(ctx):
    n = 128
    A, B, C = oracle.init_gemm(n)
    dA, dB, dC = ctx.upload(A), ctx.upload(B), ctx.upload(C)
    ctx.gemm(Precision.BF16X3, n, n, n, 32412.0, dA, n, dB, n, 2123.0, dC, n)
    ctx.synchronize()
    out = ctx.download(dC, (n, n))
    for b in (dA, dB, dC):
        ctx.free(b)
    assert oracle.verify(oracle.host_gemm(n), out)[0] == -1


def test_wait_timeout_is_reported_and_the_context_stays_usable(ctx):
    ctx.wait_probe(2000)  # 2 ms
    with pytest.raises(gbpoly.GbpolyError) as e:
        ctx.synchronize()
    assert e.value.status == gbpoly.Status.TIMEOUT
    assert "code 7" in str(e.value)
    ctx.synchronize()  # the error word was cleared
    small_gemm_ok(ctx)


def test_injected_allocation_failure_through_the_c_abi(monkeypatch):
    monkeypatch.setenv("GBPOLY_FAULT_INJECT", "alloc:2")
    with gbpoly.Context(0) as c:
        first = c.alloc(1024)  # the first allocation succeeds
        with pytest.raises(gbpoly.GbpolyError) as e:
            c.alloc(1024)
        assert e.value.status == gbpoly.Status.NOMEM
        third = c.alloc(1024)  # the injection fires once
        c.free(first)
        c.free(third)
    monkeypatch.delenv("GBPOLY_FAULT_INJECT")
    with gbpoly.Context(0) as c:  # a context created without the variable leaves nothing pending
        c.free(c.alloc(1024))


def test_injected_corruption_through_the_c_abi(monkeypatch):
    monkeypatch.setenv("GBPOLY_FAULT_INJECT", "corrupt:1")
    with gbpoly.Context(0) as c:
        x = np.arange(16, dtype=np.float32) + 3.0
        d = c.upload(x)
        got = c.download(d, (16,))
        assert got[0] == 2 * 3.0 + 1 and np.array_equal(got[1:], x[1:])
        assert np.array_equal(c.download(d, (16,)), x)  # only the one copy
    monkeypatch.delenv("GBPOLY_FAULT_INJECT")


def run_gemm_exe(env_value):
    """The gemm executable (its float benchmark, then its double variant); stdout per benchmark."""
    env = dict(os.environ, GBPOLY_FAULT_INJECT=env_value)
    r = subprocess.run([str(BIN / "gemm"), "--size=64", "--num-runs=1", "--device=gpu"], capture_output=True,
                       text=True, timeout=120, env=env)
    blocks = {}
    for part in r.stdout.split("********** Results for ")[1:]:
        name, _, body = part.partition("**********")
        blocks[name.strip()] = body
    return r, blocks


def test_dropin_discards_results_on_allocation_failure():
    # the first allocation is the float benchmark's first buffer: that benchmark
    # is abandoned (no timings, no verification line) and the next one runs
    r, blocks = run_gemm_exe("alloc:1")
    assert r.returncode == 0, r.stderr
    assert "allocation failure injected" in r.stderr, r.stderr
    assert "Verification:" not in blocks["Polybench_Gemm"] and "run-time-mean" not in blocks["Polybench_Gemm"]
    assert "Verification: PASS" in blocks["Polybench_Gemm_fp64"], r.stdout


def test_dropin_reports_fail_on_a_corrupted_result():
    # the first copy back to the host is the float benchmark's verification read
    r, blocks = run_gemm_exe("corrupt:1")
    assert r.returncode == 0, r.stderr
    assert "Verification: FAIL" in blocks["Polybench_Gemm"], r.stdout
    assert "Verification: PASS" in blocks["Polybench_Gemm_fp64"], r.stdout
    clean, blocks = run_gemm_exe("")
    assert "Verification: PASS" in blocks["Polybench_Gemm"], clean.stdout
