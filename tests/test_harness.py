"""The drop-in executables' harness on the host device (--device=cpu): CLI,
result formats against the reference's own output, verification paths.
No GPU: the host device runs the reference kernel bodies on the CPU cores.
"""
import json
import re
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
BIN = ROOT / "sycl-bench_gb300" / "bin"
GOLDEN = ROOT / "tests" / "golden"
BENCHES = {"gemm": "Polybench_Gemm", "2mm": "Polybench_2mm", "3mm": "Polybench_3mm", "syrk": "Polybench_Syrk",
           "syr2k": "Polybench_Syr2k"}
# benchmarks the reference builds for float only
FLOAT_ONLY = {"covariance": "Polybench_Covariance", "correlation": "Polybench_Correlation",
              "matmulchain": "MatmulChain", "atax": "Polybench_Atax", "bicg": "Polybench_Bicg", "mvt": "Polybench_Mvt",
              "gesummv": "Polybench_Gesummv"}


@pytest.fixture(scope="module", autouse=True)
def executables():
    import sys
    sys.path.insert(0, str(ROOT / "sycl-bench_gb300"))
    import build
    build.build_lib()
    build.build_executables()


def run(bench, *args, cwd=None):
    r = subprocess.run([str(BIN / bench), *args], capture_output=True, text=True, cwd=cwd,
                       timeout=300)
    assert r.returncode == 0, r.stderr
    return r


def stdout_keys(text):
    return [ln.split(":", 1)[0] for ln in text.splitlines() if ln and not ln.startswith("*")]


@pytest.mark.parametrize("bench", list(BENCHES))
def test_host_device_run_verifies(bench):
    out = run(bench, "--size=48", "--device=cpu", "--num-runs=2").stdout
    blocks = out.split("**********")
    assert f"Results for {BENCHES[bench]}" in out
    assert out.count("Verification: PASS") == 2, out   # FP32 and the fp64 variant
    assert f"Results for {BENCHES[bench]}_fp64" in out


@pytest.mark.parametrize("bench", list(FLOAT_ONLY))
def test_float_only_host_device_run_verifies(bench):
    out = run(bench, "--size=48", "--device=cpu", "--num-runs=2").stdout
    assert f"********** Results for {FLOAT_ONLY[bench]}**********" in out
    assert out.count("Verification: PASS") == 1 and "_fp64" not in out, out


def test_matmulchain_stdout_matches_reference():
    # a benchmark without per-command events: the kernel-time lines stay N/A
    ref = (GOLDEN / "reference_stdout_matmulchain.txt").read_text()
    ours = run("matmulchain", "--size=16", "--num-runs=3", "--device=cpu").stdout
    assert stdout_keys(ours) == stdout_keys(ref)
    assert ours.splitlines()[0] == ref.splitlines()[0]
    kt = [ln for ln in ours.splitlines() if ln.startswith("kernel-time")]
    assert kt and all(ln.endswith("N/A") for ln in kt)


@pytest.mark.parametrize("bench", ["covariance", "correlation"])
def test_statistics_benchmarks_seeded_and_error_report(bench, tmp_path):
    rep = tmp_path / "err.jsonl"
    run(bench, "--size=40", "--device=cpu", "--num-runs=1", "--init=uniform", "--seed=3", f"--error-report={rep}")
    rows = [json.loads(x) for x in rep.read_text().splitlines()]
    assert len(rows) == 1 and rows[0]["init"] == "uniform" and rows[0]["frob_rel"] < 1e-5


def test_error_report_one_line_per_configuration(tmp_path):
    # verify() runs after every run; the report keeps one line per benchmark
    # configuration, and the double variant is labelled fp64
    rep = tmp_path / "g.jsonl"
    run("gemm", "--size=48", "--device=cpu", "--num-runs=3", "--init=uniform", f"--error-report={rep}")
    rows = [json.loads(x) for x in rep.read_text().splitlines()]
    assert [(r["benchmark"], r["precision"]) for r in rows] == [
        ("Polybench_Gemm_uniform_seed1", "fp32"), ("Polybench_Gemm_fp64_uniform_seed1", "fp64")]
    assert rows[1]["frob_rel"] < 1e-13


@pytest.mark.parametrize("bench", ["atax", "bicg", "mvt", "gesummv"])
def test_matrix_vector_benchmarks_fp32_only_and_error_report(bench, tmp_path):
    assert "fp32 form only" in run(bench, "--size=16", "--device=cpu", "--precision=bf16x3").stderr
    rep = tmp_path / "e.jsonl"
    out = run(bench, "--size=64", "--device=cpu", "--num-runs=1", "--init=normal", f"--error-report={rep}").stdout
    assert "GiB/s" in out
    rows = [json.loads(x) for x in rep.read_text().splitlines()]
    assert len(rows) == 1 and rows[0]["frob_rel"] < 1e-5


def test_host_bodies_bitwise_equal_to_per_element_loops(tmp_path):
    # the vectorised --device=cpu bodies keep each element's reference order
    import sys
    sys.path.insert(0, str(ROOT / "sycl-bench_gb300"))
    import build
    exe = tmp_path / "host_bodies_check"
    cmd = ["g++", *build.CXX_FLAGS, "-I", str(build.HARNESS), "-I", str(build.POLY), "-I", str(build.INCLUDE),
           "-I", str(build.cuda_home() / "include"), str(ROOT / "tests" / "host_bodies_check.cpp"), "-o", str(exe),
           "-L", str(build.LIB_DIR), "-lgbpoly", f"-Wl,-rpath,{build.LIB_DIR}"]
    subprocess.run(cmd, check=True, capture_output=True, timeout=300)
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout
    assert r.stdout.count("bitwise equal") == 7 * 12  # 7 sizes x 12 cases


def test_stdout_result_names_match_reference():
    ref = (GOLDEN / "reference_stdout_gemm.txt").read_text()
    ours = run("gemm", "--size=16", "--num-runs=3", "--device=cpu", "--precision=fp32").stdout
    first = ours.split("********** Results for Polybench_Gemm_fp64")[0]
    assert stdout_keys(first) == stdout_keys(ref)
    assert first.splitlines()[0] == ref.splitlines()[0]


def test_csv_columns_match_reference(tmp_path):
    ref_lines = (GOLDEN / "reference_csv_gemm.txt").read_text().splitlines()
    csv = tmp_path / "out.csv"
    run("gemm", "--size=16", "--num-runs=2", "--device=cpu", f"--output={csv}")
    lines = csv.read_text().splitlines()
    assert lines[0] == ref_lines[0]                         # identical header
    row = lines[1].split(",")
    assert row[0] == "Polybench_Gemm"
    # same number of fields (samples are one quoted field without commas)
    assert len(row) == len(ref_lines[1].split(","))
    header = lines[0].split(",")
    cell = dict(zip(header[1:], row[1:]))
    assert cell["Verification"] == "PASS" and cell["problem-size"] == "16" and cell["local-size"] == "256"
    assert re.fullmatch(r'"[0-9. ]+"', cell["run-time-samples"])
    assert lines[2] == ref_lines[0]                         # a header per flush, as the reference
    assert lines[3].startswith("Polybench_Gemm_fp64,")


def test_no_verification_reports_na():
    out = run("syrk", "--size=16", "--device=cpu", "--no-verification", "--num-runs=1").stdout
    assert "Verification: N/A" in out and "PASS" not in out


def test_throughput_metric_is_sp_gflop():
    out = run("gemm", "--size=32", "--device=cpu", "--num-runs=1").stdout
    m = re.search(r"throughput-metric: ([0-9.]+) \[SP GFLOP\]", out)
    assert m and float(m.group(1)) == pytest.approx(2 * 32 ** 3 / 2 ** 30, rel=2e-2)


def test_warmup_run_is_not_recorded():
    out = run("gemm", "--size=16", "--device=cpu", "--num-runs=3", "--warmup-run").stdout
    samples = re.search(r'run-time-samples: "([^"]*)"', out).group(1).split()
    assert len(samples) == 3


def test_duplicate_argument_is_reported():
    r = run("gemm", "--size=16", "--size=32", "--device=cpu")
    assert "several times" in r.stderr


def test_unknown_device_and_precision_are_reported():
    assert "unknown device type" in run("gemm", "--size=16", "--device=fpga").stderr
    assert "unknown --precision" in run("gemm", "--size=16", "--device=cpu", "--precision=fp7").stderr


def test_error_report_and_variants(tmp_path):
    rep = tmp_path / "err.jsonl"
    out = run("syr2k", "--size=40", "--device=cpu", "--num-runs=2", "--init=normal", "--seed=7",
              f"--error-report={rep}").stdout
    assert "Results for Polybench_Syr2k_normal_seed7" in out
    lines = [json.loads(x) for x in rep.read_text().splitlines()]
    assert len(lines) == 2  # one line per configuration (fp32, fp64), not per run
    assert all(x["init"] == "normal" and x["seed"] == 7 for x in lines)
    fp32 = [x for x in lines if x["benchmark"] == "Polybench_Syr2k_normal_seed7"]
    assert fp32 and all(x["frob_rel"] < 1e-5 for x in fp32)


def test_fp64_oracle_verification_mode():
    out = run("3mm", "--size=24", "--device=cpu", "--num-runs=1", "--verification-oracle=fp64").stdout
    assert out.count("Verification: PASS") == 2


def test_alpha_beta_variant_name():
    out = run("syrk", "--size=16", "--device=cpu", "--num-runs=1", "--alpha=32412", "--beta=2123").stdout
    assert "Results for Polybench_Syrk_ab32412_2123" in out
    assert "Verification: PASS" in out


def test_install_layout_runs_like_the_suite_runner(tmp_path):
    """build.py --install puts every executable under <prefix>/bin/benchmarks/,
    where the reference's bin/run-suite looks; each one run the way the runner
    invokes it (its default options with the cpu profile) exits 0 and appends
    its rows to the shared CSV."""
    import os
    import sys
    sys.path.insert(0, str(ROOT / "sycl-bench_gb300"))
    import build
    links = build.install(tmp_path)
    bench_dir = tmp_path / "bin" / "benchmarks"
    names = sorted(p.name for p in bench_dir.iterdir())
    assert names == sorted(list(BENCHES) + list(FLOAT_ONLY)) and len(links) == len(names)
    csv = tmp_path / "sycl-bench.csv"
    for name in names:
        exe = os.path.realpath(bench_dir / name)
        r = subprocess.run([exe, "--device=cpu", "--num-runs=2", f"--output={csv}", "--size=32", "--local=256"],
                           capture_output=True, text=True, timeout=300, cwd=tmp_path)
        assert r.returncode == 0, (name, r.stderr)
    rows = [ln for ln in csv.read_text().splitlines() if ln and not ln.startswith("#")]
    assert all(",PASS," in ln for ln in rows), rows
    assert {ln.split(",")[0] for ln in rows} >= set(BENCHES.values()) | set(FLOAT_ONLY.values())
