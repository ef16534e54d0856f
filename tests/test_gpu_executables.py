"""The drop-in executables on the GPU: every precision form verifies with the
reference's own host loop (matmulchain: its exact identity check), CSV
columns are the reference's, and the CUDA-event kernel timings are filled."""
import re
import subprocess
from pathlib import Path

import pytest

pytestmark = pytest.mark.gpu

ROOT = Path(__file__).resolve().parent.parent
BIN = ROOT / "sycl-bench_gb300" / "bin"
GOLDEN = ROOT / "tests" / "golden"
BENCHES = {"gemm": "Polybench_Gemm", "2mm": "Polybench_2mm", "3mm": "Polybench_3mm", "syrk": "Polybench_Syrk",
           "syr2k": "Polybench_Syr2k"}
FLOAT_ONLY = {"covariance": "Polybench_Covariance", "correlation": "Polybench_Correlation",
              "matmulchain": "MatmulChain"}
MATVEC = {"atax": "Polybench_Atax", "bicg": "Polybench_Bicg", "mvt": "Polybench_Mvt", "gesummv": "Polybench_Gesummv"}


def run(bench, *args):
    r = subprocess.run([str(BIN / bench), *args], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    assert "rror" not in r.stderr, r.stderr
    return r.stdout


@pytest.mark.parametrize("bench", list(BENCHES))
def test_all_forms_verify_on_gpu(bench):
    out = run(bench, "--size=320", "--num-runs=2", "--precision=fp32,bf16x3,tf32x3,bf16x6,fp16x3")
    names = re.findall(r"Results for (\S+?)\*", out)
    base = BENCHES[bench]
    assert names == [base, base + "_bf16x3", base + "_tf32x3", base + "_bf16x6", base + "_fp16x3", base + "_fp64"]
    assert out.count("Verification: PASS") == 6, out
    assert "kernel-time-mean: N/A" not in out
    assert "NVIDIA" in out or "GB" in out  # device-name is the CUDA device


def test_csv_columns_match_reference_on_gpu(tmp_path):
    csv = tmp_path / "o.csv"
    run("gemm", "--size=1024", "--num-runs=3", f"--output={csv}")
    lines = csv.read_text().splitlines()
    assert lines[0] == (GOLDEN / "reference_csv_gemm.txt").read_text().splitlines()[0]
    cell = dict(zip(lines[0].split(",")[1:], lines[1].split(",")[1:]))
    assert cell["Verification"] == "PASS"
    assert float(cell["kernel-time-min"]) > 0 and float(cell["kernel-time-min"]) <= float(cell["run-time-min"])


def test_fp64_oracle_and_error_report_on_gpu(tmp_path):
    rep = tmp_path / "e.jsonl"
    out = run("syr2k", "--size=512", "--num-runs=1", "--precision=fp32,bf16x3", "--verification-oracle=fp64",
              f"--error-report={rep}")
    assert out.count("Verification: PASS") == 3
    assert len(rep.read_text().splitlines()) == 3
    # random inputs: percentDiff fails near-zero results by construction, the report carries the norms
    rep2 = tmp_path / "n.jsonl"
    run("syr2k", "--size=512", "--num-runs=1", "--precision=fp32,tf32x3", "--init=normal", f"--error-report={rep2}")
    import json
    rows = [json.loads(x) for x in rep2.read_text().splitlines()]
    assert len(rows) == 3 and all(r["frob_rel"] < 1e-5 for r in rows)


@pytest.mark.parametrize("bench", ["2mm", "3mm"])
def test_graph_mode_verifies(bench):
    out = run(bench, "--size=512", "--num-runs=3", "--graph", "--precision=fp32,bf16x3")
    base = BENCHES[bench]
    names = re.findall(r"Results for (\S+?)\*", out)
    assert names == [base + "_graph", base + "_bf16x3_graph", base + "_fp64_graph"]
    assert out.count("Verification: PASS") == 3, out


@pytest.mark.parametrize("flags", [("--grouped",), ("--grouped", "--graph")])
def test_3mm_grouped_mode_verifies(flags):
    # E and F as one grouped launch (with or without the graph); the double
    # variant keeps its three launches
    out = run("3mm", "--size=300", "--num-runs=2", *flags, "--precision=fp32,bf16x3,fp16x3")
    base = BENCHES["3mm"]
    names = re.findall(r"Results for (\S+?)\*", out)
    sfx = "_grouped" + ("_graph" if "--graph" in flags else "")
    assert names == [base + sfx, base + "_bf16x3" + sfx, base + "_fp16x3" + sfx,
                     base + "_fp64" + ("_graph" if "--graph" in flags else "")]
    assert out.count("Verification: PASS") == 4, out


@pytest.mark.parametrize("size", [257, 1024])
@pytest.mark.parametrize("bench", list(FLOAT_ONLY))
def test_float_only_benchmarks_verify_on_gpu(bench, size):
    out = run(bench, f"--size={size}", "--num-runs=2", "--precision=fp32,bf16x3,tf32x3,bf16x6,fp16x3")
    names = re.findall(r"Results for (\S+?)\*", out)
    base = FLOAT_ONLY[bench]
    assert names == [base, base + "_bf16x3", base + "_tf32x3", base + "_bf16x6", base + "_fp16x3"]
    assert out.count("Verification: PASS") == 5, out
    if bench == "matmulchain":  # run() without events, as the reference
        assert "kernel-time-mean: N/A" in out
    else:
        assert "kernel-time-mean: N/A" not in out


def test_matmulchain_graph_grouped_and_seeded(tmp_path):
    out = run("matmulchain", "--size=512", "--num-runs=2", "--graph", "--grouped", "--precision=fp32,bf16x3")
    names = re.findall(r"Results for (\S+?)\*", out)
    assert names == ["MatmulChain_grouped_graph", "MatmulChain_bf16x3_grouped_graph"]
    assert out.count("Verification: PASS") == 2, out
    out = run("matmulchain", "--size=384", "--num-runs=1", "--grouped", "--precision=tf32x3,fp16x3")
    assert "Results for MatmulChain_tf32x3_grouped" in out and "Results for MatmulChain_fp16x3_grouped" in out
    assert out.count("Verification: PASS") == 2, out
    rep = tmp_path / "m.jsonl"
    out = run("matmulchain", "--size=512", "--num-runs=1", "--init=uniform", "--precision=fp32,bf16x3",
              f"--error-report={rep}")
    import json
    rows = [json.loads(x) for x in rep.read_text().splitlines()]
    assert [r["precision"] for r in rows] == ["fp32", "bf16x3"]
    assert all(r["frob_rel"] < 2e-5 for r in rows), rows


@pytest.mark.parametrize("bench", ["covariance", "correlation"])
def test_statistics_benchmarks_error_report_on_gpu(bench, tmp_path):
    rep = tmp_path / "s.jsonl"
    out = run(bench, "--size=1000", "--num-runs=1", "--precision=fp32,bf16x3,tf32x3,fp16x3", f"--error-report={rep}")
    assert out.count("Verification: PASS") == 4, out
    import json
    rows = [json.loads(x) for x in rep.read_text().splitlines()]
    assert len(rows) == 4 and all(r["frob_rel"] < 1e-5 for r in rows), rows


@pytest.mark.parametrize("size", [1024, 4099])
@pytest.mark.parametrize("bench", list(MATVEC))
def test_matrix_vector_benchmarks_verify_on_gpu(bench, size, tmp_path):
    rep = tmp_path / "v.jsonl"
    out = run(bench, f"--size={size}", "--num-runs=3", f"--error-report={rep}")
    assert f"Results for {MATVEC[bench]}*" in out
    assert out.count("Verification: PASS") == 1, out
    assert "kernel-time-mean: N/A" not in out and "[GiB/s]" in out
    import json
    rows = [json.loads(x) for x in rep.read_text().splitlines()]
    assert rows and all(r["frob_rel"] < 1e-5 for r in rows), rows
