"""The reference's own suite runner drives the installed executables.

sycl-bench's bin/run-suite (a plain Python 3 script) walks the benchmarks
directory beside itself, runs every executable there with its profile's
options (bin/run-suite:157-168: --size=1024 by default, 4096 for atax,
16384 for bicg/mvt/gesummv, --num-runs=10, --output=./sycl-bench.csv) and
aborts with a non-zero exit code if any benchmark returns one
(bin/run-suite:279-293).  This test installs the executables with
build.py --install, puts the UNCHANGED runner read from the reference tree
beside them (copied at test time into the test's temporary prefix, since the
runner locates its benchmarks relative to its own path) and runs it with the
"cpu-noverify" profile: the kernels on the host cores, as a SYCL CPU device
runs them, without the host verification loops that take minutes at these
sizes.  Skipped where the reference tree is not on the machine.
"""
import os
import shutil
import subprocess
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
RUNNER = Path(os.environ.get("REFERENCE_ROOT", "/root/reference")) / "bin" / "run-suite"

# benchmark name (the CSV's first column) of every installed executable
NAMES = {"gemm": "Polybench_Gemm", "2mm": "Polybench_2mm", "3mm": "Polybench_3mm", "syrk": "Polybench_Syrk",
         "syr2k": "Polybench_Syr2k", "covariance": "Polybench_Covariance", "correlation": "Polybench_Correlation",
         "matmulchain": "MatmulChain", "atax": "Polybench_Atax", "bicg": "Polybench_Bicg", "mvt": "Polybench_Mvt",
         "gesummv": "Polybench_Gesummv"}


@pytest.mark.skipif(not RUNNER.exists(), reason="the reference's bin/run-suite is not on this machine")
def test_unchanged_run_suite_runs_every_installed_benchmark(tmp_path):
    sys.path.insert(0, str(ROOT / "sycl-bench_gb300"))
    import build
    if not all((build.BIN_DIR / name).exists() for name in NAMES):
        pytest.skip("executables not built (run __graft_entry__.build())")
    build.install(tmp_path)
    runner = tmp_path / "bin" / "run-suite"
    shutil.copyfile(RUNNER, runner)
    work = tmp_path / "work"
    work.mkdir()
    r = subprocess.run([sys.executable, str(runner), "cpu-noverify"], capture_output=True, text=True, timeout=900,
                       cwd=work)
    assert r.returncode == 0, (r.stdout[-3000:], r.stderr[-3000:])
    assert "All benchmarks were executed successfully" in r.stdout
    # every executable appends a "# "-prefixed header line and then its rows
    # (include/result_consumer.h's appending CSV consumer)
    header, by_name = None, {}
    for ln in (work / "sycl-bench.csv").read_text().splitlines():
        if ln.startswith("# "):
            header = ln[2:].split(",")
        elif ln:
            row = ln.split(",")
            by_name[row[0]] = dict(zip(header, row))
    for exe, name in NAMES.items():
        assert name in by_name, (exe, sorted(by_name))
        row = by_name[name]
        assert row["problem-size"] == str({"atax": 4096, "bicg": 16384, "mvt": 16384,
                                           "gesummv": 16384}.get(exe, 1024)), row
        assert len(row["run-time-samples"].strip('"').split()) == 10 and row["device-name"], row
        assert float(row["run-time-min"]) > 0.0, row
