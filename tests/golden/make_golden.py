"""Generate the golden fixtures from the reference itself.

Runs the reference's own PolyBench sources, built by oracle/build_ref.sh
against the host-only SYCL stand-in (this needs the reference sources on the
machine), and stores:

  reference_outputs.npz   for each benchmark and size n:
                            <bench>_<n>_host    its host verification loop result
                                                (matmulchain: the identity its verify expects)
                            <bench>_<n>_device  its run() kernels' output (host execution)
                          covariance and correlation arrays are (n + 1) x (n + 1);
                          atax, gesummv: y; bicg: s then q; mvt: x1 then x2
  reference_stdout_gemm.txt  its main() output with --output=stdio
  reference_csv_gemm.txt     its main() output with --output=<csv file> (two flushes)
  reference_stdout_matmulchain.txt  runtime/matmulchain.cpp's main() output (a
                             benchmark without per-command events)

Usage:  python tests/golden/make_golden.py
"""
import os
import subprocess
import sys
import tempfile
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
REF_BIN = ROOT / "oracle" / "_ref"
BENCHES = ["gemm", "2mm", "3mm", "syrk", "syr2k", "covariance", "correlation", "matmulchain", "atax", "bicg", "mvt",
           "gesummv"]
PADDED = {"covariance", "correlation"}  # (n + 1) x (n + 1) arrays
VECTORS = {"atax", "bicg", "mvt", "gesummv"}  # output vectors (bicg: s then q; mvt: x1 then x2)
SIZES = [1, 2, 7, 16, 37, 64]


def main() -> None:
    subprocess.run([str(ROOT / "oracle" / "build_ref.sh")], check=True)
    arrays = {}
    with tempfile.TemporaryDirectory() as td:
        for b in BENCHES:
            for n in SIZES:
                prefix = os.path.join(td, f"{b}_{n}")
                r = subprocess.run([str(REF_BIN / f"ref_{b}"), str(n), prefix], check=True, capture_output=True,
                                   text=True)
                if "verify=PASS" not in r.stdout:
                    sys.exit(f"reference verify failed for {b} n={n}: {r.stdout}")
                m = n + 1 if b in PADDED else n
                for kind in ("host", "device"):
                    a = np.fromfile(f"{prefix}_{kind}.f32", np.float32)
                    arrays[f"{b}_{n}_{kind}"] = a if b in VECTORS else a.reshape(m, m)
        np.savez_compressed(HERE / "reference_outputs.npz", **arrays)

        out = subprocess.run([str(REF_BIN / "ref_gemm"), "--main", "--size=16", "--num-runs=3"], check=True,
                             capture_output=True, text=True).stdout
        (HERE / "reference_stdout_gemm.txt").write_text(out)
        csv = os.path.join(td, "out.csv")
        for _ in range(2):
            subprocess.run([str(REF_BIN / "ref_gemm"), "--main", "--size=16", "--num-runs=2", f"--output={csv}"],
                           check=True, capture_output=True)
        (HERE / "reference_csv_gemm.txt").write_text(Path(csv).read_text())
        out = subprocess.run([str(REF_BIN / "ref_matmulchain"), "--main", "--size=16", "--num-runs=3"], check=True,
                             capture_output=True, text=True).stdout
        (HERE / "reference_stdout_matmulchain.txt").write_text(out)
    print("wrote", HERE / "reference_outputs.npz")


if __name__ == "__main__":
    main()
