"""Build libgbpoly.so (CUDA, sm_103a) and the PolyBench executables in-tree.

    python sycl-bench_gb300/build.py            # library + executables
    python sycl-bench_gb300/build.py --lib      # library only
    python sycl-bench_gb300/build.py --install PREFIX   # + PREFIX/bin/benchmarks/<name> links

Outputs (git-ignored):
    sycl-bench_gb300/lib/libgbpoly.so
    sycl-bench_gb300/bin/{gemm,2mm,3mm,syrk,syr2k,covariance,correlation,matmulchain,
                          atax,bicg,mvt,gesummv}

Each executable is named after its source file, as the reference's build
names its targets (CMakeLists.txt:149-151), so the reference's suite runner
finds them under bin/benchmarks/<name>.

Translation units compile in parallel; a unit is rebuilt only when it or a
header it may include is newer than its object.  Host code is portable C++17
(Grace hosts are aarch64; the same sources build on x86_64).
"""
from __future__ import annotations

import argparse
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
HARNESS = PKG / "harness"
POLY = PKG / "polybench"
RUNTIME = PKG / "runtime"
LIB_DIR = PKG / "lib"
BIN_DIR = PKG / "bin"
OBJ_DIR = PKG / "_build"
INCLUDE = ROOT / "include"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr",
              "-Xptxas", "-warn-spills"] + ARCH
# The benchmarks' host oracle loops compare against the reference's own FP32
# loops: no -ffast-math and no FMA contraction, so the host results are the
# reference's operation order on every host ISA.  Double variants and queue
# profiling are on (sycl-bench's SYCL_BENCH_HAS_FP64_SUPPORT /
# SYCL_BENCH_ENABLE_QUEUE_PROFILING).
CXX_FLAGS = ["-O3", "-std=c++17", "-fopenmp", "-ffp-contract=off", "-Wall", "-Wno-unknown-pragmas",
             "-DSYCL_BENCH_HAS_FP64_SUPPORT=1", "-DSYCL_BENCH_ENABLE_QUEUE_PROFILING=1"]

# (source directory, name): the reference's polybench/<name>.cpp and runtime/<name>.cpp
BENCHMARKS = [(POLY, "gemm"), (POLY, "2mm"), (POLY, "3mm"), (POLY, "syrk"), (POLY, "syr2k"),
              (POLY, "covariance"), (POLY, "correlation"), (RUNTIME, "matmulchain"),
              (POLY, "atax"), (POLY, "bicg"), (POLY, "mvt"), (POLY, "gesummv")]


def nvcc() -> str:
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(cand).exists():
        raise RuntimeError("nvcc not found")
    return cand


def cuda_home() -> Path:
    return Path(nvcc()).resolve().parent.parent


def _newer(target: Path, deps: list[Path]) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps if d.exists())


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"command failed ({r.returncode}): {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    if r.stderr.strip():
        # ptxas spill warnings and the like: keep them visible
        sys.stderr.write(r.stderr)


def build_lib(verbose: bool = False) -> Path:
    OBJ_DIR.mkdir(exist_ok=True)
    LIB_DIR.mkdir(exist_ok=True)
    sources = sorted(CSRC.glob("*.cu"))
    headers = sorted(CSRC.glob("*.cuh")) + [INCLUDE / "gbpoly.h"]
    jobs = []
    objs = []
    for src in sources:
        obj = OBJ_DIR / (src.stem + ".o")
        objs.append(obj)
        if _newer(obj, [src] + headers):
            cmd = [nvcc(), *NVCC_FLAGS, "-I", str(INCLUDE), "-c", str(src), "-o", str(obj)]
            if verbose:
                cmd += ["-Xptxas", "-v"]
            jobs.append(cmd)
    with cf.ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        list(ex.map(_run, jobs))
    lib = LIB_DIR / "libgbpoly.so"
    if jobs or _newer(lib, objs):
        _run([nvcc(), *ARCH, "-shared", "-o", str(lib), *map(str, objs), "-lcudart"])
    return lib


def build_executables() -> list[Path]:
    BIN_DIR.mkdir(exist_ok=True)
    lib = LIB_DIR / "libgbpoly.so"
    cuda_inc = cuda_home() / "include"
    headers = sorted(HARNESS.glob("*.h")) + sorted(POLY.glob("*.h")) + [INCLUDE / "gbpoly.h", lib]
    jobs, outs = [], []
    for src_dir, name in BENCHMARKS:
        src = src_dir / f"{name}.cpp"
        if not src.exists():
            continue
        out = BIN_DIR / name
        outs.append(out)
        if _newer(out, [src] + headers):
            jobs.append([shutil.which("g++") or "g++", *CXX_FLAGS, "-I", str(HARNESS), "-I", str(POLY),
                         "-I", str(INCLUDE), "-I", str(cuda_inc), str(src), "-o", str(out),
                         "-L", str(LIB_DIR), "-lgbpoly", f"-Wl,-rpath,{LIB_DIR}", "-Wl,-rpath,$ORIGIN/../lib"])
    with cf.ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        list(ex.map(_run, jobs))
    return outs


def install(prefix: Path) -> list[Path]:
    """Link the built executables into <prefix>/bin/benchmarks/<name>, the
    layout the reference's suite runner walks (CMakeLists.txt:170 installs
    there; bin/run-suite runs every executable it finds in the benchmarks
    directory beside itself).  Links resolve to this tree, so each executable
    still finds lib/libgbpoly.so through its $ORIGIN run path."""
    dest = Path(prefix) / "bin" / "benchmarks"
    dest.mkdir(parents=True, exist_ok=True)
    out = []
    for _, name in BENCHMARKS:
        src = BIN_DIR / name
        if not src.exists():
            continue
        link = dest / name
        if link.is_symlink() or link.exists():
            link.unlink()
        link.symlink_to(src)
        out.append(link)
    return out


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--lib", action="store_true", help="library only")
    ap.add_argument("-v", "--verbose", action="store_true", help="ptxas resource usage")
    ap.add_argument("--install", metavar="PREFIX", help="also link the executables into PREFIX/bin/benchmarks/")
    args = ap.parse_args()
    lib = build_lib(verbose=args.verbose)
    print(lib)
    if not args.lib and (POLY / "gemm.cpp").exists():
        for p in build_executables():
            print(p)
        if args.install:
            for p in install(Path(args.install)):
                print(p)


if __name__ == "__main__":
    main()
