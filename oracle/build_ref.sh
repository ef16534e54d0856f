#!/bin/sh
# Compile the reference's own PolyBench sources (read in place under
# /root/reference, never copied) against the host-only SYCL stand-in, into
# oracle/_ref/ref_<benchmark>.  TEST INFRASTRUCTURE ONLY.
# Flags: no -ffast-math and no FMA contraction, so the reference's float
# operation order is kept exactly (the oracle restatement is built the same way).
set -e
HERE=$(cd "$(dirname "$0")" && pwd)
REF=${REFERENCE_ROOT:-/root/reference}
OUT="$HERE/_ref"
CXX=${CXX:-g++}
if [ ! -f "$REF/polybench/gemm.cpp" ]; then
  echo "reference sources not found under $REF; skipping oracle/_ref" >&2
  exit 0
fi
mkdir -p "$OUT"
build() {  # name macro [directory]
  src="$REF/${3:-polybench}/$1.cpp"
  bin="$OUT/ref_$1"
  if [ -f "$bin" ] && [ "$bin" -nt "$src" ] && [ "$bin" -nt "$HERE/ref_driver.cpp" ] && [ "$bin" -nt "$HERE/sycl_shim/sycl/sycl.hpp" ]; then
    return 0
  fi
  $CXX -std=c++17 -O2 -ffp-contract=off -fopenmp -w \
    -I"$HERE/sycl_shim" -I"$REF/include" -I"$REF/polybench/common" \
    -DREF_SOURCE="\"$src\"" -D"$2" "$HERE/ref_driver.cpp" -o "$bin"
}
build gemm REF_GEMM &
build 2mm REF_2MM &
build 3mm REF_3MM &
build syrk REF_SYRK &
build syr2k REF_SYR2K &
build covariance REF_COVARIANCE &
build correlation REF_CORRELATION &
build matmulchain REF_MATMULCHAIN runtime &
build atax REF_ATAX &
build bicg REF_BICG &
build mvt REF_MVT &
build gesummv REF_GESUMMV &
wait
for b in gemm 2mm 3mm syrk syr2k covariance correlation matmulchain atax bicg mvt gesummv; do test -x "$OUT/ref_$b" || { echo "failed to build ref_$b" >&2; exit 1; }; done
