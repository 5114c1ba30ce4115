#!/bin/bash
# Compiles the reference's own CPU functions from its sources, where they lie,
# into oracle/_ref/libref_cpu.so (git-ignored).  Only host C++ is compiled:
#   test/dspmv_test_smt.cu   -> csr_spmv_cpu        (:39-52)
#   test/dspmv_test_dgx1.cu  -> coo_spmv_cpu        (:55-69)
#   src/spmv_helper.cu       -> get_row_from_index, findFirstInSorted,
#                               findLastInSorted    (:18-44, :646-685)
# The CUDA / cuSPARSE calls elsewhere in those files compile against the
# host-only stand-in headers in oracle/ref_shim/ and are never executed.  The
# reference's GPU path (cuSPARSE csrmv / csrmv_mp, CSR5) does not build with
# CUDA 13 and is not compiled.
# Usage: oracle/ref_build.sh [REFERENCE_ROOT]; the root is the argument, else
# $SBLAS_REFERENCE_DIR, else the read-only location this recipe is run
# against in the build container.  The root used is recorded in
# oracle/_ref/REFERENCE_DIR for the tests that compile the reference's drivers.
set -euo pipefail
HERE="$(cd "$(dirname "$0")" && pwd)"
REF="${1:-${SBLAS_REFERENCE_DIR:-/root/reference}}"
OUT="$HERE/_ref"
if [ ! -f "$REF/test/dspmv_test_smt.cu" ]; then
  echo "reference sources not found under $REF; skipping oracle/_ref" >&2
  exit 0
fi
mkdir -p "$OUT"
CXX="${CXX:-g++}"
FLAGS="-O2 -fPIC -fopenmp -ffp-contract=off -w -x c++ -I$HERE/ref_shim -I$REF/include"
$CXX $FLAGS -Dmain=sblas_ref_unused_main_smt -c "$REF/test/dspmv_test_smt.cu" -o "$OUT/smt.o"
$CXX $FLAGS -Dmain=sblas_ref_unused_main_dgx1 -Dcsr_spmv_cpu=sblas_ref_unused_csr_dgx1 \
     -Dprint_error=sblas_ref_unused_print_error_dgx1 -c "$REF/test/dspmv_test_dgx1.cu" -o "$OUT/dgx1.o"
# both drivers define the header-only mmio functions; keep one copy
objcopy --weaken "$OUT/dgx1.o"
$CXX $FLAGS -c "$REF/src/spmv_helper.cu" -o "$OUT/helper.o"
$CXX -O2 -fPIC -fopenmp -ffp-contract=off -c "$HERE/ref_shim/ref_entry.cpp" -o "$OUT/entry.o"
$CXX -shared -fopenmp -o "$OUT/libref_cpu.so" "$OUT/smt.o" "$OUT/dgx1.o" "$OUT/helper.o" "$OUT/entry.o"
rm -f "$OUT"/*.o
printf '%s\n' "$REF" > "$OUT/REFERENCE_DIR"
echo "built $OUT/libref_cpu.so"
