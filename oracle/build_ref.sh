#!/bin/sh
# Compiles the reference aMat CPU path IN PLACE from the reference tree into
# oracle/_ref/libamat_ref.so (test infrastructure; never shipped or loaded by
# the product). Only the reference's own sources are compiled, against the
# single-rank MPI / minimal PETSc shims in oracle/shim/.
#   REF  - reference checkout (default: a directory named reference beside
#          this repository's root)
#   CXX  - C++ compiler (default g++)
# The reference's unconditional <immintrin.h> (include/aMat.hpp:31) limits this
# to x86 hosts; elsewhere the script exits 0 without building.
set -e
HERE=$(cd "$(dirname "$0")" && pwd)
REF=${REF:-$HERE/../../reference}
CXX=${CXX:-g++}
OUT="$HERE/_ref"
if [ ! -d "$REF/include" ]; then echo "build_ref: no reference tree at $REF, skipped"; exit 0; fi
case "$(uname -m)" in x86_64|amd64) ;; *) echo "build_ref: reference needs x86 intrinsics headers, skipped on $(uname -m)"; exit 0;; esac
mkdir -p "$OUT"
FLAGS="-O2 -std=c++14 -fopenmp -fPIC -DHYBRID_PARALLEL -w -I$HERE/shim -I$REF/include -I$REF/examples/include -I$REF"
$CXX $FLAGS -c "$REF/examples/src/ke_matrix.cpp" -o "$OUT/ke_matrix.o"
$CXX $FLAGS -c "$HERE/ref_harness.cpp" -o "$OUT/ref_harness.o"
$CXX -shared -fopenmp "$OUT/ref_harness.o" "$OUT/ke_matrix.o" -o "$OUT/libamat_ref.so"
echo "build_ref: $OUT/libamat_ref.so"
# the reference's VECTORIZED_OPENMP build (column-major element matrices, omp simd element product)
$CXX $FLAGS -DVECTORIZED_OPENMP -c "$REF/examples/src/ke_matrix.cpp" -o "$OUT/ke_matrix_simd.o"
$CXX $FLAGS -DVECTORIZED_OPENMP -c "$HERE/ref_harness.cpp" -o "$OUT/ref_harness_simd.o"
$CXX -shared -fopenmp "$OUT/ref_harness_simd.o" "$OUT/ke_matrix_simd.o" -o "$OUT/libamat_ref_simd.so"
echo "build_ref: $OUT/libamat_ref_simd.so"
