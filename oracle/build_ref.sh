#!/bin/bash
# Builds the UNMODIFIED CAPS reference (one rank) from its own sources into
# oracle/_ref/, for cross-checking the oracle restatement.  Runs only where the
# reference sources are present; outputs never leave oracle/_ref/ (git-ignored).
#   oracle/_ref/fromfile1, oracle/_ref/randombenchmark   the reference drivers
#   oracle/_ref/libcapsref.so                           multiply() & friends
#   oracle/_ref/libcholref.so                           cholesky/ mult() & friends
#   oracle/_ref/librectref.so                           rect-class/ rectMM() & friends
# Usage: oracle/build_ref.sh [REFERENCE_DIR] [THREADS]
# REFERENCE_DIR defaults to $CAPS_REFERENCE_DIR, then to where this build's
# container mounts the reference; the directory used is recorded in
# oracle/_ref/REFERENCE_DIR for the tests that read reference sources.
set -euo pipefail
here="$(cd "$(dirname "$0")" && pwd)"
ref="${1:-${CAPS_REFERENCE_DIR:-/root/reference}}"
threads="${2:-$(nproc)}"
out="$here/_ref"
[ -f "$ref/multiply.cpp" ] || { echo "reference sources not found at $ref" >&2; exit 3; }
blasdir="$(python3 -c 'import numpy,os; print(os.path.realpath(os.path.join(os.path.dirname(numpy.__file__), os.pardir, "numpy.libs")))')"
blaslib="$(ls "$blasdir"/libscipy_openblas64_*.so | head -1)"
mkdir -p "$out"
CXX="g++ -O3 -fopenmp -DNUM_THREADS=$threads -include $here/ref_shim/mpi.h -I$here/ref_shim -I$ref -w"
srcs="communication.cpp matrix.cpp multiply.cpp memory.cpp dgemm-blas.cpp counters.cpp library.cpp summa1d.cpp"
objs=""
for s in $srcs; do
  $CXX -fPIC -c "$ref/$s" -o "$out/${s%.cpp}.o"
  objs="$objs $out/${s%.cpp}.o"
done
gcc -O2 -fPIC -c "$here/ref_shim/blas_lp64.c" -o "$out/blas_lp64.o"
link="$out/blas_lp64.o $blaslib -Wl,-rpath,$blasdir"
$CXX -shared -o "$out/libcapsref.so" $objs $link
$CXX "$ref/fromfile1.cpp" $objs $link -o "$out/fromfile1"
$CXX "$ref/randombenchmark.cpp" $objs $link -o "$out/randombenchmark"
# the Cholesky subproject's multiply, mult() (cholesky/mult.cpp), one rank
chol="$ref/cholesky"
cobjs=""
for s in mult.cpp sizes.cpp communication.cpp counters.cpp library.cpp; do
  $CXX -fPIC -I"$chol" -c "$chol/$s" -o "$out/chol_${s%.cpp}.o"
  cobjs="$cobjs $out/chol_${s%.cpp}.o"
done
$CXX -shared -o "$out/libcholref.so" $cobjs $link
# the rectangular subproject's rectMM() (rect-class/rectmm.cpp), one rank
rect="$ref/rect-class"
robjs=""
for s in rectmm.cpp rectsizes.cpp; do
  $CXX -fPIC -I"$rect" -c "$rect/$s" -o "$out/rect_${s%.cpp}.o"
  robjs="$robjs $out/rect_${s%.cpp}.o"
done
$CXX -fPIC -c "$here/ref_shim/rect_comm.cpp" -o "$out/rect_comm.o"
$CXX -shared -o "$out/librectref.so" $robjs "$out/rect_comm.o" $link
rm -f "$out"/*.o
echo "$ref" > "$out/REFERENCE_DIR"
echo "built $out (threads=$threads, blas=$blaslib)"
