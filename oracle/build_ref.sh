#!/usr/bin/env bash
# Builds the reference's own, unmodified C++ sources as the oracle, straight
# from where they lie, into oracle/_ref/ (git-ignored).  TEST INFRASTRUCTURE.
#
#   oracle/_ref/libmdsc_ref.so  function-level harness (oracle/ref_harness.cpp)
#                               + v25/classes.cpp v25/functions.cpp v25/jacobi.c
#   oracle/_ref/libmdsc_ref_serial.so
#                               the same, without -fopenmp: the reference's
#                               loops use schedule(dynamic, floor(N/(16 threads)))
#                               (v25/functions.cpp:1411-1414 and the like), a
#                               chunk of 0 below 16 particles per thread, on
#                               which libgomp never advances; this build runs
#                               the same loops serially for small systems
#   oracle/_ref/DSCmd_v25       the reference driver, v25/main.cpp
#   oracle/_ref/DSCmd_v251      the later variant, v25/v251/main.cpp
#
# The only dependency the reference has that is absent here is GSL's
# random-number generator; oracle/gsl/gsl_rng.h stands in for it.  No source
# file is copied.  -ffp-contract=off keeps the arithmetic identical to the
# reference's own x86 build (no fused multiply-adds) on every host.
set -euo pipefail
# where the reference's sources lie: MDSC_REFERENCE, else this container's
# read-only mount (the one place this repository names that path)
REF="${MDSC_REFERENCE:-/root/reference}"
if [ "${1:-}" = "--where" ]; then
  echo "$REF"
  exit 0
fi
HERE="$(cd "$(dirname "$0")" && pwd)"
OUT="$HERE/_ref"
if [ ! -d "$REF/v25" ]; then
  echo "reference sources not found at $REF; nothing to build" >&2
  exit 0
fi
mkdir -p "$OUT"
CXX="${CXX:-g++}"
FLAGS=(-O2 -fopenmp -ffp-contract=off -w -I"$HERE")
V25="$REF/v25"
V251="$REF/v25/v251"

"$CXX" "${FLAGS[@]}" -fPIC -shared -I"$V25" -o "$OUT/libmdsc_ref.so" \
  "$HERE/ref_harness.cpp" "$V25/classes.cpp" "$V25/functions.cpp" "$V25/jacobi.c" &
"$CXX" -O2 -ffp-contract=off -w -I"$HERE" -fPIC -shared -I"$V25" -o "$OUT/libmdsc_ref_serial.so" \
  "$HERE/ref_harness.cpp" "$V25/classes.cpp" "$V25/functions.cpp" "$V25/jacobi.c" -lgomp &
"$CXX" "${FLAGS[@]}" -I"$V25" -o "$OUT/DSCmd_v25" \
  "$V25/main.cpp" "$V25/classes.cpp" "$V25/functions.cpp" "$V25/jacobi.c" &
# v25/v251/functions.cpp calls getcwd without including <unistd.h>
"$CXX" "${FLAGS[@]}" -include unistd.h -I"$V251" -o "$OUT/DSCmd_v251" \
  "$V251/main.cpp" "$V251/classes.cpp" "$V251/functions.cpp" "$V251/jacobi.c" &
wait
echo "built reference oracle into $OUT"
