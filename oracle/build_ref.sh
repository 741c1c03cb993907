#!/bin/sh
# Builds the reference's app binaries, its gtest suite and a row-dump harness
# from the UNMODIFIED reference sources, writing only into oracle/_ref/.
# Usage: sh oracle/build_ref.sh <reference_dir>
# The reference uses x86 SSE/AVX intrinsics (src/common.hpp includes
# x86intrin.h), so this only runs on x86-64 hosts; elsewhere it says so and
# exits 0.  Flags: GCC 13 needs <functional>/<cassert> force-included, and
# -fno-strict-aliasing (the hybrid dispatcher casts Set<hybrid>* to other
# Set<T>* types; with strict aliasing GCC 13 miscompiles similar_nodes).
set -e
REF=${1:-}
if [ -z "$REF" ]; then
  echo "build_ref: usage: sh oracle/build_ref.sh <reference tree>; skipped"
  exit 0
fi
HERE=$(cd "$(dirname "$0")" && pwd)
OUT="$HERE/_ref"
if [ "$(uname -m)" != "x86_64" ]; then
  echo "build_ref: reference needs x86-64 SSE/AVX intrinsics; skipped on $(uname -m)"
  exit 0
fi
if [ ! -d "$REF/src" ]; then
  echo "build_ref: no reference tree at $REF; skipped"
  exit 0
fi
mkdir -p "$OUT"
CXX=${CXX:-g++}
FLAGS="-include functional -include cassert -mavx -std=c++11 -fopenmp -O3 -march=native -fno-strict-aliasing -w -I$REF/src"
stamp="$OUT/.stamp"
if [ -f "$stamp" ] && [ "$stamp" -nt "$HERE/build_ref.sh" ] && [ "$stamp" -nt "$HERE/ref_rowdump.cpp" ]; then
  exit 0
fi
pids=""
for app in undirected_triangle_counting n_clique undirected_lollipop_counting similar_nodes symbiosity n_path; do
  $CXX $FLAGS "$REF/apps/$app.cpp" -o "$OUT/$app" &
  pids="$pids $!"
done
$CXX $FLAGS "$HERE/ref_rowdump.cpp" -o "$OUT/ref_rowdump" &
pids="$pids $!"
# gtest 1.7.0 as vendored by the reference, then the reference's own tests.
GT="$REF/lib/gtest-1.7.0"
if [ -d "$GT/src" ]; then
  $CXX -O2 -w -I"$GT/include" -I"$GT" -c "$GT/src/gtest-all.cc" -o "$OUT/gtest-all.o" -pthread &
  p1=$!
  $CXX -O2 -w -I"$GT/include" -I"$GT" -c "$GT/src/gtest_main.cc" -o "$OUT/gtest_main.o" -pthread &
  p2=$!
  wait $p1 $p2
  for t in undirected_triangle_counting_test n_clique_test undirected_lollipop_counting_test similar_nodes_test symbiosity_test n_path_test; do
    $CXX $FLAGS -DGOOGLE_TEST -I"$REF/apps" -I"$GT/include" "$REF/test/$t.cpp" "$OUT/gtest-all.o" "$OUT/gtest_main.o" -pthread -o "$OUT/$t" &
    pids="$pids $!"
  done
fi
for p in $pids; do wait $p; done
touch "$stamp"
echo "build_ref: reference binaries in $OUT"
