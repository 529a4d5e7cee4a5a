#!/bin/sh
# Test infrastructure: compile the reference's own pattern builder and runtime
# `loc` from its sources (read where they lie, never copied) plus the wrapper
# oracle/ref_pattern.cpp into oracle/_ref/libref_pattern.so.  Needs only g++;
# it does not run the reference's cmake build.  Skips quietly when the
# reference source tree is absent.
#
#   sh oracle/build_ref.sh [REFERENCE_SRC_DIR]
#
# The source directory (the reference's src/) comes from the argument, else
# from SIMIT_REFERENCE_SRC, else from a reference checkout beside this
# repository (../reference/src).
set -e
HERE=$(cd "$(dirname "$0")" && pwd)
REF=${1:-${SIMIT_REFERENCE_SRC:-$HERE/../../reference/src}}
OUT=$HERE/_ref
if [ ! -f "$REF/path_indices.cpp" ]; then
  echo "build_ref: reference sources not found at $REF; skipping" >&2
  exit 0
fi
mkdir -p "$OUT/obj"
# Everything in src/ and src/util/ except the program/function front door
# (which needs the LLVM backend).  path_indices pulls in stencils -> IR.
SRCS=$(ls "$REF"/*.cpp "$REF"/util/*.cpp | grep -v -E '/(program|function)\.cpp$')
echo "$SRCS" | xargs -P "${JOBS:-8}" -I{} sh -c '
  src={}; b=$(echo "$src" | sed "s|.*/src/||; s|/|_|g; s|\.cpp$||")
  obj='"$OUT"'/obj/$b.o
  if [ ! -f "$obj" ] || [ "$src" -nt "$obj" ]; then
    g++ -std=c++11 -O1 -fPIC -w -I'"$REF"' -c "$src" -o "$obj"
  fi'
g++ -std=c++11 -O2 -fPIC -w -I"$REF" -c "$HERE/ref_pattern.cpp" -o "$OUT/obj/_driver.o"
g++ -shared -o "$OUT/libref_pattern.so" "$OUT"/obj/*.o
echo "build_ref: $OUT/libref_pattern.so"
