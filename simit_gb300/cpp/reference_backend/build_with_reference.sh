#!/bin/sh
# Builds the reference-side binding against a reference checkout: the
# reference's frontend, IR, lowering and backend factory (its own sources,
# compiled unmodified from where they lie), this directory's GB300 backend,
# and isprings_main, the reference's isprings program test run through
# simit::Program / simit::Function.
#
# The reference's LLVM and GPU backends are not compiled (no LLVM in this
# image); shadow/backend/llvm/llvm_backend.h stands in for the LLVM
# backend's header so that the factory's default backend is the GB300 one.
#
# Usage: build_with_reference.sh [REFERENCE_CHECKOUT]
#   (default: $SIMIT_REFERENCE, else `reference` beside the repository)
# Output: _ref/ in this directory (objects and the isprings_main binary).
set -e
HERE=$(cd "$(dirname "$0")" && pwd)
REPO=$(cd "$HERE/../../.." && pwd)
REF=${1:-${SIMIT_REFERENCE:-$(dirname "$REPO")/reference}}
SRC="$REF/src"
OUT="$HERE/_ref"
CUDA=${CUDA_HOME:-/usr/local/cuda}
[ -f "$SRC/backend/backend_function.h" ] || { echo "no reference sources at $SRC" >&2; exit 2; }
mkdir -p "$OUT/obj"
INC="-iquote $HERE/shadow -I$SRC -I$HERE -I$CUDA/include"
CXX="g++ -std=c++14 -O1 -w"
for f in "$SRC"/*.cpp "$SRC"/frontend/*.cpp "$SRC"/lower/*.cpp \
         "$SRC"/lower/index_expressions/*.cpp "$SRC"/util/*.cpp "$SRC"/backend/*.cpp; do
  rel=${f#"$SRC"/}
  o="$OUT/obj/$(echo "$rel" | tr / _ | sed 's/\.cpp$/.o/')"
  if [ ! "$o" -nt "$f" ] || [ "$HERE/shadow/backend/llvm/llvm_backend.h" -nt "$o" ]; then
    echo "$CXX $INC -c $f -o $o"
  fi
done | xargs -P "${JOBS:-$(nproc)}" -I{} sh -c "{}"
$CXX $INC -c "$HERE/gb300_backend.cpp" -o "$OUT/gb300_backend.o"
$CXX $INC "$HERE/isprings_main.cpp" "$OUT/gb300_backend.o" "$OUT"/obj/*.o \
    -L"$REPO/simit_gb300" -lsimit_gb300 -L"$CUDA/lib64" -lcudart \
    -Wl,-rpath,"$REPO/simit_gb300" -o "$OUT/isprings_main"
echo "$OUT/isprings_main"
