#!/usr/bin/env bash
# Build the golden-vector harness from the reference's own C++ sources.
#
# TEST INFRASTRUCTURE ONLY.  The reference is compiled where it lies (nothing
# is copied into this repository); objects and the harness binary go to
# oracle/_ref/, which is git-ignored.  MPI is replaced by the single-rank stub
# oracle/ref/mpi.h, and the reference's `main` (src/TDVMC.cpp) is renamed so
# that oracle/ref/harness.cpp provides the entry point.
#
# Usage: oracle/ref/build_ref.sh [reference-root]   (default /root/reference)
set -euo pipefail
HERE="$(cd "$(dirname "${BASH_SOURCE[0]}")" && pwd)"
REF="${1:-/root/reference}"
OUT="$HERE/../_ref"
OBJ="$OUT/obj"
if [ ! -d "$REF/src" ]; then
  echo "reference sources not found at $REF" >&2
  exit 1
fi
mkdir -p "$OBJ"
CXX="${CXX:-g++}"
FLAGS="-std=c++17 -O3 -w -I$HERE -I$REF/src -I$REF/resources"

SRCS=$(cd "$REF" && ls src/*.cpp src/*/*.cpp resources/jsoncpp.cpp)
compile_one() {
  local src="$1"
  local obj="$OBJ/$(echo "$src" | tr '/' '_' | sed 's/\.cpp$/.o/')"
  local extra=""
  if [ "$src" = "src/TDVMC.cpp" ]; then extra="-Dmain=tdvmc_reference_main"; fi
  if [ ! -f "$obj" ] || [ "$REF/$src" -nt "$obj" ] || [ "$HERE/mpi.h" -nt "$obj" ]; then
    $CXX $FLAGS $extra -c "$REF/$src" -o "$obj"
  fi
}
export -f compile_one
export CXX FLAGS OBJ REF HERE
echo "$SRCS" | xargs -P "$(nproc)" -I{} bash -c 'compile_one {}'
$CXX $FLAGS -c "$HERE/harness.cpp" -o "$OBJ/harness.o"
$CXX -o "$OUT/ref_harness" "$OBJ"/*.o
echo "built $OUT/ref_harness"
