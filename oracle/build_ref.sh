#!/usr/bin/env bash
# Builds oracle/_ref/libb3ref.so from the REFERENCE's CPU sources, compiled in place (nothing
# is copied into this repository), plus oracle/ref_shim.cpp.  Test infrastructure only: the
# library generates the golden vectors under tests/golden/ and pins the plain-C oracle.
#
# Usage: oracle/build_ref.sh <reference_root>   (or set B3G_REFERENCE_ROOT)
# Needs only g++; does not run the reference's own build system.  The OpenCL host files are
# compiled with -DB3_USE_CLEW against the vendored clew loader; no OpenCL runtime is needed
# because only the CPU entry points are called.
set -euo pipefail
REF=${1:-${B3G_REFERENCE_ROOT:-}}
if [ -z "$REF" ]; then
  echo "usage: $0 <reference_root> (or set B3G_REFERENCE_ROOT)" >&2
  exit 2
fi
HERE="$(cd "$(dirname "$0")" && pwd)"
OUT="$HERE/_ref"
SRC="$REF/src"
if [ ! -d "$SRC/Bullet3Common" ]; then
  echo "reference sources not found under $SRC" >&2
  exit 2
fi
mkdir -p "$OUT/obj"
CXXFLAGS="-O2 -fPIC -w -I$SRC -I$SRC/clew -DB3_USE_CLEW"
mapfile -t SRCS < <(cd "$SRC" && ls Bullet3Common/*.cpp Bullet3Geometry/*.cpp \
  Bullet3Collision/BroadPhaseCollision/*.cpp Bullet3Collision/NarrowPhaseCollision/*.cpp \
  Bullet3Dynamics/*.cpp Bullet3Dynamics/ConstraintSolver/*.cpp \
  Bullet3OpenCL/NarrowphaseCollision/*.cpp Bullet3OpenCL/ParallelPrimitives/*.cpp \
  Bullet3OpenCL/Initialize/*.cpp Bullet3OpenCL/BroadphaseCollision/*.cpp Bullet3OpenCL/RigidBody/*.cpp \
  Bullet3OpenCL/Raycast/*.cpp 2>/dev/null)
OBJS=()
pids=()
for s in "${SRCS[@]}"; do
  o="$OUT/obj/$(echo "$s" | tr '/' '_').o"
  OBJS+=("$o")
  if [ ! -f "$o" ] || [ "$SRC/$s" -nt "$o" ]; then
    g++ $CXXFLAGS -c "$SRC/$s" -o "$o" &
    pids+=($!)
    if [ ${#pids[@]} -ge 8 ]; then wait "${pids[0]}"; pids=("${pids[@]:1}"); fi
  fi
done
wait
gcc -O2 -fPIC -w -I"$SRC/clew" -c "$SRC/clew/clew.c" -o "$OUT/obj/clew.o"
g++ $CXXFLAGS -c "$HERE/ref_shim.cpp" -o "$OUT/obj/ref_shim.o"
g++ -shared -o "$OUT/libb3ref.so" "${OBJS[@]}" "$OUT/obj/clew.o" "$OUT/obj/ref_shim.o" -ldl -lpthread
echo "built $OUT/libb3ref.so"
