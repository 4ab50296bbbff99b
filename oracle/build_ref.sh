#!/usr/bin/env bash
# Builds the REFERENCE library from its own sources (read in place, never copied) together with
# oracle/ref_harness.cpp into oracle/_ref/ (git-ignored).  Test infrastructure only.
#
#   libvxref.so      serial build: the parity authority
#   libvxref_omp.so  -fopenmp -DUSE_OMP build: the reference's own multi-threaded CPU path
#
# Flags follow the reference makefile (-O3 -std=c++11) without -DPARDISO_5 (PARDISO is absent and
# off the time-step path) and with -ffp-contract=off so no platform contracts a*b+c into an FMA.
# The shipped lib/libvoxelyze.0.9.a is never used.
#
# Usage: build_ref.sh REFERENCE_ROOT   (the checkout holding the reference's include/ and src/)
set -euo pipefail
if [ $# -lt 1 ]; then
  echo "usage: $0 REFERENCE_ROOT" >&2
  exit 2
fi
REF=$1
HERE=$(cd "$(dirname "$0")" && pwd)
OUT="$HERE/_ref"
if [ ! -d "$REF/src" ]; then
  echo "reference sources not present at $REF; skipping" >&2
  exit 0
fi
mkdir -p "$OUT"
SRCS=""
for f in Voxelyze VX_Voxel VX_External VX_Link VX_Material VX_MaterialVoxel VX_MaterialLink \
         VX_Collision VX_LinearSolver VX_MeshRender; do
  SRCS="$SRCS $REF/src/$f.cpp"
done
FLAGS="-O3 -std=c++11 -ffp-contract=off -fPIC -shared -w -I$REF/include -I$HERE"
g++ $FLAGS $SRCS "$HERE/ref_harness.cpp" -o "$OUT/libvxref.so" &
g++ $FLAGS -fopenmp -DUSE_OMP $SRCS "$HERE/ref_harness.cpp" -o "$OUT/libvxref_omp.so" &
wait
echo "built $OUT/libvxref.so $OUT/libvxref_omp.so"
