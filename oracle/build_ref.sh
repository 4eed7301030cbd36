#!/usr/bin/env bash
# build_ref.sh — compile the reference engine's own core sources, read in place
# from the reference checkout (never copied), together with oracle/ref_shim.cpp
# into oracle/_ref/libusx_ref.so. Test infrastructure only: the library is the
# checker that pins the CPU oracle and generates golden fixtures; nothing in the
# product links it. Usage: oracle/build_ref.sh [reference_dir]
#
# Flags follow the reference's Release build (CMakeLists.txt: -O3, OpenMP, no
# -ffast-math, no -march) plus -ffp-contract=off so that a compiler which
# contracts by default (GCC on aarch64) keeps the reference's float arithmetic.
# The checkout is the first argument, else $USX_REFERENCE_DIR, else the
# location this container mounts it at; exit status 3 = no sources there.
set -euo pipefail
REF="${1:-${USX_REFERENCE_DIR:-/root/reference}}"
HERE="$(cd "$(dirname "$0")" && pwd)"
OUT="$HERE/_ref"
if [ ! -d "$REF/core/src" ]; then
  echo "reference sources not found at $REF; oracle/_ref not built" >&2
  exit 3
fi
mkdir -p "$OUT"
SRCS=(types geometry simulator demodulate beamformer doppler postprocess)
pids=()
for s in "${SRCS[@]}"; do
  g++ -std=c++17 -O3 -fPIC -fopenmp -ffp-contract=off -DNDEBUG -I"$REF/core/include" \
      -c "$REF/core/src/$s.cpp" -o "$OUT/$s.o" &
  pids+=($!)
done
g++ -std=c++17 -O3 -fPIC -fopenmp -ffp-contract=off -DNDEBUG -I"$REF/core/include" \
    -c "$HERE/ref_shim.cpp" -o "$OUT/ref_shim.o" &
pids+=($!)
for p in "${pids[@]}"; do wait "$p"; done
g++ -shared -fopenmp -o "$OUT/libusx_ref.so" "$OUT"/*.o
rm -f "$OUT"/*.o
echo "built $OUT/libusx_ref.so"
