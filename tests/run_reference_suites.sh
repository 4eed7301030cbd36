#!/usr/bin/env bash
# run_reference_suites.sh — the reference's own test suites, unchanged,
# against this engine (the drop-in check; needs a CUDA device):
#   * core/tests/test_main.cpp, compiled against this engine's C++ headers
#     (ultrasound-engine_gb300/host/usx/*.hpp) and linked with libusx.so;
#   * tests/test_usx.py, run by pytest with this engine's `usx` package first
#     on the path.
# The reference's files are read where they lie and never copied into the
# repository.
#
# Usage: tests/run_reference_suites.sh [reference_dir] [work_dir]
#   reference_dir: the checkout (or a directory holding its core/tests and
#                  tests folders); else $USX_REFERENCE_DIR, else the location
#                  this container mounts it at.
#   work_dir:      where the compiled C++ suite and the logs go (default: a
#                  temporary directory).
# Exit status: 0 when both suites pass.
set -uo pipefail
HERE="$(cd "$(dirname "$0")" && pwd)"
ROOT="$(cd "$HERE/.." && pwd)"
REF="${1:-${USX_REFERENCE_DIR:-/root/reference}}"
WORK="${2:-$(mktemp -d)}"
PKG="$ROOT/ultrasound-engine_gb300"
mkdir -p "$WORK"
WORK="$(cd "$WORK" && pwd)"
REF="$(cd "$REF" 2>/dev/null && pwd || echo "$REF")"
if [ ! -f "$REF/core/tests/test_main.cpp" ] || [ ! -f "$REF/tests/test_usx.py" ]; then
  echo "reference suites not found under $REF" >&2
  exit 3
fi
if [ ! -f "$PKG/lib/libusx.so" ]; then
  python "$PKG/build.py" --no-oracle >/dev/null || exit 1
fi

CUDA_HOME="${CUDA_HOME:-/usr/local/cuda}"
g++ -std=c++17 -O2 -I "$PKG/host" -I "$ROOT/include" -I "$CUDA_HOME/include" \
    "$REF/core/tests/test_main.cpp" -L "$PKG/lib" -lusx -lusx_cu -Wl,-rpath,"$PKG/lib" \
    -o "$WORK/usx_tests" > "$WORK/cpp_build.log" 2>&1
rc_build=$?
rc_cpp=1
if [ $rc_build -eq 0 ]; then
  "$WORK/usx_tests" > "$WORK/cpp_suite.log" 2>&1
  rc_cpp=$?
fi
echo "C++ suite (core/tests/test_main.cpp): build rc=$rc_build run rc=$rc_cpp"
tail -3 "$WORK/cpp_suite.log" 2>/dev/null

# The Python suite from a scratch directory, so that pytest's rootdir and
# caches stay out of the reference checkout.
mkdir -p "$WORK/py"
( cd "$WORK/py" && PYTHONPATH="$PKG/python${PYTHONPATH:+:$PYTHONPATH}" \
    python -m pytest -q -p no:cacheprovider --rootdir "$WORK/py" "$REF/tests/test_usx.py" ) > "$WORK/py_suite.log" 2>&1
rc_py=$?
echo "Python suite (tests/test_usx.py): rc=$rc_py"
tail -3 "$WORK/py_suite.log"
exit $(( rc_build | rc_cpp | rc_py ))
