#!/usr/bin/env bash
# Builds oracle/_ref/libpointint_ref.so from the reference's own sources where
# they lie (default /root/reference, override with POINTINT_REF_DIR): the
# standalone-compilable element functions and the header-only quadrature,
# behind the C-ABI shim oracle/ref_shim.cpp.  Outputs go to oracle/_ref/ only.
# The rest of the reference path needs Eigen, TBB and libigl (absent), so it is
# not built; the oracle restates it instead.
set -euo pipefail
HERE="$(cd "$(dirname "$0")" && pwd)"
REF="${POINTINT_REF_DIR:-/root/reference}"
if [ ! -f "$REF/cpp/src/element_functions.cpp" ]; then
  echo "reference sources not found under $REF; skipping oracle/_ref" >&2
  exit 0
fi
mkdir -p "$HERE/_ref"
g++ -O2 -std=c++17 -fPIC -shared \
  -I"$REF/cpp/include" \
  "$REF/cpp/src/element_functions.cpp" "$HERE/ref_shim.cpp" \
  -o "$HERE/_ref/libpointint_ref.so"
echo "built $HERE/_ref/libpointint_ref.so"
