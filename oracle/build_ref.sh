#!/usr/bin/env bash
# Compile the reference's own FP64 CPU physical-optics path (PyPO
# src/CPU/InterfaceCPU.cpp + Propagation.h, src/common/InterfaceReflector.cpp
# for grid generation, src/common/InterfaceBeam.cpp for the Gaussian feed)
# straight from its sources with g++, into oracle/_ref/. Nothing is copied:
# the sources are read where they lie. The result is a pinning oracle for
# oracle/po_oracle.c and a CPU baseline; it is test infrastructure only.
#
# Usage: oracle/build_ref.sh [--where] [REFERENCE_ROOT]
#   REFERENCE_ROOT defaults to $PYPO_REFERENCE, else /root/reference.
#   Exits 3 when the sources are not there. --where prints the checkout's
#   root (tests that read the reference's own Python files use it) and exits.
set -euo pipefail
WHERE=0
if [ "${1:-}" = "--where" ]; then WHERE=1; shift; fi
REF="${1:-${PYPO_REFERENCE:-/root/reference}}"
HERE="$(cd "$(dirname "${BASH_SOURCE[0]}")" && pwd)"
OUT="$HERE/_ref"
if [ ! -f "$REF/src/CPU/InterfaceCPU.cpp" ]; then
    echo "build_ref: reference sources not found under $REF" >&2
    exit 3
fi
if [ "$WHERE" = 1 ]; then echo "$REF"; exit 0; fi
mkdir -p "$OUT"
g++ -O3 -std=c++17 -shared -fPIC -pthread \
    -I"$REF/src/include" -I"$REF/src/common" -I"$REF/src/CPU" \
    "$REF/src/CPU/InterfaceCPU.cpp" \
    "$REF/src/common/InterfaceReflector.cpp" \
    "$REF/src/common/InterfaceBeam.cpp" \
    -o "$OUT/libpypo_ref.so.tmp"
mv "$OUT/libpypo_ref.so.tmp" "$OUT/libpypo_ref.so"
echo "build_ref: wrote $OUT/libpypo_ref.so"
