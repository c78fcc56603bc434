#!/usr/bin/env bash
# Builds oracle/_ref/libcdmf_ref.so from the reference's own CPU sources,
# unmodified, where they lie: the first argument, else $CDMF_REFERENCE, else
# a checkout named `reference` beside this repository.  Test infrastructure
# only; the output stays out of git.
# Flags follow the reference's CMakeLists.txt:15-17 (-DVALUE_TYPE=float, C++14,
# OpenMP); -O2 is added and changes no result on x86-64 (no FMA in the
# baseline ISA, no fast-math).
set -euo pipefail
HERE="$(cd "$(dirname "$0")" && pwd)"
REF="${1:-${CDMF_REFERENCE:-$HERE/../../reference}}"
if [ ! -f "$REF/src/cdmf_ref.cpp" ]; then
    echo "build_ref.sh: reference sources not found under $REF; skipping" >&2
    exit 0
fi
mkdir -p "$HERE/_ref"
g++ -std=c++14 -O2 -fopenmp -fPIC -shared -DVALUE_TYPE=float -w \
    -I "$HERE/ref_stub" -I "$REF/src" \
    "$REF/src/cdmf_ref.cpp" "$REF/src/tools.cpp" "$HERE/ref_driver.cpp" \
    -o "$HERE/_ref/libcdmf_ref.so"
echo "built $HERE/_ref/libcdmf_ref.so"
