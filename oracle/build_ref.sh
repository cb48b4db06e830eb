#!/bin/sh
# Test infrastructure: compile the unmodified reference C++ hot path (from the
# read-only reference checkout) plus oracle/ref_shim.cpp into
# oracle/_ref/libfsref.so, with the reference's own flags
# (-O3 -ffast-math -fopenmp; reference Makefile:10, setup.py:57).
# Usage: oracle/build_ref.sh [reference_root]
#   (default $FSG_REFERENCE_ROOT, else a "reference" directory beside this repository)
set -e
HERE0="$(cd "$(dirname "$0")" && pwd)"
REF="${1:-${FSG_REFERENCE_ROOT:-$HERE0/../../reference}}"
SRC="$REF/fake_spectra"
HERE="$(cd "$(dirname "$0")" && pwd)"
if [ ! -f "$SRC/part_int.cpp" ]; then
    echo "reference sources not found under $SRC" >&2
    exit 2
fi
mkdir -p "$HERE/_ref"
${CXX:-g++} -O3 -ffast-math -fopenmp -fPIC -shared -I"$SRC" \
    "$HERE/ref_shim.cpp" "$SRC/part_int.cpp" "$SRC/absorption.cpp" \
    "$SRC/index_table.cpp" "$SRC/Faddeeva.cpp" \
    -o "$HERE/_ref/libfsref.so.tmp"
mv "$HERE/_ref/libfsref.so.tmp" "$HERE/_ref/libfsref.so"
echo "built $HERE/_ref/libfsref.so"
