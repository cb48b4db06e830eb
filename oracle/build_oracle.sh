#!/bin/sh
# Test infrastructure: build the C oracle (oracle/fsg_oracle.c) into
# oracle/_build/libfsgoracle.so.  FMA contraction is off so the reference's
# mixed float/double sightline predicate is reproduced on every host.
set -e
HERE="$(cd "$(dirname "$0")" && pwd)"
mkdir -p "$HERE/_build"
${CC:-gcc} -O2 -fopenmp -ffp-contract=off -fno-fast-math -fPIC -shared -std=c99 -Wall \
    "$HERE/fsg_oracle.c" -o "$HERE/_build/libfsgoracle.so.tmp" -lm
mv "$HERE/_build/libfsgoracle.so.tmp" "$HERE/_build/libfsgoracle.so"
echo "built $HERE/_build/libfsgoracle.so"
