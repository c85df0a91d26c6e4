#!/bin/sh
# Builds the C restatement oracle (test infrastructure only) into
# oracle/_build/libek_oracle.so, and, when the reference sources are present,
# the reference harness into oracle/_ref/ (see Makefile.ref).
set -e
here=$(cd "$(dirname "$0")" && pwd)
mkdir -p "$here/_build"
${CC:-gcc} -std=c99 -O2 -ffp-contract=off -fopenmp -fPIC -shared \
  -o "$here/_build/libek_oracle.so" "$here/ek_oracle.c" -lm
if [ -d "${EK_REFERENCE:-/root/reference}/src" ] && [ "${EK_SKIP_REF:-0}" = "0" ]; then
  make -s -C "$here" -f Makefile.ref REF="${EK_REFERENCE:-/root/reference}" all
fi
