#!/bin/sh
# Builds the C restatement oracle (test infrastructure only) into
# oracle/_build/libek_oracle.so (and its op-counting build), and, when the reference sources are present,
# the reference harness into oracle/_ref/ (see Makefile.ref) when EK_REFERENCE
# names the reference's source tree.
set -e
here=$(cd "$(dirname "$0")" && pwd)
mkdir -p "$here/_build"
${CC:-gcc} -std=c99 -O2 -ffp-contract=off -fopenmp -fPIC -shared \
  -o "$here/_build/libek_oracle.so" "$here/ek_oracle.c" -lm
# the op-counting build of the same restatement (FLOPs per cell-update)
${CXX:-g++} -std=gnu++20 -O2 -ffp-contract=off -fPIC -shared -fpermissive -Wno-unknown-pragmas \
  -o "$here/_build/libek_oracle_ops.so" "$here/ek_opcount.cpp" -lm
# the reference harness: only where EK_REFERENCE names the reference's source tree
if [ -n "${EK_REFERENCE:-}" ] && [ -d "${EK_REFERENCE}/src" ] && [ "${EK_SKIP_REF:-0}" = "0" ]; then
  make -s -C "$here" -f Makefile.ref REF="${EK_REFERENCE}" all
  # where the harness came from, for the tests that build more of the reference
  printf '%s\n' "${EK_REFERENCE}" > "$here/_ref/reference_path"
fi
