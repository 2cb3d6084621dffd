#!/bin/sh
# Builds the CPU restatement (oracle/cp_oracle.c) and the seeded workloads
# (chipmunk2d_gb300/csrc/scenes.c) into oracle/_build/liboracle.so.
# Test infrastructure: loaded only by tests/, the smoke check and the
# CPU-baseline leg of bench.py.  Strict IEEE double arithmetic: no
# -ffast-math and no FMA contraction (GNU C contracts by default on aarch64).
set -e
HERE=$(cd "$(dirname "$0")" && pwd)
REPO=$(cd "$HERE/.." && pwd)
OUT="$HERE/_build"
mkdir -p "$OUT"
gcc -std=gnu11 -O2 -fPIC -ffp-contract=off -Wall -Wno-unused-function -shared \
	-o "$OUT/liboracle.so.tmp" "$HERE/cp_oracle.c" "$REPO/chipmunk2d_gb300/csrc/scenes.c" -lm -lpthread
mv "$OUT/liboracle.so.tmp" "$OUT/liboracle.so"
echo "$OUT/liboracle.so"
