#!/bin/sh
# Builds the unmodified Chipmunk2D reference, straight from its read-only
# source tree, into oracle/_ref/libcpref.so together with the state-export
# harness (oracle/ref_harness.c) and the seeded workloads
# (chipmunk2d_gb300/csrc/scenes.c).  Test infrastructure: only the tests and
# the CPU-baseline leg of bench.py load the result.
#
# Flags: the reference's own Release flags add -ffast-math, which makes its
# cpBodyGetType() test of idleTime == INFINITY unreliable (the pyramid scene
# spins forever under gcc 13), so this recipe builds with strict IEEE
# semantics and no FMA contraction (GNU C contracts by default on aarch64).
#
# Usage: oracle/build_ref.sh REFERENCE_ROOT
#    or: CHIPMUNK_REF_ROOT=... oracle/build_ref.sh
set -e
REF=${1:-$CHIPMUNK_REF_ROOT}
if [ -z "$REF" ]; then
	echo "usage: $0 REFERENCE_ROOT (or set CHIPMUNK_REF_ROOT)" >&2
	exit 2
fi
HERE=$(cd "$(dirname "$0")" && pwd)
REPO=$(cd "$HERE/.." && pwd)
OUT="$HERE/_ref"
if [ ! -d "$REF/src" ]; then
	echo "reference sources not found at $REF; skipping" >&2
	exit 0
fi
mkdir -p "$OUT/obj"
CFLAGS="-std=gnu99 -O2 -fPIC -ffp-contract=off -DNDEBUG -I$REF/include"
pids=""
for f in "$REF"/src/*.c; do
	b=$(basename "$f" .c)
	gcc $CFLAGS -c "$f" -o "$OUT/obj/$b.o" &
	pids="$pids $!"
done
gcc $CFLAGS -c "$HERE/ref_harness.c" -o "$OUT/obj/ref_harness.o" &
pids="$pids $!"
gcc -std=gnu99 -O2 -fPIC -ffp-contract=off -c "$REPO/chipmunk2d_gb300/csrc/scenes.c" -o "$OUT/obj/scenes.o" &
pids="$pids $!"
for p in $pids; do wait $p; done
gcc -shared -o "$OUT/libcpref.so" "$OUT"/obj/*.o -lm -lpthread
echo "$OUT/libcpref.so"
