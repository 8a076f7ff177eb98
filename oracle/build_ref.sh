#!/bin/sh
# TEST INFRASTRUCTURE.  Compiles the reference's own src/kgraph.cpp (through
# ref_harness.cpp) and src/metric.cpp, unmodified, with the self-written
# Boost-subset shim under oracle/compat, into oracle/_ref/libkcna_ref.so, and
# its src/fvec2lshit.cpp into oracle/_ref/fvec2lshit.  Flags follow the
# reference's CMakeLists.txt:8 (-O3 -std=c++11 -DDEBUG -DNSG + OpenMP,
# -march=native); on x86-64 the AVX distance path is enabled with -mavx2 -mfma
# in place of -march=native.  -ftrivial-auto-var-init=zero: src/kgraph.cpp:2207
# (findroot) reads a variable in its own initialiser (`unsigned id=nhoods[id]
# .pool[i].id;`, undefined behaviour that crashed with SIGSEGV on aarch64); the
# flag gives that read the value 0 (node 0's pool is scanned) on every machine,
# with the source unchanged.
#
# Where the sources are read from, in order:
#   1. $KCNA_REF_SRC;
#   2. /root/reference/src, the reference checkout, when this machine has one;
#   3. oracle/_ref/src, a staging copy of the six source files the build uses.
# When the sources come from 1 or 2, they are also staged into oracle/_ref/src
# (git-ignored, never committed) so that a machine without the reference
# checkout can compile the same sources for its own architecture.
# Exit status 2: no sources anywhere.
set -e
HERE=$(cd "$(dirname "$0")" && pwd)
STAGE="$HERE/_ref/src"
FILES="kgraph.cpp kgraph.h kgraph-data.h metric.cpp neighbor.h fvec2lshit.cpp"
SRC=${KCNA_REF_SRC:-}
if [ -z "$SRC" ] && [ -f /root/reference/src/kgraph.cpp ]; then SRC=/root/reference/src; fi
if [ -z "$SRC" ] && [ -f "$STAGE/kgraph.cpp" ]; then SRC="$STAGE"; fi
if [ -z "$SRC" ] || [ ! -f "$SRC/kgraph.cpp" ]; then
    echo "build_ref.sh: reference sources not found (KCNA_REF_SRC, /root/reference/src, $STAGE)" >&2
    exit 2
fi
mkdir -p "$HERE/_ref"
if [ "$SRC" != "$STAGE" ]; then
    mkdir -p "$STAGE"
    for f in $FILES; do cp "$SRC/$f" "$STAGE/$f"; chmod u+w "$STAGE/$f"; done
fi
FLAGS="-O3 -std=c++11 -DDEBUG -DNSG -fopenmp -fPIC -w -ftrivial-auto-var-init=zero"
case "$(uname -m)" in
    x86_64) FLAGS="$FLAGS -mavx2 -mfma" ;;
    *) if echo 'int main(){return 0;}' | g++ -march=native -x c++ -o /dev/null - 2>/dev/null; then
           FLAGS="$FLAGS -march=native"
       fi ;;
esac
g++ $FLAGS -I"$HERE/compat" -I"$SRC" -I"$HERE/../include" -shared \
    -rdynamic -o "$HERE/_ref/libkcna_ref.so" "$HERE/ref_harness.cpp" "$SRC/metric.cpp"
echo "built $HERE/_ref/libkcna_ref.so ($(uname -m), $FLAGS)"
# the reference's fvecs -> lshkit converter, src/fvec2lshit.cpp, as is
g++ -O2 -w -I"$HERE/compat" -o "$HERE/_ref/fvec2lshit" "$SRC/fvec2lshit.cpp"
echo "built $HERE/_ref/fvec2lshit"
