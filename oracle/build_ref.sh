#!/bin/sh
# TEST INFRASTRUCTURE.  Compiles the reference's own src/kgraph.cpp (through
# ref_harness.cpp) and src/metric.cpp, read in place from the reference tree,
# with the self-written Boost-subset shim under oracle/compat, into
# oracle/_ref/libkcna_ref.so, and its src/fvec2lshit.cpp into
# oracle/_ref/fvec2lshit.  Flags follow the reference's CMakeLists.txt:8
# (-O3 -std=c++11 -DDEBUG -DNSG + OpenMP); on x86-64 the AVX distance path is
# enabled with -mavx2 -mfma in place of -march=native.
set -e
HERE=$(cd "$(dirname "$0")" && pwd)
SRC=${KCNA_REF_SRC:-/root/reference/src}
if [ ! -f "$SRC/kgraph.cpp" ]; then
    echo "build_ref.sh: reference sources not found at $SRC" >&2
    exit 2
fi
mkdir -p "$HERE/_ref"
FLAGS="-O3 -std=c++11 -DDEBUG -DNSG -fopenmp -fPIC -w"
case "$(uname -m)" in x86_64) FLAGS="$FLAGS -mavx2 -mfma" ;; esac
g++ $FLAGS -I"$HERE/compat" -I"$SRC" -I"$HERE/../include" -shared \
    -o "$HERE/_ref/libkcna_ref.so" "$HERE/ref_harness.cpp" "$SRC/metric.cpp"
echo "built $HERE/_ref/libkcna_ref.so"
# the reference's fvecs -> lshkit converter, src/fvec2lshit.cpp, as is
g++ -O2 -w -I"$HERE/compat" -o "$HERE/_ref/fvec2lshit" "$SRC/fvec2lshit.cpp"
echo "built $HERE/_ref/fvec2lshit"
