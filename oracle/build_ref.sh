#!/usr/bin/env bash
# Builds the reference's own scalar ray tracer from its sources into
# oracle/_ref/libprayref_<variant>.so, one library per set of compile-time
# constants. Test infrastructure only: the libraries pin the CPU restatement
# (pray_oracle.cpp) and generate tests/golden/ fixtures in a container that has
# the reference sources. The product never loads them.
#
# Parity build: default x86-64 target (neither __AVX__ nor __SSE3__, so
# include/options.h selects the plain scalar code), -ffp-contract=off (no FMA
# contraction), -O2. The reference is compiled where it lies; constants that a
# workload changes (kd_tree.h THRESHOLD/MAX_DEPTH, kd_tree_sah.h traversalCost,
# geometry.h EPSILON) are patched into a temporary copy of its include/
# directory under /tmp, which is removed afterwards.
#
# Usage: oracle/build_ref.sh [variant ...]   (default: all variants)
set -euo pipefail
REF="${REF_ROOT:-/root/reference}"
HERE="$(cd "$(dirname "$0")" && pwd)"
OUT="$HERE/_ref"

if [ ! -d "$REF/src" ] || [ ! -d "$REF/include" ]; then
    echo "build_ref: reference sources not found at $REF; nothing built"
    exit 0
fi
if [ "$(uname -m)" != "x86_64" ]; then
    echo "build_ref: parity build expects an x86_64 host; nothing built"
    exit 0
fi
mkdir -p "$OUT"

# name leaf max_depth sah_traversal_cost det_epsilon
VARIANTS=(
    "default 32 20 5.f 1.e-4f"
    "leaf8 8 24 5.f 1.e-4f"
    "sahct1 32 20 1.f 1.e-4f"
    "sahct1_eps0 32 20 1.f 0.0f"
    "leaf8_eps0 8 24 5.f 0.0f"
)
# the reference's own optimised build (AVX packets, CMakeLists.txt:49 flags) for
# timing only, built when asked for by name: oracle/build_ref.sh avx_sahct1_eps0
TIMING_VARIANTS=(
    "avx_sahct1_eps0 32 20 1.f 0.0f -march=native -Ofast -fno-fast-math"
)

build_variant() {
    local name=$1 leaf=$2 depth=$3 ct=$4 eps=$5 flags=${6:-"-O2 -ffp-contract=off"}
    local lib="$OUT/libprayref_${name}.so"
    if [ -f "$lib" ] && [ "$lib" -nt "$HERE/ref_harness.cpp" ] && [ "$lib" -nt "$0" ]; then
        return 0
    fi
    local tmp
    tmp="$(mktemp -d /tmp/prayref_${name}_XXXXXX)"
    cp -r "$REF/include" "$tmp/include"
    sed -i "s/THRESHOLD = 32;/THRESHOLD = ${leaf};/; s/MAX_DEPTH = 20;/MAX_DEPTH = ${depth};/" "$tmp/include/kd_tree.h"
    sed -i "s/float traversalCost = 5.f;/float traversalCost = ${ct};/" "$tmp/include/kd_tree_sah.h"
    sed -i "s/EPSILON = 1.e-4f;/EPSILON = ${eps};/" "$tmp/include/geometry.h"
    grep -q "THRESHOLD = ${leaf};" "$tmp/include/kd_tree.h"
    grep -q "MAX_DEPTH = ${depth};" "$tmp/include/kd_tree.h"
    grep -q "traversalCost = ${ct};" "$tmp/include/kd_tree_sah.h"
    grep -q "EPSILON = ${eps};" "$tmp/include/geometry.h"
    g++ -std=c++14 $flags -fopenmp -fPIC -shared -w \
        -include limits -include fstream \
        -I"$tmp/include" -I"$REF/ext" \
        "$REF/src/kd_tree.cpp" "$REF/src/kd_tree_sah.cpp" "$REF/src/geometry.cpp" "$REF/src/geometry_simd.cpp" \
        "$REF/src/scene_preprocessor.cpp" "$REF/src/pray.cpp" "$REF/src/io.cpp" \
        "$HERE/ref_harness.cpp" -o "$lib.tmp" -lstdc++fs
    mv "$lib.tmp" "$lib"
    rm -rf "$tmp"
    echo "build_ref: built $lib"
}

want=("$@")
pids=()
for v in "${VARIANTS[@]}"; do
    set -- $v
    if [ ${#want[@]} -eq 0 ] || printf '%s\n' "${want[@]}" | grep -qx "$1"; then
        build_variant "$@" &
        pids+=($!)
    fi
done
for v in "${TIMING_VARIANTS[@]}"; do
    set -- $v
    if [ ${#want[@]} -gt 0 ] && printf '%s\n' "${want[@]}" | grep -qx "$1"; then
        build_variant "$1" "$2" "$3" "$4" "$5" "${*:6}" &
        pids+=($!)
    fi
done
rc=0
for p in "${pids[@]}"; do wait "$p" || rc=1; done
exit $rc
