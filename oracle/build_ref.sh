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
# It also compiles the reference's GPU path tracer (src/path_trace.cu, device
# code only) into oracle/_ref/prayref_path_trace.cubin for sm_103a, and the
# reference-side binding (integration/gpu_kdtree.cpp)
# against the reference's own headers, once per instruction set the
# reference's include/options.h distinguishes (scalar, and on x86 also SSE3
# and AVX), into oracle/_ref/gpu_kdtree_<isa>.o, and records the reference's
# location in oracle/_ref/ref_root.txt for the tests that read its example
# scenes.
#
# The scalar build is portable C++ (include/options.h picks the plain code
# without __AVX__ / __SSE3__), so it is built on any host; only the AVX
# timing variant is x86-only.
#
# Usage: REF_ROOT=<reference checkout> oracle/build_ref.sh [variant ...]
#        (default: all parity variants)
set -euo pipefail
HERE="$(cd "$(dirname "$0")" && pwd)"
OUT="$HERE/_ref"
if [ -z "${REF_ROOT:-}" ]; then
    echo "build_ref: REF_ROOT is not set; nothing built"
    exit 0
fi
REF="$REF_ROOT"

if [ ! -d "$REF/src" ] || [ ! -d "$REF/include" ]; then
    echo "build_ref: reference sources not found at $REF; nothing built"
    exit 0
fi
mkdir -p "$OUT"
echo "$REF" > "$OUT/ref_root.txt"
ARCH="$(uname -m)"

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
        "$REF/src/scene_preprocessor.cpp" "$REF/src/pray.cpp" "$REF/src/io.cpp" "$REF/src/gpu_util.cpp" \
        "$HERE/ref_harness.cpp" -o "$lib.tmp" -lstdc++fs
    mv "$lib.tmp" "$lib"
    rm -rf "$tmp"
    echo "build_ref: built $lib"
}

build_binding() {
    local isa=$1 flags=$2
    local obj="$OUT/gpu_kdtree_${isa}.o"
    local src="$HERE/../integration/gpu_kdtree.cpp"
    if [ -f "$obj" ] && [ "$obj" -nt "$src" ] && [ "$obj" -nt "$HERE/../integration/gpu_kdtree.h" ] &&
       [ "$obj" -nt "$HERE/../include/nostrum_pray.h" ]; then
        return 0
    fi
    g++ -std=c++14 $flags -O1 -fPIC -Wall -Wextra -Wno-reorder -include limits -include fstream \
        -I"$REF/include" -I"$REF/ext" -I"$HERE/../include" -c "$src" -o "$obj.tmp"
    mv "$obj.tmp" "$obj"
    echo "build_ref: built $obj"
}

# The reference's GPU path tracer (src/path_trace.cu) as an sm_103a cubin,
# device code only, for oracle/ref_gpu_launch.cpp to load and time.
build_cubin() {
    local cubin="$OUT/prayref_path_trace.cubin"
    command -v nvcc >/dev/null 2>&1 || return 0
    if [ -f "$cubin" ] && [ "$cubin" -nt "$0" ]; then
        return 0
    fi
    nvcc -cubin -gencode arch=compute_103a,code=sm_103a -O3 -std=c++14 -include limits -include fstream \
        -diag-suppress 20012,20013,20015 -I"$REF/include" -I"$REF/ext" -DWITH_CUDA \
        "$REF/src/path_trace.cu" -o "$cubin.tmp"
    mv "$cubin.tmp" "$cubin"
    echo "build_ref: built $cubin"
}

want=("$@")
pids=()
if [ ${#want[@]} -eq 0 ]; then
    build_cubin &
    pids+=($!)
    build_binding scalar "" &
    pids+=($!)
    if [ "$ARCH" = "x86_64" ]; then
        build_binding sse "-msse3" &
        pids+=($!)
        build_binding avx "-mavx" &
        pids+=($!)
    fi
fi
for v in "${VARIANTS[@]}"; do
    set -- $v
    if [ ${#want[@]} -eq 0 ] || printf '%s\n' "${want[@]}" | grep -qx "$1"; then
        build_variant "$@" &
        pids+=($!)
    fi
done
for v in "${TIMING_VARIANTS[@]}"; do
    set -- $v
    if [ "$ARCH" = "x86_64" ] && [ ${#want[@]} -gt 0 ] && printf '%s\n' "${want[@]}" | grep -qx "$1"; then
        build_variant "$1" "$2" "$3" "$4" "$5" "${*:6}" &
        pids+=($!)
    fi
done
rc=0
for p in "${pids[@]}"; do wait "$p" || rc=1; done
exit $rc
