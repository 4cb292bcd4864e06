#!/usr/bin/env bash
# Recipe for oracle/_ref/: builds the reference's OWN hot-path translation units into shared
# libraries used as the parity pin of the C port (oracle/sph_oracle.c) and, where available, as
# the CPU baseline.  Test infrastructure only; nothing here is part of the product.
#
#   SPHCODE_REFERENCE=<checkout> oracle/build_ref.sh
#                                  build from the reference checkout at <checkout> (required)
#
# The reference fixes DIM with `#define DIM 1` (include/defines.hpp:5) and resolves quoted
# includes next to each header, so per-DIM copies of include/ with that one line changed are
# written to oracle/_ref/d{1,2,3}/include; the .cpp files are compiled where they lie.  Solver,
# Output and Logger need Boost (absent here) and are not built; oracle/ref_harness.cpp restates
# their glue.  GCC 13 needs `-include limits -include string` for headers the reference relies on
# transitively (src/bhtree.cpp:63, src/timestep.cpp:23, include/simulation.hpp:3-5).
#
# Two flavours per DIM:
#   libref_strict_dD.so : -O2 -fno-fast-math -ffp-contract=off  (parity pin)
#   libref_fast_dD.so   : -O3 -funroll-loops -ffast-math        (the reference Makefile's flags,
#                                                                 Makefile:4-10; timing)
# Where the sphgpu library is built (sphcode_gb300/_lib/libsphgpu.so, or $SPHGPU_LIB_DIR), a
# third flavour links the GPU Module drop-ins (sphcode_gb300/cxx/gpu_modules.cpp) in place of the
# reference's PreInteraction, FluidForce and GravityForce, with the reference's Simulation,
# TimeStep and tree sources and the same harness glue:
#   libref_gpu_dD.so    : ref_harness.cpp -DUSE_SPHGPU + gpu_modules.cpp + the strict objects
# Outputs go only to oracle/_ref/ (git-ignored).  A snapshot of the consumed reference sources is
# kept in oracle/_ref/snapshot/ so that the same recipe can rebuild them on a machine without the
# reference checkout (SPHCODE_REFERENCE pointing at the snapshot).
set -euo pipefail
HERE="$(cd "$(dirname "${BASH_SOURCE[0]}")" && pwd)"
ROOT="$(cd "$HERE/.." && pwd)"
GPU_LIB_DIR="${SPHGPU_LIB_DIR:-$ROOT/sphcode_gb300/_lib}"
if [ -z "${SPHCODE_REFERENCE:-}" ]; then
    echo "build_ref.sh: set SPHCODE_REFERENCE to the reference checkout (or its snapshot)" >&2
    exit 2
fi
REF="$SPHCODE_REFERENCE"
OUT="$HERE/_ref"
CXX="${CXX:-g++}"
JOBS="${JOBS:-$(nproc)}"

SRCS="src/simulation.cpp src/bhtree.cpp src/exhaustive_search.cpp src/pre_interaction.cpp
src/fluid_force.cpp src/gravity_force.cpp src/timestep.cpp src/disph/d_pre_interaction.cpp
src/disph/d_fluid_force.cpp src/gsph/g_pre_interaction.cpp src/gsph/g_fluid_force.cpp"

if [ ! -f "$REF/include/defines.hpp" ]; then
    echo "build_ref.sh: reference sources not found at $REF" >&2
    exit 3
fi

mkdir -p "$OUT"
# snapshot of the consumed sources (only when building from a real checkout)
if [ "$(cd "$REF" && pwd)" != "$OUT/snapshot" ]; then
    rm -rf "$OUT/snapshot"
    mkdir -p "$OUT/snapshot/src/disph" "$OUT/snapshot/src/gsph"
    cp -r "$REF/include" "$OUT/snapshot/include"
    for s in $SRCS; do cp "$REF/$s" "$OUT/snapshot/$s"; done
    # the sample parameter files (read by the parameter-reader tests)
    for j in "$REF"/sample/*/*.json; do
        d="$OUT/snapshot/sample/$(basename "$(dirname "$j")")"
        mkdir -p "$d"
        cp "$j" "$d/"
    done
    chmod -R u+w "$OUT/snapshot"
fi

COMMON="-std=gnu++14 -fPIC -fopenmp -include limits -include string -w"
STRICT="-O2 -fno-fast-math -ffp-contract=off"
FAST="-O3 -funroll-loops -ffast-math"

pids=()
run() {  # run a job with bounded parallelism
    "$@" &
    pids+=($!)
    if [ "${#pids[@]}" -ge "$JOBS" ]; then wait "${pids[0]}"; pids=("${pids[@]:1}"); fi
}

for D in 1 2 3; do
    INC="$OUT/d$D/include"
    rm -rf "$OUT/d$D"
    mkdir -p "$OUT/d$D"
    cp -r "$REF/include" "$INC"
    chmod -R u+w "$INC"
    sed -i "s/^#define DIM 1\$/#define DIM $D/" "$INC/defines.hpp"
    grep -q "^#define DIM $D\$" "$INC/defines.hpp" || { echo "DIM edit failed" >&2; exit 4; }
    for FL in strict fast; do
        FLAGS="$STRICT"; [ "$FL" = fast ] && FLAGS="$FAST"
        mkdir -p "$OUT/d$D/obj_$FL"
        for s in $SRCS; do
            o="$OUT/d$D/obj_$FL/$(basename "${s%.cpp}").o"
            run $CXX $COMMON $FLAGS -I"$INC" -c "$REF/$s" -o "$o"
        done
        run $CXX $COMMON $FLAGS -DDIM_FROM_HEADER -I"$INC" -I"$HERE" -c "$HERE/ref_harness.cpp" \
            -o "$OUT/d$D/obj_$FL/ref_harness.o"
    done
    if [ -f "$GPU_LIB_DIR/libsphgpu.so" ]; then
        mkdir -p "$OUT/d$D/obj_gpu"
        GINC="-I$INC -I$HERE -I$ROOT/include -I$ROOT/sphcode_gb300/cxx"
        run $CXX $COMMON $STRICT -DUSE_SPHGPU $GINC -c "$HERE/ref_harness.cpp" -o "$OUT/d$D/obj_gpu/ref_harness.o"
        run $CXX $COMMON $STRICT $GINC -c "$ROOT/sphcode_gb300/cxx/gpu_modules.cpp" -o "$OUT/d$D/obj_gpu/gpu_modules.o"
    fi
done
for p in "${pids[@]}"; do wait "$p"; done

for D in 1 2 3; do
    for FL in strict fast; do
        $CXX -shared -fopenmp -o "$OUT/libref_${FL}_d$D.so" "$OUT"/d$D/obj_$FL/*.o
    done
    if [ -f "$GPU_LIB_DIR/libsphgpu.so" ]; then
        REFOBJ=$(ls "$OUT"/d$D/obj_strict/*.o | grep -v '/ref_harness.o$')
        $CXX -shared -fopenmp -o "$OUT/libref_gpu_d$D.so" $REFOBJ "$OUT"/d$D/obj_gpu/*.o \
            -L"$GPU_LIB_DIR" -lsphgpu -Wl,-rpath,"$GPU_LIB_DIR"
    fi
done
echo "build_ref.sh: built $(ls "$OUT"/libref_*.so | wc -l) libraries in $OUT"
