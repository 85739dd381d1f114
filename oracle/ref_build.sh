#!/bin/bash
# Builds the reference's own generic NLM kernels as sm_103a cubins into oracle/_ref/,
# from the sources where they lie (no copies): each configuration gets a directory of
# symlinks to the reference's main.cu / main.h / cuda_utility.h next to a config.h with
# that configuration's values, which is how the reference itself is configured
# (3DNLM/run.sh:13-19 rewrites config.h).  Only device code is built (-cubin); the
# cubins are test infrastructure, loaded by tests/golden/make_ref_golden.py.
#
# At NS=3 the reference's host launcher names shift kernels that exist only for
# NS=5..17 (3DNLM/main.cu:7644-7666 vs the #if NS== blocks); -D aliases point those
# names at the generic kernel so the file compiles; only the generic kernel is launched.
# With --if-present the script exits quietly when the sources are not there (the
# cubins then come from an earlier build, or the tests that need them skip).
set -euo pipefail
# The reference checkout: $REF, else a directory named "reference" beside the repository.
REF=${REF:-$(cd "$(dirname "$0")/../.." && pwd)/reference}
if [ "${1:-}" = "--if-present" ] && [ ! -d "$REF/3DNLM" ]; then exit 0; fi
HERE="$(cd "$(dirname "$0")" && pwd)"
OUT="$HERE/_ref"
NVCC=${NVCC:-nvcc}
ARCH="-arch=sm_103a"
[ -d "$REF/3DNLM" ] || { echo "reference sources not found at $REF" >&2; exit 1; }
mkdir -p "$OUT"

build3d() {  # SS NS X Y DEPTH
    local ss=$1 ns=$2 x=$3 y=$4 d=$5
    local name="ref3d_ss${ss}_ns${ns}_x${x}_y${y}_d${d}"
    local dir="$OUT/src_$name"
    mkdir -p "$dir"
    for f in main.cu main.h cuda_utility.h; do ln -sf "$REF/3DNLM/$f" "$dir/$f"; done
    cat > "$dir/config.h" <<CFG
#ifndef CONFIG_H
#define CONFIG_H
#define SS $ss
#define NS $ns
#define IMAGE_SIZE_X $x
#define IMAGE_SIZE_Y $y
#define depth $d
#endif
CFG
    local alias=""
    if [ "$ns" -lt 5 ]; then
        alias="-DNLmeansOnGPU_shift_1=shuffle_without_optimization -DNLmeansOnGPU_shift_2=shuffle_without_optimization -DNLmeansOnGPU_shift_3=shuffle_without_optimization"
    fi
    $NVCC $ARCH -O3 -cubin $alias -I"$dir" -o "$OUT/$name.cubin" "$dir/main.cu"
    echo "$OUT/$name.cubin"
}

build2d() {
    local dir="$OUT/src_ref2d"
    mkdir -p "$dir"
    for f in main.cu main.h cuda_utility.h; do ln -sf "$REF/2D NLM/11x11/$f" "$dir/$f"; done
    $NVCC $ARCH -O3 -cubin -I"$dir" -o "$OUT/ref2d.cubin" "$dir/main.cu"
    echo "$OUT/ref2d.cubin"
}

# Golden sizes keep reads inside the padded buffers: X a multiple of 33-NS, Y a
# multiple of 64 (16 blocks x 4 rows; Y = 128 exercises the y slide), depth a
# multiple of 8; 2D: X = Y a multiple of both 22 and 64.  The 256^3 build is timed
# only; its reads run past row ends, which the timing test covers with slack.
build3d 7 3 120 128 16
build3d 7 5 112 128 16
# large-patch golden sizes (X a multiple of 33-NS): search 11 / patch 13, search 13 / patch 17
build3d 11 13 120 128 8
build3d 13 17 128 128 8
# timing only (the 256^3 search-7 / patch-3 workload at the reference's own sizes)
build3d 7 3 256 256 256 &
build2d &
# timing only: the reference's large-patch sweep, search 11/13 x patch 13/15/17 on
# 512 x 512 slices of depth 16/32/64/128 (3DNLM/run.sh:25-34)
for ss in 11 13; do
    for ns in 13 15 17; do
        for d in 16 32 64 128; do
            build3d $ss $ns 512 512 $d &
        done
        wait
    done
done
wait
