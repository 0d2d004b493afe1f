#!/usr/bin/env bash
# Builds oracle/_ref/ffr_ref and oracle/_ref/ffr_img_ref from the
# reference's own, unmodified sources where they lie (REF_ROOT, default
# /root/reference), plus the project's shims in oracle/shim (a JSON class
# standing in for the absent nlohmann/json, the parts of Boost.GIL and
# Boost.program_options the reference uses) and the drivers
# oracle/ref_driver.cpp and oracle/img_driver.cpp.
# Output goes only to oracle/_ref/ (git-ignored).  The reference's own CMake
# build is not used: it needs Boost.program_options, Boost.GIL and libpng,
# none of which is installed.  -ffp-contract=off keeps FP64 results
# identical between x86-64 and aarch64.
set -euo pipefail
HERE="$(cd "$(dirname "${BASH_SOURCE[0]}")" && pwd)"
REF_ROOT="${REF_ROOT:-/root/reference}"
if [ ! -d "$REF_ROOT/src" ]; then
    echo "build_ref.sh: reference sources not found at $REF_ROOT/src" >&2
    exit 1
fi
mkdir -p "$HERE/_ref"
# rebuild a binary only when a source it is built from (the reference's
# sources, the shims, the drivers, this script) is newer than it
stale() {
    local out="$1"
    [ ! -e "$out" ] && return 0
    [ -n "$(find "$REF_ROOT/src" "$HERE/shim" "$HERE/ref_driver.cpp" "$HERE/img_driver.cpp" \
            "${BASH_SOURCE[0]}" -newer "$out" -print -quit)" ]
}
if stale "$HERE/_ref/ffr_ref"; then
    g++ -std=c++23 -O3 -DNDEBUG -ffp-contract=off -w \
        -I "$HERE/shim" -I "$HERE/shim/nest/nest" -I "$REF_ROOT/src" \
        "$HERE/ref_driver.cpp" \
        "$REF_ROOT/src/rng/flame_rng.cpp" \
        "$REF_ROOT/src/utils/json.cpp" \
        -o "$HERE/_ref/ffr_ref" -lpthread
fi
# the reference's own ffr-img (src/ffr_img.cpp, unmodified) with the
# project's Boost.GIL / program_options shims and an unencoded image writer
# (oracle/img_driver.cpp) in place of libpng
if stale "$HERE/_ref/ffr_img_ref"; then
    g++ -std=c++23 -O2 -DNDEBUG -ffp-contract=off -w \
        -I "$HERE/shim" -I "$HERE/shim/nest/nest" -I "$REF_ROOT/src" \
        "$HERE/img_driver.cpp" \
        "$REF_ROOT/src/ffr_img.cpp" \
        "$REF_ROOT/src/rng/flame_rng.cpp" \
        "$REF_ROOT/src/utils/json.cpp" \
        -o "$HERE/_ref/ffr_img_ref" -lpthread
fi
