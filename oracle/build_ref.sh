#!/bin/sh
# Builds oracle/_ref/libpwmref.so from the UNMODIFIED reference headers where they
# lie, plus oracle/ref_harness.cpp and the boost shims in oracle/ref_shim, and
# oracle/_ref/calc_stats from Util_Scripts/calc_stats.cpp (unmodified, wrapped by
# oracle/ref_stats_main.cpp).  Test infrastructure only; outputs go to oracle/_ref/
# (git-ignored).  The reference tree is taken from $PWM_REFERENCE_DIR, else from
# the development container's mount /root/reference; where neither exists (a GPU
# host) nothing is built and the script exits 0.  The tree it built from is
# recorded in oracle/_ref/reference_dir.txt for the tests that compile against it.
# The reference's own build system (dpcpp/icx, Boost.Test, oneTBB) is not used:
# -DNTBB drops the TBB paths and the shims stand in for the three Boost headers.
set -e
HERE=$(cd "$(dirname "$0")" && pwd)
REF=${PWM_REFERENCE_DIR:-/root/reference}
if [ ! -d "$REF/Matrix" ]; then
    echo "reference tree not found at $REF: oracle/_ref not built"
    exit 0
fi
mkdir -p "$HERE/_ref"
g++ -std=c++17 -O2 -fopenmp -ffp-contract=off -DNTBB -DNDEBUG -fPIC -shared \
    -I"$HERE/ref_shim" -I"$REF" -include cstring -include climits \
    -o "$HERE/_ref/libpwmref.so" "$HERE/ref_harness.cpp"
echo "built $HERE/_ref/libpwmref.so"
g++ -std=c++17 -O2 -ffp-contract=off -DNTBB -DNDEBUG \
    -I"$HERE/ref_shim" -I"$REF" -include cstring -include climits \
    -o "$HERE/_ref/calc_stats" "$HERE/ref_stats_main.cpp"
echo "built $HERE/_ref/calc_stats"
printf '%s\n' "$REF" > "$HERE/_ref/reference_dir.txt"
