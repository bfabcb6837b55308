#!/bin/sh
# Builds oracle/_ref/libpwmref.so from the UNMODIFIED reference headers where they
# lie (default /root/reference), plus oracle/ref_harness.cpp and the boost shims in
# oracle/ref_shim, and oracle/_ref/calc_stats from Util_Scripts/calc_stats.cpp
# (unmodified, wrapped by oracle/ref_stats_main.cpp).  Test infrastructure only; outputs go to oracle/_ref/ (git-ignored).
# The reference's own build system (dpcpp/icx, Boost.Test, oneTBB) is not used:
# -DNTBB drops the TBB paths and the shims stand in for the three Boost headers.
set -e
HERE=$(cd "$(dirname "$0")" && pwd)
REF=${PWM_REFERENCE_DIR:-/root/reference}
[ -d "$REF/Matrix" ] || { echo "reference tree not found at $REF" >&2; exit 1; }
mkdir -p "$HERE/_ref"
g++ -std=c++17 -O2 -fopenmp -ffp-contract=off -DNTBB -DNDEBUG -fPIC -shared \
    -I"$HERE/ref_shim" -I"$REF" -include cstring -include climits \
    -o "$HERE/_ref/libpwmref.so" "$HERE/ref_harness.cpp"
echo "built $HERE/_ref/libpwmref.so"
g++ -std=c++17 -O2 -ffp-contract=off -DNTBB -DNDEBUG \
    -I"$HERE/ref_shim" -I"$REF" -include cstring -include climits \
    -o "$HERE/_ref/calc_stats" "$HERE/ref_stats_main.cpp"
echo "built $HERE/_ref/calc_stats"
