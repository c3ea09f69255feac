#!/bin/sh
# Compiles the reference's own CPU mesh collector, as archived by the reference
# (Slang-generated C++ of collectMeshFrontiers with the per-pair enclosure
# plane and its six call counters), from where it lies in the reference tree,
# with the reference CPU backend's flags (src/sand_atlas_dem/cpu.py:323-334).
# Output only into oracle/_ref/.  Used to pin the oracle restatement; absent on
# machines without the reference tree.
set -e
REF=${SAND_DEM_REFERENCE:-/root/reference}
SRC="$REF/evidence/hostun424-cpu-pair-plane-counts-v1/native-profile-pair_plane_serial/instrumented-collector.cpp"
HERE=$(cd "$(dirname "$0")" && pwd)
if [ ! -f "$SRC" ]; then
    echo "reference collector source not present: $SRC" >&2
    exit 3
fi
mkdir -p "$HERE/_ref"
${CXX:-g++} -std=c++17 -O3 -fno-fast-math -ffp-contract=off -shared -fPIC -pthread -w \
    "$SRC" -o "$HERE/_ref/collector_ref.so"
echo "$HERE/_ref/collector_ref.so"
