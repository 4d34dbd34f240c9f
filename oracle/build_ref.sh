#!/usr/bin/env bash
# Builds oracle/_ref/libfreud_ref.so from the reference's own CPU sources, compiled
# in place from the read-only reference tree (nothing is copied into this repo),
# against the TBB-compatible shim and fsph stand-in under oracle/ref_shim/.
# Test infrastructure only (golden vectors + oracle pinning); never shipped.
#
# Flags: -O3 -ffp-contract=off, so the float32 arithmetic matches the reference's
# x86-64 Release build (which has no FMA contraction).
set -euo pipefail
HERE="$(cd "$(dirname "${BASH_SOURCE[0]}")" && pwd)"
REF="${FREUD_REFERENCE_DIR:-/root/reference}"
SRC="$REF/freud"
if [ ! -d "$SRC/locality" ]; then
    echo "reference sources not found under $REF; skipping oracle/_ref build" >&2
    exit 0
fi
OUT="$HERE/_ref"
mkdir -p "$OUT"
CXX="${CXX:-g++}"
FLAGS=(-O3 -ffp-contract=off -std=c++17 -fPIC -shared -w
       -I"$HERE/ref_shim" -I"$SRC/box" -I"$SRC/util" -I"$SRC/locality" -I"$SRC/density" -I"$SRC/pmft" -I"$SRC/order")
SOURCES=("$SRC/locality/LinkCell.cc" "$SRC/locality/AABBQuery.cc" "$SRC/locality/CellQuery.cc"
         "$SRC/locality/NeighborList.cc"
         "$SRC/locality/NeighborComputeFunctional.cc" "$SRC/density/RDF.cc"
         "$SRC/density/CorrelationFunction.cc" "$SRC/pmft/PMFTR12.cc" "$SRC/pmft/PMFTXYT.cc"
         "$SRC/pmft/PMFTXY.cc" "$SRC/pmft/PMFTXYZ.cc" "$SRC/order/Steinhardt.cc"
         "$SRC/order/Wigner3j.cc" "$HERE/ref_harness.cpp")
OBJS=()
for s in "${SOURCES[@]}"; do
    o="$OUT/$(basename "$s").o"
    if [ ! -f "$o" ] || [ "$s" -nt "$o" ]; then
        "$CXX" "${FLAGS[@]}" -c "$s" -o "$o" &
    fi
    OBJS+=("$o")
done
wait
"$CXX" -shared -o "$OUT/libfreud_ref.so" "${OBJS[@]}" -lpthread
echo "built $OUT/libfreud_ref.so"
