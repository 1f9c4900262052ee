#!/usr/bin/env bash
# Test infrastructure only. Compiles the REFERENCE's own LocARNA sources (read
# in place, never copied) into oracle/_ref/ together with the project-written
# ViennaRNA stub headers (oracle/stub/) and link stubs (oracle/ref_link_stubs.cc).
# Outputs: oracle/_ref/locarna, oracle/_ref/locarna_p, oracle/_ref/ref_harness.
# The reference needs autotools + ViennaRNA for its own build; neither is used.
# Folding code (rna_ensemble.cc, mcc_matrices.cc, exact_matcher.cc) is left out:
# PP inputs carry base-pair probabilities, so folding is never reached.
set -euo pipefail
HERE=$(cd "$(dirname "$0")" && pwd)
# the reference tree: $LOCARNA_REF, else a checkout named "reference" beside
# the repository
REF=${LOCARNA_REF:-$(cd "$HERE/../.." && pwd)/reference}
OUT=$HERE/_ref
SRC=$REF/src
if [ ! -d "$SRC/LocARNA" ]; then
  echo "build_ref: reference sources not found at $REF" >&2
  exit 3
fi
mkdir -p "$OUT/obj" "$OUT/gen/LocARNA"
CXX=${CXX:-g++}
# -ffp-contract=off: no FMA contraction on any host, so the floating-point
# envelope is the same sequence of IEEE operations as an x86 build.
FLAGS="-std=c++17 -O2 -DNDEBUG -DHAVE_CONFIG_H -ffp-contract=off -w"
INC="-I$HERE/stub -I$OUT/gen -I$SRC -I$SRC/LocARNA"
pids=()
for f in "$SRC"/LocARNA/*.cc; do
  b=$(basename "$f" .cc)
  case $b in exact_matcher|mcc_matrices|rna_ensemble) continue;; esac
  if [ ! -f "$OUT/obj/$b.o" ] || [ "$f" -nt "$OUT/obj/$b.o" ]; then
    $CXX $FLAGS $INC -c "$f" -o "$OUT/obj/$b.o" & pids+=($!)
  fi
done
$CXX $FLAGS $INC -c "$HERE/ref_link_stubs.cc" -o "$OUT/obj/ref_link_stubs.o" & pids+=($!)
for p in "${pids[@]}"; do wait "$p"; done
# RIBOSUM85_60 built-in matrix, generated the way the reference's build does it
$CXX $FLAGS $INC "$SRC/ribosum2cc.cc" "$OUT/obj/ribosum.o" "$OUT/obj/aux.o" -o "$OUT/ribosum2cc"
"$OUT/ribosum2cc" Ribosum85_60 "$REF/Data/Matrices/RIBOSUM85_60" "$OUT/gen/LocARNA/ribosum85_60.icc"
$CXX $FLAGS $INC "$SRC/locarna.cc" "$OUT"/obj/*.o -lquadmath -o "$OUT/locarna" &
$CXX $FLAGS $INC "$SRC/locarna_p.cc" "$OUT"/obj/*.o -lquadmath -o "$OUT/locarna_p" &
$CXX $FLAGS $INC "$HERE/ref_harness.cc" "$OUT"/obj/*.o -lquadmath -o "$OUT/ref_harness" &
$CXX $FLAGS $INC "$HERE/ref_harness_p.cc" "$OUT"/obj/*.o -lquadmath -o "$OUT/ref_harness_p" &
wait
echo "build_ref: ok ($OUT)"
