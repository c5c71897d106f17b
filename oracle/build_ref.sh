#!/usr/bin/env bash
# Compile the reference's own CPU programs for the FDK and Monte Carlo hot
# paths, unmodified, from their sources under the reference tree, into
# oracle/_ref/.  Used only to generate and re-check the golden fixtures in
# tests/golden/; nothing here is shipped or timed as product.
#
#   recon/bp3d20.cpp        FDK, 65x65 detector       -> oracle/_ref/bp3d20
#   recon/bp3d20_325.cpp    FDK, 325x325 detector     -> oracle/_ref/bp3d20_325
#   recon/fbp2.cpp          2-D fan-beam FBP          -> oracle/_ref/fbp2
#   monte_cpp/CBCT_real2.cpp CPU Monte Carlo (FP64)    -> oracle/_ref/CBCT_real2
#   monte_cpp/make_image01.cpp sphere label volume     -> oracle/_ref/make_image01
#
# FORTIFY is switched off because the programs sprintf into buffers that
# are too small (recon/bp3d20.cpp:10,170; recon/fbp2.cpp:9-11,153;
# monte_cpp/CBCT_real2.cpp:16,614);
# with FORTIFY the default Ubuntu build aborts after computing.
set -euo pipefail
HERE=$(cd "$(dirname "$0")" && pwd)
# the reference tree: MONTE_REFERENCE, else a "reference" directory beside
# the repository
REF=${MONTE_REFERENCE:-$(dirname "$(dirname "$HERE")")/reference}
OUT="$HERE/_ref"
if [ ! -d "$REF/recon" ]; then
  echo "reference tree not found at $REF; nothing to build" >&2
  exit 0
fi
mkdir -p "$OUT"
CXXFLAGS="-O2 -U_FORTIFY_SOURCE -D_FORTIFY_SOURCE=0 -w"
g++ $CXXFLAGS -o "$OUT/bp3d20"      "$REF/recon/bp3d20.cpp"
g++ $CXXFLAGS -o "$OUT/bp3d20_325"  "$REF/recon/bp3d20_325.cpp"
g++ $CXXFLAGS -o "$OUT/fbp2"        "$REF/recon/fbp2.cpp"
g++ $CXXFLAGS -I "$HERE/ref_shim" -I "$REF/monte_cpp" -o "$OUT/CBCT_real2" "$REF/monte_cpp/CBCT_real2.cpp"
g++ $CXXFLAGS -o "$OUT/make_image01" "$REF/monte_cpp/make_image01.cpp"
echo "built reference programs into $OUT"
