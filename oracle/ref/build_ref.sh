#!/usr/bin/env bash
# Builds oracle/_ref/libhcref.so: the reference's own pointwise physics
# (fluxes, limiters, transforms, geometry, boundary conditions, RK tables, mesh
# generators) compiled from the headers where they lie in the reference tree,
# behind the extern "C" probe in ref_probe.cpp.  Test infrastructure only.
#
# The reference HEAD does not compile with g++ >= 10; four headers need a
# one-token fix each.  Patched copies of exactly those files are written to
# oracle/_ref/overlay/ (searched before the reference tree); nothing else is
# copied and the reference tree is never written to:
#   geometry/geometry.h:195            missing ';' after the declaration of norm
#   conservationLaws/base/fluxes/{centralFlux,rusanovFlux,roeFlux}.ipp
#                                      out-of-line definitions lack the class
#                                      template's 'requires ImplementedLawType<Law>'
# <iostream> is included by the probe before any reference header
# (utils/maths/affineSpace.ipp uses std::ostream without including it).
set -euo pipefail
REF=${HC_REFERENCE_ROOT:-/root/reference}
INC="$REF/cpp/inc"
HERE="$(cd "$(dirname "$0")" && pwd)"
OUT="$HERE/../_ref"
if [ ! -d "$INC" ]; then
  echo "reference tree not found at $INC; skipping oracle/_ref" >&2
  exit 0
fi
mkdir -p "$OUT/overlay/geometry" "$OUT/overlay/conservationLaws/base/fluxes"
sed '195s/^\(.*norm( const Direction<nDim,Real>& d )\)\s*$/\1;/' \
    "$INC/geometry/geometry.h" > "$OUT/overlay/geometry/geometry.h"
for f in centralFlux rusanovFlux roeFlux; do
  sed 's/^\(\s*template<LawType Law>\)\s*$/\1 requires ImplementedLawType<Law>/' \
      "$INC/conservationLaws/base/fluxes/$f.ipp" > "$OUT/overlay/conservationLaws/base/fluxes/$f.ipp"
done
grep -q 'norm( const Direction<nDim,Real>& d );' "$OUT/overlay/geometry/geometry.h"
${CXX:-g++} -std=c++2a -fconcepts-ts -O2 -ffp-contract=off -fno-fast-math -fPIC -shared \
    -w -I"$OUT/overlay" -I"$INC" -o "$OUT/libhcref.so" "$HERE/ref_probe.cpp"
echo "built $OUT/libhcref.so"
${CXX:-g++} -std=c++2a -fconcepts-ts -O2 -ffp-contract=off -fno-fast-math -fPIC -shared \
    -w -I"$OUT/overlay" -I"$INC" -o "$OUT/libhcref_scalar.so" "$HERE/ref_probe_scalar.cpp"
echo "built $OUT/libhcref_scalar.so"
