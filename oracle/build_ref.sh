#!/usr/bin/env bash
# Builds the reference renderer (Sanaxen/prender, proj/) as a CPU checker.
#
# Test infrastructure only.  The reference sources are read where they lie
# (default /root/reference/proj), transcoded from CP932 and given the
# mechanical Linux fixes below in a scratch staging directory OUTSIDE the
# repository, and the binaries land in oracle/_ref/ (git-ignored).  Nothing
# here is shipped or imported by the product path.
#
#   usage: oracle/build_ref.sh [REFERENCE_ROOT]
set -euo pipefail
REF="${1:-/root/reference}"
HERE="$(cd "$(dirname "${BASH_SOURCE[0]}")" && pwd)"
OUT="$HERE/_ref"
STAGE="${PRENDER_REF_STAGE:-${TMPDIR:-/tmp}/prender_ref_stage}"
[ -d "$REF/proj" ] || { echo "reference not found at $REF" >&2; exit 2; }
rm -rf "$STAGE"; mkdir -p "$STAGE" "$OUT"

# 1. transcode (files with a UTF-8 BOM are already UTF-8)
for f in "$REF"/proj/*.h "$REF"/proj/*.cpp "$REF"/proj/*.c; do
  b="$(basename "$f")"
  if head -c3 "$f" | grep -q $'\xef\xbb\xbf'; then cp "$f" "$STAGE/$b"
  else iconv -f CP932 -t UTF-8 "$f" > "$STAGE/$b"; fi
done
# 2. case-insensitive include names used by the sources
ln -sf vector3d.h "$STAGE/Vector3d.h"
ln -sf sceneObject.h "$STAGE/SceneObject.h"

# 3. mechanical fixes: MSVC binds temporaries to non-const references and
#    glibc already declares sincos(); none of these change arithmetic.
cd "$STAGE"
sed -i 's/\bsincos(/prender_sincos(/g' KerrBlackHole.h vector3d.h WormHole.h
sed -i -E 's/WorldAxisSystem\((Spherical|Cartesian)& /WorldAxisSystem(const \1\& /' KerrBlackHole.h WormHole.h
sed -i -E 's/(RayToOrdinaryDifferentialEquationInitial[A-Za-z0-9_]*\([^)]*)Vector3d& dir/\1const Vector3d\& dir/' KerrBlackHole.h
sed -i -E 's/Coordinate_transformation\(Vector3d& /Coordinate_transformation(const Vector3d\& /' WormHole.h
sed -i 's/operator \* ( Matrix4x4& mtx,  Vector3d& vec)/operator * (Matrix4x4\& mtx, const Vector3d\& vec)/' matrix.h
sed -i 's/Vector3d& v = mesh->vertex/Vector3d v = mesh->vertex/' polygon.h
sed -i 's/Color& Intensity = light.SpotLightEmission/Color Intensity = light.SpotLightEmission/' directLight_radiance.h
# bitmap.cpp: stb from the reference tree; drop the C++ AMP colormap utility
sed -i 's#"\.\.\\stb\\stb_image\.h"#"'"$REF"'/stb/stb_image.h"#' bitmap.cpp
sed -i -E '/#include <amp(_math)?\.h>/d; /^using (namespace )?concurrency/d' bitmap.cpp
# Kerr loop probe (read-only copy of loop state; see ref_harness/linux_shim.h)
sed -i 's/^\(\s*\)double delta = (org2 -org1).length();/&\n\1PRENDER_KERR_PROBE(0, cnt, y, org2, dir2);/' scene.cpp
sed -i 's/^\(\s*\)if (intersect_scene_(Ray(org2, dir2), intersection, depth))/\1PRENDER_KERR_PROBE(1, cnt, y, org2, dir2);\n&/' scene.cpp
grep -q 'PRENDER_KERR_PROBE(1' scene.cpp && grep -q 'PRENDER_KERR_PROBE(0' scene.cpp

# 4. compile the reference translation units and the harness
CXX="${CXX:-g++}"
FLAGS=(-std=c++17 -O2 -fopenmp -fpermissive -w -ffp-contract=off -include "$HERE/ref_harness/linux_shim.h" -I "$STAGE")
UNITS=(BVH.cpp Expr.cpp ObjLoader.cpp QBVH.cpp QMC.cpp random.cpp scene.cpp Spectrum.cpp bitmap.cpp)
pids=()
for u in "${UNITS[@]}"; do "$CXX" "${FLAGS[@]}" -c "$STAGE/$u" -o "$STAGE/${u%.cpp}.o" & pids+=($!); done
"$CXX" "${FLAGS[@]}" -c "$HERE/ref_harness/ref_main.cpp" -o "$STAGE/ref_main.o" & pids+=($!)
gcc -O2 -w -ffp-contract=off -c "$STAGE/raytri.c" -o "$STAGE/raytri.o" & pids+=($!)
for p in "${pids[@]}"; do wait "$p"; done
"$CXX" -fopenmp -o "$OUT/prender_ref" "$STAGE"/*.o
echo "built $OUT/prender_ref"
