#!/bin/sh
# Builds oracle/_ref/libref_models.so from the reference's generated ionic
# model headers, compiled verbatim where they lie in the reference tree.
# Usage: oracle/ref/build_ref.sh <cardiacFoam checkout>   (oracle/build.py passes it)
# Test infrastructure only: it pins the oracle's model code; nothing ships it.
set -e
REF=${1:?usage: build_ref.sh <cardiacFoam checkout>}
HERE=$(cd "$(dirname "$0")" && pwd)
OUT="$HERE/../_ref"
IM="$REF/src/ionicModels"
[ -d "$IM" ] || { echo "reference not found at $REF" >&2; exit 2; }
mkdir -p "$OUT"
CXX=${CXX:-g++}
FLAGS="-std=c++17 -O2 -fPIC -ffp-contract=off -w -I$HERE/shim"
objs=""
build() {  # name dir header prefix rates vars [vars2]
    o="$OUT/ref_$1.o"
    extra=""
    [ -n "$7" ] && extra="-DVARS_FN2=$7"
    $CXX $FLAGS -I"$IM/$2" -DMODEL_HEADER="\"$3\"" -DREF_PREFIX="ref_$1" \
        -DMODEL_PREFIX="$4" -DRATES_FN="$5" -DVARS_FN="$6" $extra \
        -c "$HERE/ref_model.cpp" -o "$o"
    objs="$objs $o"
}
build tnnp TNNP TNNP_2004.H TNNP TNNPcomputeRates TNNPcomputeVariables TNNPcomputeRates
build ord ORd ORd_2011.H ORd ORdcomputeVariables ORdcomputeVariables
build torord_dyncl ToRORd_dynCl ToRORd_dynCl_2023.H ToRORd_dynCl ToRORd_dynClcomputeVariables ToRORd_dynClcomputeVariables
build alievpanfilov AlievPanfilov AlievPanfilov_1996.H AlievPanfilov AlievPanfilovcomputeVariables AlievPanfilovcomputeVariables
build buenoorovio BuenoOrovio BuenoOrovio_2008.H BuenoOrovio BuenoOroviocomputeVariables BuenoOroviocomputeVariables
$CXX -shared -o "$OUT/libref_models.so" $objs
rm -f $objs
echo "built $OUT/libref_models.so"
