#!/usr/bin/env bash
# Compile the reference's evaluator / flow-field headers IN PLACE (include path
# into the read-only azplugins tree, nothing copied) into a pybind11 module under
# oracle/_ref/, and the param_type size probe (oracle/ref_sizes.cpp) for HOOMD's
# double- and single-precision builds. Test infrastructure only.
#
# Usage: build_ref.sh <azplugins src directory>   (or AZP_REFERENCE_SRC=<dir>)
# Without a path, or where the tree is absent, it does nothing and exits 0.
set -euo pipefail
HERE="$(cd "$(dirname "${BASH_SOURCE[0]}")" && pwd)"
REF_SRC="${1:-${AZP_REFERENCE_SRC:-}}"
if [ -z "$REF_SRC" ] || [ ! -f "$REF_SRC/PairEvaluatorPerturbedLennardJones.h" ]; then
    echo "build_ref: no azplugins source tree given or found (${REF_SRC:-unset}); skipping"
    exit 0
fi
OUT="$HERE/_ref"
mkdir -p "$OUT"
PYBIND_INC="$(python3 -c 'import pybind11; print(pybind11.get_include())')"
PY_INC="$(python3 -c 'import sysconfig; print(sysconfig.get_paths()["include"])')"
EXT="$(python3 -c 'import sysconfig; print(sysconfig.get_config_var("EXT_SUFFIX"))')"
PY_LD="$(python3-config --ldflags --embed)"
# -ffp-contract=off: the same rounding on x86 and Arm (no fused multiply-add)
g++ -std=c++17 -O2 -ffp-contract=off -fPIC -shared \
    -I"$HERE/ref_shim" -I"$REF_SRC" -I"$PYBIND_INC" -I"$PY_INC" \
    "$HERE/ref_module.cpp" -o "$OUT/azp_ref$EXT"
for prec in double single; do
    DEF=""
    [ "$prec" = single ] && DEF="-DAZP_REF_SINGLE"
    # shellcheck disable=SC2086
    g++ -std=c++17 -O0 $DEF -I"$HERE/ref_shim_sizes" -I"$HERE/ref_shim" -I"$REF_SRC" -I"$PYBIND_INC" -I"$PY_INC" \
        "$HERE/ref_sizes.cpp" -o "$OUT/ref_sizes_$prec" $PY_LD
done
echo "build_ref: wrote $OUT/azp_ref$EXT and $OUT/ref_sizes_{double,single}"
