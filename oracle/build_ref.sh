#!/usr/bin/env bash
# Compile the reference's evaluator / flow-field headers IN PLACE (include path
# into the read-only azplugins tree, nothing copied) into a pybind11 module under
# oracle/_ref/. Test infrastructure only. Runs only where the reference tree
# exists; elsewhere it does nothing and exits 0.
set -euo pipefail
HERE="$(cd "$(dirname "${BASH_SOURCE[0]}")" && pwd)"
REF_SRC="${AZP_REFERENCE_SRC:-/root/reference/src}"
if [ ! -f "$REF_SRC/PairEvaluatorPerturbedLennardJones.h" ]; then
    echo "build_ref: reference tree not found at $REF_SRC; skipping"
    exit 0
fi
OUT="$HERE/_ref"
mkdir -p "$OUT"
PYBIND_INC="$(python3 -c 'import pybind11; print(pybind11.get_include())')"
PY_INC="$(python3 -c 'import sysconfig; print(sysconfig.get_paths()["include"])')"
EXT="$(python3 -c 'import sysconfig; print(sysconfig.get_config_var("EXT_SUFFIX"))')"
# -ffp-contract=off: the same rounding on x86 and Arm (no fused multiply-add)
g++ -std=c++17 -O2 -ffp-contract=off -fPIC -shared \
    -I"$HERE/ref_shim" -I"$REF_SRC" -I"$PYBIND_INC" -I"$PY_INC" \
    "$HERE/ref_module.cpp" -o "$OUT/azp_ref$EXT"
echo "build_ref: wrote $OUT/azp_ref$EXT"
