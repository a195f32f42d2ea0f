#!/usr/bin/env bash
# Build the CPU oracle restatement (test infrastructure) into oracle/libazp_oracle.so.
# Plain g++, no architecture flags, -ffp-contract=off: same rounding on x86 and Arm.
set -euo pipefail
HERE="$(cd "$(dirname "${BASH_SOURCE[0]}")" && pwd)"
g++ -std=c++17 -O3 -ffp-contract=off -fopenmp -fPIC -shared \
    "$HERE/azp_oracle.cpp" -o "$HERE/libazp_oracle.so.tmp"
mv -f "$HERE/libazp_oracle.so.tmp" "$HERE/libazp_oracle.so"
echo "build_oracle: wrote $HERE/libazp_oracle.so"
