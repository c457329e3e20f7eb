#!/usr/bin/env bash
# ORACLE / TEST INFRASTRUCTURE — builds the oracle port (C++ restatement of the
# reference step) into oracle/_port/veritas_port.  -ffp-contract=off keeps IEEE
# double arithmetic identical on x86-64 and aarch64.
set -euo pipefail
HERE="$(cd "$(dirname "${BASH_SOURCE[0]}")" && pwd)"
OUT="$HERE/../_port"
mkdir -p "$OUT"
"${CXX:-g++}" -O3 -std=c++17 -fopenmp -ffp-contract=off -o "$OUT/veritas_port" "$HERE/veritas_port.cpp"
echo "built $OUT/veritas_port"
