#!/usr/bin/env bash
# Compile the oracle (CPU restatement, test infrastructure only) into
# oracle/_build/liblbm_oracle.so. No FMA contraction so results are the same on
# x86-64 and aarch64 hosts.
set -euo pipefail
here="$(cd "$(dirname "$0")" && pwd)"
out="$here/_build"
mkdir -p "$out"
omp="-fopenmp"
echo 'int main(void){return 0;}' > "$out/omp_probe.c"
gcc -fopenmp "$out/omp_probe.c" -o "$out/omp_probe" 2>/dev/null || omp=""
rm -f "$out/omp_probe.c" "$out/omp_probe"
gcc -std=c99 -O2 -fPIC -shared -Wall -Wno-unknown-pragmas -ffp-contract=off $omp \
    "$here/lbm_oracle.c" -lm -o "$out/liblbm_oracle.so.tmp"
mv -f "$out/liblbm_oracle.so.tmp" "$out/liblbm_oracle.so"
echo "built $out/liblbm_oracle.so"
